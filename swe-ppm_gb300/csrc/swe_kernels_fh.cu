// Step kernels instantiated for the f-wave and HLLE solvers.
#include "swe_launch.hpp"
#include "swe_bound.cuh"
#include "swe_warp.cuh"

namespace swegb {


template <int S> static cudaError_t speed(const DomainDev &d, int n, int th, cudaStream_t s) {
    if (d.variant == VARIANT_WARP) {
        if (d.semantics == SEM_SPLIT)
            speedSplitWarpKernel<S, 4><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, false, 4><<<n, 128, 0, s>>>(d);
    } else if (d.variant == VARIANT_WARP2) {
        if (d.semantics == SEM_SPLIT)
            speedSplitWarpKernel<S, 2><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, false, 2><<<n, 128, 0, s>>>(d);
    } else if (d.variant == VARIANT_WARP1) {
        if (d.semantics == SEM_SPLIT)
            speedSplitWarpKernel<S, 1><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, false, 1><<<n, 128, 0, s>>>(d);
    } else if (d.semantics == SEM_SPLIT) {
        speedSplitKernel<S><<<n, th, 0, s>>>(d);
    } else {
        sweepKernel<S, SEM_UNSPLIT, false><<<n, th, 0, s>>>(d);
    }
    return cudaGetLastError();
}
template <int S> static cudaError_t update(const DomainDev &d, int n, int th, cudaStream_t s) {
    if (d.variant == VARIANT_WARP) {
        if (d.semantics == SEM_SPLIT)
            sweepWarpKernel<S, SEM_SPLIT, true, 4><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, true, 4><<<n, 128, 0, s>>>(d);
    } else if (d.variant == VARIANT_WARP2) {
        if (d.semantics == SEM_SPLIT)
            sweepWarpKernel<S, SEM_SPLIT, true, 2><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, true, 2><<<n, 128, 0, s>>>(d);
    } else if (d.variant == VARIANT_WARP1) {
        if (d.semantics == SEM_SPLIT)
            sweepWarpKernel<S, SEM_SPLIT, true, 1><<<n, 128, 0, s>>>(d);
        else
            sweepWarpKernel<S, SEM_UNSPLIT, true, 1><<<n, 128, 0, s>>>(d);
    } else if (d.semantics == SEM_SPLIT) {
        sweepKernel<S, SEM_SPLIT, true><<<n, th, 0, s>>>(d);
    } else {
        cudaError_t e = launchPdl(sweepKernel<S, SEM_UNSPLIT, true>, dim3(n), dim3(th), s, d);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t launchSpeedFH(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_FWAVE ? speed<SOLVER_FWAVE>(d, n, th, s) : speed<SOLVER_HLLE>(d, n, th, s);
}
cudaError_t launchUpdateFH(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_FWAVE ? update<SOLVER_FWAVE>(d, n, th, s) : update<SOLVER_HLLE>(d, n, th, s);
}

cudaError_t launchSpeedBound(const DomainDev &d, int grid, cudaStream_t s) {
    cudaError_t e = d.solver == SOLVER_FWAVE ? launchPdl(speedBoundKernel<SOLVER_FWAVE>, dim3(grid), dim3(256), s, d)
                                             : launchPdl(speedBoundKernel<SOLVER_HLLE>, dim3(grid), dim3(256), s, d);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <class K> static int occ(K kernel, int th) {
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, kernel, th, 0);
    return a;
}

/// resident CTAs per SM of one pass's kernel
template <int S> static int occupancy(int variant, int sem, bool upd, int th) {
    const bool split = sem == SEM_SPLIT;
    if (variant == VARIANT_WARP)
        return upd ? (split ? occ(sweepWarpKernel<S, SEM_SPLIT, true, 4>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, true, 4>, 128))
                   : (split ? occ(speedSplitWarpKernel<S, 4>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, false, 4>, 128));
    if (variant == VARIANT_WARP1)
        return upd ? (split ? occ(sweepWarpKernel<S, SEM_SPLIT, true, 1>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, true, 1>, 128))
                   : (split ? occ(speedSplitWarpKernel<S, 1>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, false, 1>, 128));
    if (variant == VARIANT_WARP2)
        return upd ? (split ? occ(sweepWarpKernel<S, SEM_SPLIT, true, 2>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, true, 2>, 128))
                   : (split ? occ(speedSplitWarpKernel<S, 2>, 128) : occ(sweepWarpKernel<S, SEM_UNSPLIT, false, 2>, 128));
    return upd ? (split ? occ(sweepKernel<S, SEM_SPLIT, true>, th) : occ(sweepKernel<S, SEM_UNSPLIT, true>, th))
               : (split ? occ(speedSplitKernel<S>, th) : occ(sweepKernel<S, SEM_UNSPLIT, false>, th));
}

int occupancyFH(int variant, int solver, int sem, bool update, int threads) {
    return solver == SOLVER_FWAVE ? occupancy<SOLVER_FWAVE>(variant, sem, update, threads)
                           : occupancy<SOLVER_HLLE>(variant, sem, update, threads);
}

int occupancyBound(int solver) {
    return solver == SOLVER_FWAVE ? occ(speedBoundKernel<SOLVER_FWAVE>, 256) : occ(speedBoundKernel<SOLVER_HLLE>, 256);
}

} // namespace swegb
