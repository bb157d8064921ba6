// Step kernels instantiated for the f-wave and HLLE solvers.
#include "swe_launch.hpp"
#include "swe_bound.cuh"
#include "swe_sweep.cuh"

namespace swegb {

template <int S> static cudaError_t speed(const DomainDev &d, int n, int th, cudaStream_t s) {
    if (d.semantics == SEM_SPLIT)
        speedSplitKernel<S><<<n, th, 0, s>>>(d);
    else
        sweepKernel<S, SEM_UNSPLIT, false><<<n, th, 0, s>>>(d);
    return cudaGetLastError();
}
template <int S> static cudaError_t update(const DomainDev &d, int n, int th, cudaStream_t s) {
    if (d.semantics == SEM_SPLIT) {
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
template <int S> static int occupancy(int sem, bool upd, int th) {
    const bool split = sem == SEM_SPLIT;
    return upd ? (split ? occ(sweepKernel<S, SEM_SPLIT, true>, th) : occ(sweepKernel<S, SEM_UNSPLIT, true>, th))
               : (split ? occ(speedSplitKernel<S>, th) : occ(sweepKernel<S, SEM_UNSPLIT, false>, th));
}

int occupancyFH(int solver, int sem, bool update, int threads) {
    return solver == SOLVER_FWAVE ? occupancy<SOLVER_FWAVE>(sem, update, threads)
                                  : occupancy<SOLVER_HLLE>(sem, update, threads);
}

int occupancyBound(int solver) {
    return solver == SOLVER_FWAVE ? occ(speedBoundKernel<SOLVER_FWAVE>, 256) : occ(speedBoundKernel<SOLVER_HLLE>, 256);
}

} // namespace swegb
