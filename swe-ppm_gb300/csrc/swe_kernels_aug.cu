// Step kernels instantiated for the augmented Riemann solver and the hybrid
// (f-wave / augmented) solver.
#include "swe_launch.hpp"
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
    if (d.semantics == SEM_SPLIT)
        sweepKernel<S, SEM_SPLIT, true><<<n, th, 0, s>>>(d);
    else
        sweepKernel<S, SEM_UNSPLIT, true><<<n, th, 0, s>>>(d);
    return cudaGetLastError();
}

cudaError_t launchSpeedAug(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_AUGRIE ? speed<SOLVER_AUGRIE>(d, n, th, s) : speed<SOLVER_HYBRID>(d, n, th, s);
}
cudaError_t launchUpdateAug(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_AUGRIE ? update<SOLVER_AUGRIE>(d, n, th, s) : update<SOLVER_HYBRID>(d, n, th, s);
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

int occupancyAug(int solver, int sem, bool update, int threads) {
    return solver == SOLVER_AUGRIE ? occupancy<SOLVER_AUGRIE>(sem, update, threads)
                                   : occupancy<SOLVER_HYBRID>(sem, update, threads);
}

} // namespace swegb
