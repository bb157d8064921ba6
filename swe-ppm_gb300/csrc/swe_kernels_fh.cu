// Step kernels instantiated for the f-wave and HLLE solvers.
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

cudaError_t launchSpeedFH(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_FWAVE ? speed<SOLVER_FWAVE>(d, n, th, s) : speed<SOLVER_HLLE>(d, n, th, s);
}
cudaError_t launchUpdateFH(const DomainDev &d, int n, int th, cudaStream_t s) {
    return d.solver == SOLVER_FWAVE ? update<SOLVER_FWAVE>(d, n, th, s) : update<SOLVER_HLLE>(d, n, th, s);
}

template <int S> static int occupancy(int sem, int th) {
    int a = 0, b = 0;
    if (sem == SEM_SPLIT) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, speedSplitKernel<S>, th, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sweepKernel<S, SEM_SPLIT, true>, th, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, sweepKernel<S, SEM_UNSPLIT, false>, th, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sweepKernel<S, SEM_UNSPLIT, true>, th, 0);
    }
    return a < b ? a : b;
}

int occupancyFH(int solver, int sem, int threads) {
    return solver == SOLVER_FWAVE ? occupancy<SOLVER_FWAVE>(sem, threads) : occupancy<SOLVER_HLLE>(sem, threads);
}

} // namespace swegb
