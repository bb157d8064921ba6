// Host-side launchers of the templated step kernels (one translation unit per
// solver family so the library compiles in parallel).
#pragma once

#include <cuda_runtime.h>

#include "swe_device.cuh"

namespace swegb {

/// launch with programmatic stream serialization: the kernel may start while
/// the previous kernel of the stream finishes; it waits for it on the device
/// (pdlWaitAndRelease, swe_sweep.cuh) before touching its results
template <class... P, class... A>
inline cudaError_t launchPdl(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

/// launchPdl with dynamic shared memory
template <class... P, class... A>
inline cudaError_t launchPdlSmem(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// speed pass (computeNumericalFluxes' wave speeds + maxTimestep) and fused
// solve-and-update pass (updateUnknowns) of the f-wave and HLLE solvers
cudaError_t launchSpeedFH(const DomainDev &d, int nunits, int threads, cudaStream_t s);
cudaError_t launchUpdateFH(const DomainDev &d, int nunits, int threads, cudaStream_t s);
// same for the augmented and hybrid solvers
cudaError_t launchSpeedAug(const DomainDev &d, int nunits, int threads, cudaStream_t s);
cudaError_t launchUpdateAug(const DomainDev &d, int nunits, int threads, cudaStream_t s);

// bounded speed pass of the f-wave and HLLE unsplit step over the bound
// tiles (d.tileInfo, d.tileW, d.tileKey), 256 threads per CTA
cudaError_t launchSpeedBound(const DomainDev &d, int grid, cudaStream_t s);
int occupancyBound(int solver);

// local time stepping: exchange, ghost-layer check and interval end of one
// inner iteration (swe_lts.cu)
// (split: two CTAs per block, the second taking the BOTTOM and TOP sides,
// of `threads` threads, the largest block's positions per CTA; not with the
// check's own speed pass, which reads the whole ring: one CTA of 1024)
cudaError_t launchLtsCheck(const DomainDev &d, cudaStream_t s, bool split, int threads = 0);
// getRoundTimestep of the speed pass for a device array of time steps
cudaError_t launchLtsRound(const float *t, int n, float tsync, int maxDivisor, int *stepSize, cudaStream_t s);

// resident CTAs per SM of the step kernels (the smaller of the two passes)
int occupancyFH(int solver, int sem, bool update, int threads);
int occupancyAug(int solver, int sem, bool update, int threads);
inline int passOccupancy(int solver, int sem, bool update, int threads) {
    return (solver == SOLVER_FWAVE || solver == SOLVER_HLLE) ? occupancyFH(solver, sem, update, threads)
                                                           : occupancyAug(solver, sem, update, threads);
}

inline cudaError_t launchSpeed(const DomainDev &d, int nunits, int threads, cudaStream_t s) {
    return (d.solver == SOLVER_FWAVE || d.solver == SOLVER_HLLE) ? launchSpeedFH(d, nunits, threads, s)
                                                                 : launchSpeedAug(d, nunits, threads, s);
}
inline cudaError_t launchUpdate(const DomainDev &d, int nunits, int threads, cudaStream_t s) {
    return (d.solver == SOLVER_FWAVE || d.solver == SOLVER_HLLE) ? launchUpdateFH(d, nunits, threads, s)
                                                                 : launchUpdateAug(d, nunits, threads, s);
}

} // namespace swegb
