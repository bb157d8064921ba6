// Local time stepping on the device: the per-block ghost-layer state machine
// and interval bookkeeping of SWE_Block (src/blocks/SWE_Block.hh:311-562) and
// the overdecomposed driver's inner loop (src/examples/swe_mpi_overdecomp.cpp:266-343).
//
// Every block is its own dt group.  One inner iteration is five launches, all
// decided on the device so that iterations can be replayed from a graph:
//   ltsExchangeKernel  boundary conditions of every block and, for each side
//                      connected to a neighbour that is receivable, the
//                      neighbour's copy layer into the block's receive ring and
//                      the neighbour's total local time (exchangeGhosts)
//   ltsCheckKernel     checkAllGhostlayers: copy (same time) or time-interpolate
//                      (neighbour ahead) each received layer into the ghost
//                      ring, ghost-layer states, last-timestep notice, step
//                      counter; the block steps this iteration iff its layers
//                      are in sync (GroupState::enabled)
//   speed pass         per block; maxTimestep rounded to Tsync / 2^k
//   update pass        per enabled block (ghost ring carried into the new buffer)
//   ltsDoneKernel      every block at its interval end: t += Tsync, counters reset
// Once t reaches the target the kernels return at once, so a batch of
// iterations can be queued ahead of the checkpoint.
#include <cfloat>

#include "swe_launch.hpp"
#include "swe_sweep.cuh"

namespace swegb {

namespace {

__device__ __forceinline__ bool ltsRunning(const LtsControl &C) { return C.t < C.target && C.iterations < C.iterLimit; }

__device__ __forceinline__ bool ltsReceivable(const LtsBlock &L, int side) {
    if (L.notified) return false;
    const int s = L.received[side];
    return s == GL_NEXT || s == GL_UNVALID || s == GL_SYNC;
}

__device__ __forceinline__ bool ltsInSync(const LtsBlock &L) {
    return L.received[0] != GL_UNVALID && L.received[1] != GL_UNVALID && L.received[2] != GL_UNVALID &&
           L.received[3] != GL_UNVALID && L.stepSizeCounter <= L.stepSize;
}

/// ghost position p of side `side` (LEFT / RIGHT: rows 1..ny, BOTTOM / TOP:
/// columns 1..nx) and the interior cell next to it
__device__ __forceinline__ void ghostCell(const BlockDesc &B, int side, int p, int &gx, int &gy, int &sx, int &sy) {
    switch (side) {
    case 0: gx = 0; gy = p; sx = 1; sy = p; break;
    case 1: gx = B.nx + 1; gy = p; sx = B.nx; sy = p; break;
    case 2: gx = p; gy = 0; sx = p; sy = 1; break;
    default: gx = p; gy = B.ny + 1; sx = p; sy = B.ny; break;
    }
}

__device__ __forceinline__ long long ringOffset(const BlockDesc &B, int side, int p) {
    switch (side) {
    case 0: return B.ring + (p - 1);
    case 1: return B.ring + B.ny + (p - 1);
    case 2: return B.ring + 2LL * B.ny + (p - 1);
    default: return B.ring + 2LL * B.ny + B.nx + (p - 1);
    }
}

/// decodes thread index i of a block's perimeter into (side, position);
/// side 4 = corner 0..3
__device__ __forceinline__ bool perimeterIndex(const BlockDesc &B, int i, int &side, int &pos) {
    const int nx = B.nx, ny = B.ny;
    if (i < ny) { side = 0; pos = i + 1; }
    else if (i < 2 * ny) { side = 1; pos = i - ny + 1; }
    else if (i < 2 * ny + nx) { side = 2; pos = i - 2 * ny + 1; }
    else if (i < 2 * ny + 2 * nx) { side = 3; pos = i - 2 * ny - nx + 1; }
    else if (i < 2 * ny + 2 * nx + 4) { side = 4; pos = i - 2 * ny - 2 * nx; }
    else return false;
    return true;
}

/// applyBoundaryConditions of every block (src/blocks/SWE_Block.hh:757-911)
/// and the receive half of exchangeGhosts
/// (src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304 with
/// local time stepping): grid (perimeter chunks, blocks)
__global__ void ltsExchangeKernel(const DomainDev d) {
    pdlWaitAndRelease();
    const LtsControl C = *d.ltsCtl;
    if (!ltsRunning(C)) return;
    const int k = blockIdx.y;
    const BlockDesc B = d.blocks[k];
    const int cur = d.groups[k].cur;
    float *F[3] = {pick(d.h, cur) + B.base, pick(d.hu, cur) + B.base, pick(d.hv, cur) + B.base};
    const size_t P = size_t(B.pitch);
    int side, pos;
    if (!perimeterIndex(B, blockIdx.x * blockDim.x + threadIdx.x, side, pos)) return;
    if (side == 4) {  // corners from the diagonal interior cell
        const int gx = (pos & 1) ? B.nx + 1 : 0, gy = (pos & 2) ? B.ny + 1 : 0;
        const int sx = (pos & 1) ? B.nx : 1, sy = (pos & 2) ? B.ny : 1;
        for (int f = 0; f < 3; f++) F[f][size_t(gx) * P + gy] = F[f][size_t(sx) * P + sy];
        return;
    }
    int gx, gy, sx, sy;
    ghostCell(B, side, pos, gx, gy, sx, sy);
    const int type = B.bnd[side];
    if (type == WALL || type == OUTFLOW) {
        const int negate = (type == WALL) ? (side < 2 ? 1 : 2) : -1;  // hu or hv of a wall, nothing for outflow
        for (int f = 0; f < 3; f++) {
            const float v = F[f][size_t(sx) * P + sy];
            F[f][size_t(gx) * P + gy] = (negate == f) ? -v : v;
        }
    } else if (type == CONNECT_WITHIN_RANK) {
        LtsBlock &L = d.lts[k];
        if (!ltsReceivable(L, side)) return;
        const int n = B.nbr[side];
        const BlockDesc N = d.blocks[n];
        const int ncur = d.groups[n].cur;
        int nx = sx, ny = sy;  // the neighbour's copy layer
        switch (side) {
        case 0: nx = N.nx; break;
        case 1: nx = 1; break;
        case 2: ny = N.ny; break;
        default: ny = 1; break;
        }
        const size_t o = size_t(N.base) + size_t(nx) * size_t(N.pitch) + size_t(ny);
        const long long r = ringOffset(B, side, pos);
        d.ring[0][r] = pick(d.h, ncur)[o];
        d.ring[1][r] = pick(d.hu, ncur)[o];
        d.ring[2][r] = pick(d.hv, ncur)[o];
        if (pos == 1) L.borderTimestep[side] = ltsTotalLocal(d.lts[n], C);
    }
}

/// checkAllGhostlayers (src/blocks/SWE_Block.hh:375-436): one CTA per block
__global__ void ltsCheckKernel(const DomainDev d) {
    __shared__ int sAction[4];  // 0 none, 1 copy, 2 interpolate
    __shared__ float sFactor;
    pdlWaitAndRelease();
    const int k = blockIdx.x;
    GroupState *G = d.groups + k;
    const LtsControl C = *d.ltsCtl;
    if (!ltsRunning(C)) {
        if (threadIdx.x == 0) G->enabled = 0;
        return;
    }
    const BlockDesc B = d.blocks[k];
    LtsBlock &L = d.lts[k];
    const float local = ltsTotalLocal(L, C);
    if (threadIdx.x == 0) {
        for (int s = 0; s < 4; s++) sAction[s] = 0;
        sFactor = 0.f;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int s = threadIdx.x;
        const int type = B.bnd[s];
        if (type == CONNECT || type == CONNECT_WITHIN_RANK) {
            const float bt = L.borderTimestep[s];
            if (fabs(double(bt - local)) <= DBL_EPSILON) sAction[s] = 1;
            else if (bt > local) sAction[s] = 2;
        }
    }
    __syncthreads();
    // the received layers into the ghost ring of the current buffer
    const int cur = G->cur;
    float *F[3] = {pick(d.h, cur) + B.base, pick(d.hu, cur) + B.base, pick(d.hv, cur) + B.base};
    const size_t P = size_t(B.pitch);
    for (int i = threadIdx.x; i < 2 * B.ny + 2 * B.nx; i += blockDim.x) {
        int side, pos;
        perimeterIndex(B, i, side, pos);
        const int a = sAction[side];
        if (!a) continue;
        int gx, gy, sx, sy;
        ghostCell(B, side, pos, gx, gy, sx, sy);
        const long long r = ringOffset(B, side, pos);
        // interpolateValue: old + (new - old) * (local / remote)
        const float factor = a == 2 ? local / L.borderTimestep[side] : 0.f;
        for (int f = 0; f < 3; f++) {
            float &g = F[f][size_t(gx) * P + gy];
            const float nv = d.ring[f][r];
            g = (a == 1) ? nv : g + (nv - g) * factor;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int s = 0; s < 4; s++) {
            const int type = B.bnd[s];
            if (type != CONNECT && type != CONNECT_WITHIN_RANK) continue;
            const float bt = L.borderTimestep[s];
            L.received[s] = sAction[s] == 1 ? GL_SYNC : sAction[s] == 2 ? GL_INTER : GL_UNVALID;
            if (bt >= C.duration) L.received[s] = GL_DONE;
        }
        if (fabs(double(C.duration - local)) <= DBL_EPSILON || local >= C.duration) L.notified = 1;
        if (ltsInSync(L)) {
            for (int s = 0; s < 4; s++)
                if (L.received[s] != GL_DONE) L.received[s] = (L.received[s] == GL_INTER) ? GL_INTER : GL_NEXT;
        }
        if (ltsInSync(L) && L.stepSizeCounter < L.stepSize) L.stepSizeCounter++;
        G->enabled = ltsInSync(L) ? 1 : 0;  // read by the next kernels, after this grid ends
    }
}

/// end of an inner iteration: once every block has reached its interval end
/// (hasMaxLocalTimestep, src/blocks/SWE_Block.hh:311-367) the interval is
/// done: t += Tsync, counters reset (src/examples/swe_mpi_overdecomp.cpp:332-342)
__global__ void ltsDoneKernel(const DomainDev d) {
    pdlWaitAndRelease();
    LtsControl &C = *d.ltsCtl;
    if (!ltsRunning(C)) return;
    bool done = true;
    for (int k = threadIdx.x; k < d.nblocks; k += blockDim.x) {
        const LtsBlock &L = d.lts[k];
        if (!((L.stepSizeCounter >= L.stepSize && ltsInSync(L)) || L.notified)) done = false;
    }
    done = __syncthreads_and(done);
    if (done) {
        for (int k = threadIdx.x; k < d.nblocks; k += blockDim.x) {
            LtsBlock &L = d.lts[k];
            L.lastStepSize = L.stepSize;
            L.stepSizeCounter = 0;
            L.stepSize = 0;
            L.timestepCounter++;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        C.iterations++;
        if (done) {
            C.t = C.t + C.maxTimestepLocal;
            C.intervals++;
        }
    }
}

} // namespace

cudaError_t launchLtsExchange(const DomainDev &d, int maxPerimeter, cudaStream_t s) {
    const int threads = 128;
    return launchPdl(ltsExchangeKernel, dim3((maxPerimeter + 4 + threads - 1) / threads, unsigned(d.nblocks)),
                     dim3(threads), s, d);
}
cudaError_t launchLtsCheck(const DomainDev &d, cudaStream_t s) {
    return launchPdl(ltsCheckKernel, dim3(unsigned(d.nblocks)), dim3(256), s, d);
}
cudaError_t launchLtsDone(const DomainDev &d, cudaStream_t s) {
    return launchPdl(ltsDoneKernel, dim3(1), dim3(256), s, d);
}

/// getRoundTimestep of a block at the start of an interval for every entry
/// of `t` (the step sizes it picks), as the speed pass computes it
__global__ void ltsRoundKernel(const float *t, int n, float tsync, int maxDivisor, int *stepSize) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    LtsBlock L{};
    LtsControl C{};
    C.maxTimestepLocal = tsync;
    C.maxDivisor = maxDivisor;
    L.stepSizeCounter = 0;
    ltsRoundTimestep(L, C, t[i]);
    stepSize[i] = L.stepSize;
}

cudaError_t launchLtsRound(const float *t, int n, float tsync, int maxDivisor, int *stepSize, cudaStream_t s) {
    ltsRoundKernel<<<(n + 255) / 256, 256, 0, s>>>(t, n, tsync, maxDivisor, stepSize);
    return cudaGetLastError();
}

} // namespace swegb
