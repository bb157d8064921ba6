// Local time stepping on the device: the per-block ghost-layer state machine
// and interval bookkeeping of SWE_Block (src/blocks/SWE_Block.hh:311-562) and
// the overdecomposed driver's inner loop (src/examples/swe_mpi_overdecomp.cpp:266-343).
//
// Every block is its own dt group.  One inner iteration is three launches
// (two where the check runs the speed pass, below), all decided on the
// device so that iterations can be replayed from a graph:
//   ltsCheckKernel  one CTA per block: boundary conditions of the block and,
//                   for each side connected to a neighbour that is
//                   receivable, the neighbour's copy layer into the block's
//                   receive ring with the neighbour's total local time
//                   (exchangeGhosts); then checkAllGhostlayers: copy (same
//                   time) or time-interpolate (neighbour ahead) each received
//                   layer into the ghost ring, ghost-layer states,
//                   last-timestep notice, step counter.  The block steps this
//                   iteration iff its layers are in sync (GroupState::enabled).
//                   The kernel's last CTA lists the enabled blocks and those
//                   at the start of their interval (DomainDev::ltsWork), and
//                   gives the others their step Tsync / stepSize.  For the
//                   f-wave and HLLE solvers on blocks of up to 128^2 cells
//                   the CTA of a block at the start of its interval runs the
//                   block's speed pass itself and there is no speed launch.
//   speed pass      the blocks at the start of an interval: maxTimestep
//                   rounded to Tsync / 2^k (within an interval the step does
//                   not depend on the wave speed)
//   update pass     the enabled blocks (no ghost pushes: the next check
//                   carries the ring into the new buffer); its last CTA ends
//                   the iteration: every block at
//                   its interval end means t += Tsync, counters reset, and
//                   every block's total local time is published for the next
//                   exchange (neighbours read it while their own check runs)
// Both passes split their list's (row tile, column) pairs evenly over the
// grid.  Once t reaches the target the kernels do nothing, so a batch of
// iterations can be queued ahead of the checkpoint.
#include <algorithm>
#include <cfloat>

#include "swe_launch.hpp"
#include "swe_sweep.cuh"

namespace swegb {

namespace {

constexpr int kLtsCheckThreads = 1024;  // one perimeter position per thread for blocks up to 254 x 254

__device__ __forceinline__ bool ltsReceivable(const LtsBlock &L, int side) {
    if (L.notified) return false;
    const int s = L.received[side];
    return s == GL_NEXT || s == GL_UNVALID || s == GL_SYNC;
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

/// decodes thread index i of a block's perimeter (corners excluded) into
/// (side, position)
__device__ __forceinline__ void perimeterIndex(const BlockDesc &B, int i, int &side, int &pos) {
    const int nx = B.nx, ny = B.ny;
    if (i < ny) { side = 0; pos = i + 1; }
    else if (i < 2 * ny) { side = 1; pos = i - ny + 1; }
    else if (i < 2 * ny + nx) { side = 2; pos = i - 2 * ny + 1; }
    else { side = 3; pos = i - 2 * ny - nx + 1; }
}

/// The block's speed pass by one CTA (computeNumericalFluxes' maximum wave
/// speed, src/blocks/SWE_DimensionalSplittingMpi.cpp:391-446): every x-edge
/// (x-1|x), x = 1..nx+1, of rows 1..ny and every y-edge (y-1|y), y =
/// 1..ny+1, of columns 1..nx, with the speed pass's cell quantities and edge
/// speeds; returns the thread's maximum.  Threads take rows (consecutive
/// threads, consecutive rows) and march along x through one of up to
/// blockDim / ny column ranges.
template <int S> __device__ float blockEdgeSpeed(const DomainDev &d, const BlockDesc &B, int cur) {
    const float *H = pick(d.h, cur) + B.base, *HU = pick(d.hu, cur) + B.base, *HV = pick(d.hv, cur) + B.base;
    const float *BT = d.b + B.base;
    const size_t P = size_t(B.pitch);
    const int T = blockDim.x, t = threadIdx.x;
    const int rt = min(B.ny, T), ng = min(T / rt, B.nx);
    float smax = 0.f;
    if (t >= rt * ng) return smax;
    const int g = t / rt;
    const int xa = 1 + int((long long)B.nx * g / ng), xb = int((long long)B.nx * (g + 1) / ng);
    for (int y = 1 + t % rt; y <= B.ny; y += rt) {
        Cell px, dummy;
        {
            const size_t o = size_t(xa - 1) * P + y;
            cellQuantities<S>(H[o], HU[o], HV[o], BT[o], px, dummy);
        }
        for (int x = xa; x <= xb; x++) {
            const size_t o = size_t(x) * P + y;
            Cell cx, cy, bx, by;
            cellQuantities<S>(H[o], HU[o], HV[o], BT[o], cx, cy);
            cellQuantities<S>(H[o - 1], HU[o - 1], HV[o - 1], BT[o - 1], bx, by);
            smax = vmax(smax, edgeSpeed<S>(px, cx));  // (x-1|x)
            smax = vmax(smax, edgeSpeed<S>(by, cy));  // (y-1|y)
            if (y == B.ny) {                           // (ny|ny+1)
                Cell ax, ay;
                cellQuantities<S>(H[o + 1], HU[o + 1], HV[o + 1], BT[o + 1], ax, ay);
                smax = vmax(smax, edgeSpeed<S>(cy, ay));
            }
            px = cx;
        }
        if (xb == B.nx) {  // (nx|nx+1)
            const size_t o = size_t(B.nx + 1) * P + y;
            Cell gx, gy;
            cellQuantities<S>(H[o], HU[o], HV[o], BT[o], gx, gy);
            smax = vmax(smax, edgeSpeed<S>(px, gx));
        }
    }
    return smax;
}

/// exchangeGhosts + checkAllGhostlayers (src/blocks/SWE_Block.hh:375-436):
/// one CTA per block, or with a grid of two per block (large blocks) a
/// second CTA that takes the BOTTOM and TOP sides of the perimeter, whose
/// ghosts and copy layers lie one pitch apart per position; the last of the
/// blocks' first CTAs lists the iteration's work
__global__ void ltsCheckKernel(const DomainDev d) {
    __shared__ int sAction[4], sRecv[4];  // per side: 0 none, 1 copy, 2 interpolate; layer received now
    __shared__ float sFactor[4];
    __shared__ float sNbrLocal[4];  // per side within the rank: the neighbour's total local time,
    __shared__ int sNbrCur[4];      // its current buffer
    __shared__ long long sNbrOff[4];  // and its copy layer: cell of position p at sNbrOff + p sNbrStride
    __shared__ int sNbrStride[4];
    __shared__ int sLast;
    __shared__ int sScan[4][kLtsCheckThreads / 32];
    __shared__ LtsBlock L;   // the block's state, staged: its reads and writes stay on chip
    __shared__ int sCur, sStale, sSpeed;
    __shared__ float sRed[kLtsCheckThreads / 32];
    static_assert(sizeof(LtsBlock) % 4 == 0 && sizeof(LtsBlock) / 4 + 2 <= 32, "staging by warp 0");
    static_assert(kLtsCheckThreads % 32 == 0 && kLtsCheckThreads <= 1024, "warp scan");
    pdlWaitAndRelease();
    const bool split = int(gridDim.x) == 2 * d.nblocks;
    const int k = split ? int(blockIdx.x >> 1) : int(blockIdx.x), t = threadIdx.x;
    const bool rows = split && (blockIdx.x & 1);  // the second CTA: BOTTOM and TOP only
    GroupState *G = d.groups + k;
    const LtsControl C = *d.ltsCtl;
    const bool running = ltsRunning(C);
    const BlockDesc &B = d.blocks[k];
    constexpr int kLInts = int(sizeof(LtsBlock) / 4);
    // one round of loads: the block's state (warp 0) and, per side connected
    // within the rank, the neighbour's local time published at the end of the
    // last iteration and its current buffer (warp 1; the neighbour's own
    // check, running at the same time, writes neither)
    if (t < kLInts) {
        reinterpret_cast<int *>(&L)[t] = reinterpret_cast<const int *>(d.lts + k)[t];
    } else if (t == kLInts) {
        sCur = G->cur;
    } else if (t == kLInts + 1) {
        // the update pass writes no ghosts: after it the current buffer's
        // ring (and corners) are still in the other buffer; the reference's
        // single array keeps them, so they are carried over first
        sStale = G->ringStale;
    } else if (t >= 32 && t < 36 && B.bnd[t - 32] == CONNECT_WITHIN_RANK) {
        const int s = t - 32, n = B.nbr[s];
        sNbrLocal[s] = __ldcg(&d.ltsLocal[n]);
        sNbrCur[s] = __ldcg(&d.groups[n].cur);
        // the neighbour's copy layer: LEFT its column nx, RIGHT its column 1,
        // BOTTOM its row ny, TOP its row 1
        const BlockDesc &N = d.blocks[n];
        const long long P = N.pitch;
        sNbrOff[s] = N.base + (s == 0 ? N.nx * P : s == 1 ? P : s == 2 ? N.ny : 1);
        sNbrStride[s] = s < 2 ? 1 : N.pitch;
    }
    __syncthreads();
    const int cur = sCur;
    const bool stale = sStale != 0;
    float local = 0.f;
    if (running) {
        local = ltsTotalLocal(L, C);
        // per side: whether the neighbour's layer is received now (with the
        // neighbour's total local time), the border time after that, and
        // what checkAllGhostlayers does with the layer: copy (same time) or
        // interpolate (neighbour ahead)
        if (t < 4) {
            const int s = t;
            const int type = B.bnd[s];
            int recv = 0, a = 0;
            float bt = L.borderTimestep[s];
            if (type == CONNECT_WITHIN_RANK && ltsReceivable(L, s)) {
                recv = 1;
                bt = sNbrLocal[s];
                L.borderTimestep[s] = bt;
            }
            if (type == CONNECT || type == CONNECT_WITHIN_RANK) {
                if (fabs(double(bt - local)) <= DBL_EPSILON) a = 1;
                else if (bt > local) a = 2;
            }
            sRecv[s] = recv;
            sAction[s] = a;
            sFactor[s] = a == 2 ? local / bt : 0.f;  // interpolateValue: old + (new - old) * (local / remote)
        }
        __syncthreads();
    }
    if (running || stale) {
        // one pass over the perimeter: the carried ring, then boundary
        // conditions and corners (applyBoundaryConditions,
        // src/blocks/SWE_Block.hh:757-911), the received layer into the
        // receive ring (exchangeGhosts,
        // src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304) and the
        // ring into the ghost ring (checkAllGhostlayers)
        float *F[3] = {pick(d.h, cur) + B.base, pick(d.hu, cur) + B.base, pick(d.hv, cur) + B.base};
        const float *Fo[3] = {pick(d.h, cur ^ 1) + B.base, pick(d.hu, cur ^ 1) + B.base, pick(d.hv, cur ^ 1) + B.base};
        const size_t P = size_t(B.pitch);
        // corners copy the diagonal interior cell (or, carried only, the
        // other buffer's corner); threads 0..3 load them ahead of their side
        // positions and store them after, so both loads are in flight at once
        float cv[3];
        size_t cog = 0;
        const bool corners = t < 4 && !rows;
        if (corners) {
            const int gx = (t & 1) ? B.nx + 1 : 0, gy = (t & 2) ? B.ny + 1 : 0;
            const int sx = (t & 1) ? B.nx : 1, sy = (t & 2) ? B.ny : 1;
            cog = size_t(gx) * P + gy;
            for (int f = 0; f < 3; f++) cv[f] = running ? F[f][size_t(sx) * P + sy] : Fo[f][cog];
        }
        const int iBegin = rows ? 2 * B.ny : 0, iEnd = split && !rows ? 2 * B.ny : 2 * B.ny + 2 * B.nx;
        for (int i = iBegin + t; i < iEnd; i += blockDim.x) {
            int side, pos, gx, gy, sx, sy;
            perimeterIndex(B, i, side, pos);
            ghostCell(B, side, pos, gx, gy, sx, sy);
            const size_t og = size_t(gx) * P + gy;
            // where the ghost's new value comes from: the cell inside (wall,
            // outflow), the neighbour's copy layer received now, or the
            // receive ring (a layer kept from an earlier exchange); its loads
            // go out together with the ghost's own
            const int type = B.bnd[side];
            const bool inside = running && (type == WALL || type == OUTFLOW);
            const bool recv = running && !inside && sRecv[side];
            const int a = (running && !inside) ? sAction[side] : 0;
            const long long r = ringOffset(B, side, pos);
            const float *src[3] = {nullptr, nullptr, nullptr};
            size_t so = 0;
            if (inside) {
                for (int f = 0; f < 3; f++) src[f] = F[f];
                so = size_t(sx) * P + sy;
            } else if (recv) {
                const int ncur = sNbrCur[side];
                src[0] = pick(d.h, ncur);
                src[1] = pick(d.hu, ncur);
                src[2] = pick(d.hv, ncur);
                so = size_t(sNbrOff[side] + (long long)pos * sNbrStride[side]);
            } else if (a) {
                for (int f = 0; f < 3; f++) src[f] = d.ring[f];
                so = size_t(r);
            }
            // the ghost's value now is needed to interpolate and to carry the
            // ring over; walls, outflow and copied layers replace it
            float g[3] = {0.f, 0.f, 0.f}, v[3];
            if (a == 2 || (stale && !inside && a == 0))
                for (int f = 0; f < 3; f++) g[f] = stale ? Fo[f][og] : F[f][og];
            if (src[0])
                for (int f = 0; f < 3; f++) v[f] = src[f][so];
            bool changed = stale;
            if (inside) {
                // walls negate the normal momentum
                const int negate = type == WALL ? (side < 2 ? 1 : 2) : -1;
                for (int f = 0; f < 3; f++) g[f] = (negate == f) ? -v[f] : v[f];
                changed = true;
            } else {
                if (recv)
                    for (int f = 0; f < 3; f++) d.ring[f][r] = v[f];
                if (a) {
                    const float factor = sFactor[side];
                    for (int f = 0; f < 3; f++) g[f] = (a == 1) ? v[f] : g[f] + (v[f] - g[f]) * factor;
                    changed = true;
                }
            }
            if (changed)
                for (int f = 0; f < 3; f++) F[f][og] = g[f];
        }
        if (corners)
            for (int f = 0; f < 3; f++) F[f][cog] = cv[f];
        __syncthreads();
    }
    if (rows) return;  // (the first CTA keeps the block's state and lists)
    if (t == 0) {
        // the update's last CTA sets the flag of every block in the next
        // iteration; a check of one CTA per block (also the one after the
        // run) clears it here.  With two, the second may not have read it yet.
        if (stale && !split) G->ringStale = 0;
        if (running) {
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
            G->enabled = ltsInSync(L) ? 1 : 0;
            G->ltsStep = L.stepSizeCounter <= 0 ? 0 : L.stepSize;
            sSpeed = d.ltsCheckSpeed && ltsInSync(L) && L.stepSizeCounter <= 0;
        } else {
            G->enabled = 0;
            sSpeed = 0;
        }
    }
    __syncthreads();
    if (sSpeed) {
        // the block starts its interval: its speed pass and getRoundTimestep
        // here, on the ghost ring just set (f-wave / HLLE, small blocks)
        const float m = blockReduceMax(d.solver == SOLVER_FWAVE ? blockEdgeSpeed<SOLVER_FWAVE>(d, B, cur)
                                                                : blockEdgeSpeed<SOLVER_HLLE>(d, B, cur),
                                       sRed);
        if (t == 0) {
            G->speed = m;
            G->dt = ltsRoundTimestep(L, C, timestepFromSpeed(m, B.dx, B.dy, d.semantics));
            if (!(m == m)) G->status |= 1;  // NaN wave speed
        }
        __syncthreads();
    }
    // the block's state back to global memory (read by the next kernels
    // only); the last CTA lists the enabled blocks (update pass) and those at
    // the start of their interval (speed pass) from what thread 0 wrote
    // before its release; the others take Tsync / stepSize, the step the
    // speed pass would round to (SWE_Block::getRoundTimestep)
    if (running && t < kLInts) reinterpret_cast<int *>(d.lts + k)[t] = reinterpret_cast<const int *>(&L)[t];
    if (t == 0)
        sLast = arriveAcqRel(reinterpret_cast<unsigned *>(d.ltsWork + kLwArrCheck), 1u) + 1u == unsigned(d.nblocks);
    __syncthreads();
    if (sLast) {
        // thread i takes blocks [i c, (i+1) c); exclusive scans of the counts
        // and pairs over the threads give every entry its place (block order)
        int *W = d.ltsWork;
        const int nb = d.nblocks, TY = d.tileRows, T = blockDim.x, i = threadIdx.x;
        const int chunk = (nb + T - 1) / T;
        const int j0 = min(nb, i * chunk), j1 = min(nb, j0 + chunk);
        auto entry = [&](int j, int &pairs, bool &upd, bool &spd, int &step) {
            const BlockDesc &Bj = d.blocks[j];
            const int en = __ldcg(&d.groups[j].enabled);  // one round: independent loads
            step = __ldcg(&d.groups[j].ltsStep);
            pairs = ((Bj.ny + TY - 1) / TY) * Bj.nx;
            upd = en != 0;
            spd = upd && step == 0 && !d.ltsCheckSpeed;  // (else the check set its dt)
        };
        int v[4] = {0, 0, 0, 0};  // enabled blocks, their pairs, interval starts, their pairs
        constexpr int kCache = 4;  // the first entries' values, kept for the second pass
        int cPairs[kCache];
        bool cUpd[kCache], cSpd[kCache];
        for (int j = j0; j < j1; j++) {
            int pairs, step;
            bool upd, spd;
            entry(j, pairs, upd, spd, step);
            if (j - j0 < kCache) {
                cPairs[j - j0] = pairs;
                cUpd[j - j0] = upd;
                cSpd[j - j0] = spd;
            }
            if (upd) {
                v[0]++;
                v[1] += pairs;
            }
            if (spd) {
                v[2]++;
                v[3] += pairs;
            } else if (upd && step != 0) {
                d.groups[j].dt = C.maxTimestepLocal / float(step);
            }
        }
        // exclusive scans of the four counts over the CTA: within each warp
        // by shuffles, then over the warps' totals
        const int lane = i & 31, warp = i >> 5, nwarps = T >> 5;
        int c[4];
        for (int q = 0; q < 4; q++) c[q] = v[q];
        for (int off = 1; off < 32; off *= 2)
            for (int q = 0; q < 4; q++) {
                const int w = __shfl_up_sync(0xffffffffu, c[q], off);
                if (lane >= off) c[q] += w;
            }
        if (lane == 31)
            for (int q = 0; q < 4; q++) sScan[q][warp] = c[q];
        __syncthreads();
        if (warp == 0) {
            for (int q = 0; q < 4; q++) {
                int w = lane < nwarps ? sScan[q][lane] : 0;
                for (int off = 1; off < 32; off *= 2) {
                    const int u = __shfl_up_sync(0xffffffffu, w, off);
                    if (lane >= off) w += u;
                }
                if (lane < nwarps) sScan[q][lane] = w;
            }
        }
        __syncthreads();
        int o[4];
        for (int q = 0; q < 4; q++) o[q] = c[q] - v[q] + (warp ? sScan[q][warp - 1] : 0);
        int *lU = lwList(W, nb, true), *pU = lwPrefix(W, nb, true);
        int *lS = lwList(W, nb, false), *pS = lwPrefix(W, nb, false);
        for (int j = j0; j < j1; j++) {
            int pairs, step;
            bool upd, spd;
            if (j - j0 < kCache) {
                pairs = cPairs[j - j0];
                upd = cUpd[j - j0];
                spd = cSpd[j - j0];
            } else {
                entry(j, pairs, upd, spd, step);
            }
            if (upd) {
                pU[o[0]] = o[1];
                lU[o[0]++] = j;
                o[1] += pairs;
            }
            if (spd) {
                pS[o[2]] = o[3];
                lS[o[2]++] = j;
                o[3] += pairs;
            }
        }
        if (i == T - 1) {
            W[kLwNUpd] = o[0];
            W[kLwTotUpd] = o[1];
            W[kLwNSpd] = o[2];
            W[kLwTotSpd] = o[3];
            pU[o[0]] = o[1];
            pS[o[2]] = o[3];
            W[kLwArrCheck] = 0;
        }
    }
}

} // namespace

cudaError_t launchLtsCheck(const DomainDev &d, cudaStream_t s, bool split, int threads) {
    threads = split ? std::min(kLtsCheckThreads, std::max(64, (threads + 31) / 32 * 32)) : kLtsCheckThreads;
    return launchPdl(ltsCheckKernel, dim3(unsigned(d.nblocks * (split ? 2 : 1))), dim3(unsigned(threads)), s, d);
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
