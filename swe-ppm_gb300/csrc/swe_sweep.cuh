// Step kernels of the block step, templated on solver and semantics.
//
// One global time step of a group of blocks is two launches (plus a ghost
// kernel only when the ghost ring is not already valid):
//   sweepKernel<..., false>  speed pass: every edge's max wave speed, CTA max
//                    by warp shuffles, group max by atomicMax; the last
//                    segment of the group turns it into maxTimestep
//                    (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-472)
//   sweepKernel<..., true>   fused pass: solves every edge again, sums the net
//                    updates per cell in registers and writes Q^{n+1} with the
//                    dry clamp (src/blocks/SWE_DimensionalSplittingMpi.cpp:484-518)
//                    or the split update (src/blocks/SWE_DimensionalSplitting.cpp:187-210),
//                    then pushes the next step's ghost layer: boundary
//                    conditions (src/blocks/SWE_Block.hh:757-911) and the copy
//                    layers into the neighbour blocks' ghosts (the on-device
//                    form of src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304).
// The speed pass is needed because dt depends on the same step's wave speeds;
// at 2048^2 the state (67 MB) stays in L2 between the two passes, so DRAM
// sees each input byte once.
//
// Work partition: the rows of every block are cut into tiles of TY rows and
// the list of (tile, column) pairs of all blocks is split evenly over a
// persistent grid (a few CTAs per SM); each CTA gets one or two contiguous
// segments.  Within a segment a CTA owns TY consecutive rows (one per thread;
// y is the contiguous direction) and marches along x.  The x-edge (x-1|x) is
// solved from the previous column kept in registers, the y-edge (y|y+1) from
// the neighbouring thread's cell in shared memory, and the tile's two boundary
// y-edges per column are solved up front; a cell's update is finished one
// column later, when its right edge is known.
#pragma once

#include <cstddef>

#include "swe_device.cuh"

namespace swegb {

__device__ __forceinline__ float blockReduceMax(float v, float *sRed) {
    for (int o = 16; o > 0; o >>= 1) v = vmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sRed[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < int(blockDim.x >> 5)) ? sRed[l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = vmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

/// dt from the group's max wave speed: unsplit blocks
/// (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456) or the split block
/// (src/blocks/SWE_DimensionalSplitting.cpp:136)
__device__ __forceinline__ float timestepFromSpeed(float s, float dx, float dy, int semantics) {
    if (semantics == SEM_SPLIT) return 0.4f * (dx / s);
    if (double(s) > 0.00001) {
        const float a = dx / s, b = dy / s;
        float dt = (b < a) ? b : a;
        dt *= 0.4f;
        return dt;
    }
    return FLT_MAX;
}

/// programmatic dependent launch: wait until the grids this one depends on
/// have finished and their writes are visible, then let the stream's next
/// kernel start launching (it waits the same way).  No-ops for a kernel
/// launched without the programmatic-serialization attribute.
__device__ __forceinline__ void pdlWaitAndRelease() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

/// arrival of `n` units of work on a pass counter, acquire-release at GPU
/// scope: the writes and atomics this thread issued before (and, through the
/// barrier before it, its CTA's) are visible to every thread that sees a later
/// count, so the last arrival sees all of them.  Returns the previous count.
__device__ __forceinline__ unsigned arriveAcqRel(unsigned *counter, unsigned n) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(counter), "r"(n) : "memory");
    return old;
}

/// pulls the cache lines of an object into L1 ahead of its use
template <class T> __device__ __forceinline__ void prefetchL1(const T *p) {
    const char *c = reinterpret_cast<const char *>(p);
    asm volatile("prefetch.global.L1 [%0];" ::"l"(c));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(c + sizeof(T) - 1));
}

/// buffer p of a double-buffered field without dynamic indexing of the kernel parameter
__device__ __forceinline__ float *pick(float *const (&f)[2], int p) { return p ? f[1] : f[0]; }

/// the group still steps (time < target).  Time, target, the current buffer
/// and dt change only in the last CTA of a pass, after every other CTA of the
/// pass has read them, so the passes read them through the read-only path.
__device__ __forceinline__ bool groupActive(const GroupState *G) {
    return __ldg(&G->time) < __ldg(&G->target) && __ldg(&G->enabled);
}

/// total local time of a block (SWE_Block::getTotalLocalTimestep,
/// src/blocks/SWE_Block.hh:557-562)
__device__ __forceinline__ float ltsTotalLocal(const LtsBlock &L, const LtsControl &C) {
    return float(C.maxTimestepLocal * L.timestepCounter) +
           (L.stepSize > 0 ? float(C.maxTimestepLocal * L.stepSizeCounter) / float(L.stepSize) : 0.f);
}

/// the block's time step rounded to Tsync / 2^k at the start of an interval
/// (SWE_Block::getRoundTimestep, src/blocks/SWE_Block.hh:536-555), same float
/// and double operations as the CPU restatement
__device__ __forceinline__ float ltsRoundTimestep(LtsBlock &L, const LtsControl &C, float timestep) {
    if (L.stepSizeCounter <= 0) {
        if (timestep > C.maxTimestepLocal) timestep = C.maxTimestepLocal;
        if (timestep < C.maxTimestepLocal / float(C.maxDivisor)) timestep = C.maxTimestepLocal / float(C.maxDivisor);
        const float logT = logf(timestep);
        const double ln2 = 0x1.62e42fefa39efp-1;  // ln 2, correctly rounded
        const double e = ceil(double(logT) / ln2);
        int divisor = int(ldexp(1.0, -int(e)));
        if (1.f / float(divisor) > timestep) divisor *= 2;
        L.stepSize = divisor > C.maxDivisor ? C.maxDivisor : divisor;
    }
    return C.maxTimestepLocal / float(L.stepSize);
}

/// maxTimestep of a group from its max wave speed; under local time stepping
/// the group is one block and the step is rounded to its interval's grid
__device__ __forceinline__ float groupTimestep(const DomainDev &d, const GroupState *G, float s, float dx, float dy) {
    float dt = timestepFromSpeed(s, dx, dy, d.semantics);
    if (d.lts) dt = ltsRoundTimestep(d.lts[G - d.groups], *d.ltsCtl, dt);
    return dt;
}

/// per-cell quantities in x (normal momentum hu) and y (hv) direction:
/// u = hu * (1/h), v = hv * (1/h), sqrt(h), sqrt(g) sqrt(h).  Those of a dry
/// cell are never read (an edge with a dry side solves with the mirrored wet
/// side), so they are formed without a test.
template <int S> __device__ __forceinline__ void cellQuantities(float h, float hu, float hv, float b, Cell &cx, Cell &cy) {
    float sq = 0.f, c = 0.f, ux = 0.f, uy = 0.f;
    if (S != SOLVER_AUGRIE) {
        const float rh = 1.f / h;
        sq = sqrtf(h);
        if (S == SOLVER_HLLE) c = kSqrtG * sq;
        ux = hu * rh;
        uy = hv * rh;
    }
    cx = makeCell(h, hu, b, ux, sq, c);
    cy = makeCell(h, hv, b, uy, sq, c);
}

__device__ __forceinline__ bool ltsRunning(const LtsControl &C) { return C.t < C.target && C.iterations < C.iterLimit; }

__device__ __forceinline__ bool ltsInSync(const LtsBlock &L) {
    return L.received[0] != GL_UNVALID && L.received[1] != GL_UNVALID && L.received[2] != GL_UNVALID &&
           L.received[3] != GL_UNVALID && L.stepSizeCounter <= L.stepSize;
}

/// Segments of this CTA under local time stepping: the pass's work list
/// (DomainDev::ltsWork) names the blocks that take part, with the prefix sums
/// of their (row tile, column) pairs; CTA c takes pairs [total c / grid,
/// total (c+1) / grid), cut at tile ends and every kMaxTileCols columns.
/// segment(unit, pairs, block's pairs) runs each piece.  Called by every
/// thread of the CTA.
template <bool UPDATE, class Seg>
__device__ __forceinline__ void ltsSegments(const DomainDev &d, int TY, Seg &&segment) {
    int *W = d.ltsWork;
    const int n = __ldcg(W + (UPDATE ? kLwNUpd : kLwNSpd));
    const long long total = __ldcg(W + (UPDATE ? kLwTotUpd : kLwTotSpd));
    const int *list = lwList(W, d.nblocks, UPDATE);
    const int *pref = lwPrefix(W, d.nblocks, UPDATE);
    long long pos = total * blockIdx.x / gridDim.x;
    const long long end = total * (blockIdx.x + 1) / gridDim.x;
    if (pos >= end || n <= 0) return;
    // the entry holding pair pos, pref[j] <= pos < pref[j+1], with its block
    // and prefixes: every thread tests its own entries, so the search is one
    // round of loads (a binary search is log2(n) dependent ones)
    __shared__ int sJ, sK, sP0, sP1;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int a = __ldcg(pref + i), b = __ldcg(pref + i + 1), k = __ldcg(list + i);
        if (a <= pos && pos < b) {
            sJ = i;
            sK = k;
            sP0 = a;
            sP1 = b;
        }
    }
    __syncthreads();
    int j = sJ, k = sK, p0 = sP0, p1 = sP1;
    while (pos < end) {
        const BlockDesc &B = d.blocks[k];
        const long long local = pos - p0;
        const int nx = B.nx;
        const int tile = int(local / nx), col = int(local % nx) + 1;
        const int len = int(min((long long)min(nx + 1 - col, kMaxTileCols), end - pos));
        const int tiles = (B.ny + TY - 1) / TY;
        segment(WorkUnit{k, 1 + tile * TY, col, col + len}, unsigned(len), unsigned(tiles * nx));
        pos += len;
        if (pos >= p1 && pos < end) {  // the next entry
            ++j;
            k = __ldcg(list + j);
            p0 = p1;
            p1 = __ldcg(pref + j + 1);
        }
    }
}

/// End of a local-time-stepping iteration, run by one CTA (the update pass's
/// last): once every block has reached its interval end (hasMaxLocalTimestep,
/// src/blocks/SWE_Block.hh:311-367) the interval is done: t += Tsync,
/// counters reset (src/examples/swe_mpi_overdecomp.cpp:332-342).  Every
/// block's total local time is published for the next iteration's exchange.
__device__ __forceinline__ void ltsEndIteration(const DomainDev &d) {
    static_assert(sizeof(LtsBlock) == 64 && offsetof(LtsBlock, stepSize) == 32 && alignof(LtsBlock) >= 16,
                  "LtsBlock as four int4");
    LtsControl &C = *d.ltsCtl;
    const bool running = ltsRunning(C);
    // each block's ghost-layer states and counters in one load round (the
    // counters of a thread's first kCache blocks stay in registers between
    // the passes)
    constexpr int kCache = 4;
    int4 cnt[kCache];  // stepSize, stepSizeCounter, timestepCounter, notified
    auto load = [&](int k, int4 &r, int4 &c) {
        const int4 *p = reinterpret_cast<const int4 *>(d.lts + k);
        r = p[0];
        c = p[2];
    };
    auto finished = [](const int4 &r, const int4 &c) {
        const bool inSync = r.x != GL_UNVALID && r.y != GL_UNVALID && r.z != GL_UNVALID && r.w != GL_UNVALID &&
                            c.y <= c.x;
        return (c.y >= c.x && inSync) || c.w != 0;
    };
    bool done = true;
    for (int j = 0, k = threadIdx.x; k < d.nblocks; j++, k += blockDim.x) {
        int4 r, c;  // received[4]; the counters
        load(k, r, c);
        if (j < kCache) cnt[j] = c;
        if (running && !finished(r, c)) done = false;
    }
    done = __syncthreads_and(done);
    for (int j = 0, k = threadIdx.x; k < d.nblocks; j++, k += blockDim.x) {
        // the blocks that stepped flipped their buffers: the next check
        // carries their ghost ring over; the others' rings are in place
        d.groups[k].ringStale = d.groups[k].enabled ? 1 : 0;
        int4 r, c;
        if (j < kCache) {
            c = cnt[j];
        } else {
            load(k, r, c);
        }
        if (running && done) {
            int *L = reinterpret_cast<int *>(d.lts + k);
            L[offsetof(LtsBlock, lastStepSize) / 4] = c.x;
            c = make_int4(0, 0, c.z + 1, c.w);
            reinterpret_cast<int4 *>(d.lts + k)[2] = c;
        }
        LtsBlock T{};
        T.stepSize = c.x;
        T.stepSizeCounter = c.y;
        T.timestepCounter = c.z;
        d.ltsLocal[k] = ltsTotalLocal(T, C);
    }
    if (threadIdx.x == 0 && running) {
        C.iterations++;
        if (done) {
            C.t = C.t + C.maxTimestepLocal;
            C.intervals++;
        }
    }
}

/// the segment's share of the running pass is done; the last segment of the
/// group finishes the pass (dt after the speed pass; clock, step count and
/// current buffer after the update pass)
///
/// A segment adds `count` to the group's arrivals; the pass is complete at
/// `total` (0: the group's segment count of the static partition).
template <bool UPDATE>
__device__ __forceinline__ void segmentDone(const DomainDev &d, GroupState *G, float segMax, float *sRed, int *sLast,
                                            int cur, unsigned count = 1u, unsigned total = 0u) {
    float m = 0.f;
    if (!UPDATE) m = blockReduceMax(segMax, sRed);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (!UPDATE) atomicMax(&G->speedBits, __float_as_uint(m));
        const unsigned prev = arriveAcqRel(&G->arrived, count);
        const unsigned need = total ? total : unsigned(UPDATE ? G->unitsUpd : G->units);
        *sLast = (prev + count == need);
    }
    __syncthreads();
    // the group state the last segment writes is read by the next kernel,
    // which starts after this grid completes (or waits for it): no fence
    if (*sLast && threadIdx.x == 0) {
        if (UPDATE) {
            G->arrived = 0u;
            G->time = G->time + G->dt;
            G->steps = G->steps + 1;
            G->cur = cur ^ 1;
            G->ghostsAhead = d.lts ? 0 : 1;  // local time stepping rebuilds the ring itself
            G->ringStale = d.lts ? 1 : 0;    // ... from the ring the other buffer holds
            // speed bounds now describe the output buffer
            G->boundsValid[cur] = 0;
            G->boundsValid[cur ^ 1] = d.tileW ? 1 : 0;
        } else {
            float s = __uint_as_float(__ldcg(&G->speedBits));  // every CTA's maximum (acquired above)
            const BlockDesc &F = d.blocks[G->firstBlock];
            if (d.semantics == SEM_SPLIT && d.splitDtMode == SPLIT_DT_LAST_EDGE) {
                // speed of the last x-edge the serial loop solves: (nx | nx+1) in row ny+1
                const float *Hc = pick(d.h, cur) + F.base, *HUc = pick(d.hu, cur) + F.base, *Bc = d.b + F.base;
                const size_t o = size_t(F.nx) * size_t(F.pitch) + size_t(F.ny + 1);
                const size_t o2 = o + size_t(F.pitch);
                Cell L, R, dummy;
                switch (d.solver) {
                case SOLVER_FWAVE:
                    cellQuantities<SOLVER_FWAVE>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                    cellQuantities<SOLVER_FWAVE>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
                    s = edgeSpeed<SOLVER_FWAVE>(L, R);
                    break;
                case SOLVER_HLLE:
                    cellQuantities<SOLVER_HLLE>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                    cellQuantities<SOLVER_HLLE>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
                    s = edgeSpeed<SOLVER_HLLE>(L, R);
                    break;
                case SOLVER_AUGRIE:
                    cellQuantities<SOLVER_AUGRIE>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                    cellQuantities<SOLVER_AUGRIE>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
                    s = edgeSpeed<SOLVER_AUGRIE>(L, R);
                    break;
                default:
                    cellQuantities<SOLVER_HYBRID>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                    cellQuantities<SOLVER_HYBRID>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
                    s = edgeSpeed<SOLVER_HYBRID>(L, R);
                    break;
                }
                s = vmax(0.f, s);
            }
            G->speed = s;
            G->dt = groupTimestep(d, G, s, F.dx, F.dy);
            if (!(s == s)) G->status |= 1;  // NaN wave speed
            G->speedBits = 0u;
            G->arrived = 0u;
        }
    }
}

/// Upper bound of the wave speed of any f-wave / HLLE edge touching a cell:
/// max(|hu|, |hv|)/h + sqrt(g h) for wet cells, 0 for dry ones (a dry side
/// takes the mirrored wet state).  The Roe speed |uRoe| + cRoe of an edge is at
/// most the sqrt(h)-weighted mean of its two cells' |u| + c (cRoe <= that mean
/// of c by the quadratic-arithmetic mean inequality), and the Einfeldt speeds
/// u_L - c_L, u_R + c_R are bounded by the cells' own values, so every edge
/// speed is at most the larger bound of its two cells.  Approximate reciprocal
/// and square root: the bound is used with a relative margin far above their
/// error; non-finite or huge states give +inf (never skipped).
__device__ __forceinline__ float cellSpeedBound(float h, float hu, float hv) {
    if (h < kDryTol) return 0.f;
    const float m = fmaxf(fabsf(hu), fabsf(hv));
    const float w = fmaf(m, __fdividef(1.f, h), kSqrtG * (h * rsqrtf(h)));
    return (w <= FLT_MAX && h < 1e30f) ? w : INFINITY;
}

/// folds the warp's cell bounds since the last flush into bound tile
/// (column of cell xcell, rows of the warp) of parity `out` (all lanes call)
__device__ __forceinline__ void boundFlush(const DomainDev &d, const BlockDesc &B, int out, int xcell, int warpRow0,
                                           int yTop, int y, float &wmax, int &xarg) {
    unsigned long long key = (wmax > 0.f && xarg >= 0)
                                 ? ((unsigned long long)__float_as_uint(wmax) << 32) |
                                       ((unsigned long long)xarg << 16) | (unsigned long long)y
                                 : 0ull;
    float wm = wmax;
    for (int o = 16; o > 0; o >>= 1) {
        wm = vmax(wm, __shfl_xor_sync(0xffffffffu, wm, o));
        const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
        key = k2 > key ? k2 : key;
    }
    if ((threadIdx.x & 31) == 0 && warpRow0 <= yTop && wm > 0.f) {
        const size_t tile = size_t(out) * size_t(d.ntiles) + size_t(B.tileBase) +
                            size_t((xcell - 1) / kBoundTile) * size_t(B.tilesY) + size_t((warpRow0 - 1) / kBoundTile);
        atomicMax(&d.tileW[tile], __float_as_uint(wm));
        atomicMax(&d.tileKey[tile], key);
    }
    wmax = 0.f;
    xarg = -1;
}

/// relative margin of the speed bounds (rounding of the bound and of the
/// edge speeds is a few ulp)
constexpr float kBoundMargin = 1.0f + 1.0f / 4096.0f;

/// pushes Q^{n+1} of a cell on the block's rim into every ghost cell whose
/// value the next step's setGhostLayer takes from it (kept out of line: only
/// rim cells call it)
static __device__ __noinline__ void pushGhosts(const DomainDev &d, const BlockDesc &B, int outBuf, size_t P, int x,
                                               int y, float h, float hu, float hv) {
    float *HO = pick(d.h, outBuf), *HUO = pick(d.hu, outBuf), *HVO = pick(d.hv, outBuf);
    const bool edgeX = (x == 1) || (x == B.nx);
    const bool edgeY = (y == 1) || (y == B.ny);
    // sides: LEFT (x == 1), RIGHT (x == nx), BOTTOM (y == 1), TOP (y == ny)
    for (int side = 0; side < 4; side++) {
        const bool on = side == 0 ? x == 1 : side == 1 ? x == B.nx : side == 2 ? y == 1 : y == B.ny;
        if (!on) continue;
        const int type = B.bnd[side];
        const int gx = side == 0 ? 0 : side == 1 ? B.nx + 1 : x;
        const int gy = side == 2 ? 0 : side == 3 ? B.ny + 1 : y;
        const size_t g = size_t(B.base) + size_t(gx) * P + size_t(gy);
        if (type == OUTFLOW) {
            HO[g] = h; HUO[g] = hu; HVO[g] = hv;
        } else if (type == WALL) {
            HO[g] = h;
            HUO[g] = side < 2 ? -hu : hu;
            HVO[g] = side < 2 ? hv : -hv;
        } else if (type == CONNECT_WITHIN_RANK) {
            const BlockDesc &N = d.blocks[B.nbr[side]];
            const int nxg = side == 0 ? N.nx + 1 : side == 1 ? 0 : x;
            const int nyg = side == 2 ? N.ny + 1 : side == 3 ? 0 : y;
            const size_t gn = size_t(N.base) + size_t(nxg) * size_t(N.pitch) + size_t(nyg);
            HO[gn] = h; HUO[gn] = hu; HVO[gn] = hv;
        } else {
            // CONNECT, INFLOW, PASSIVE: the ghost keeps its value (set elsewhere)
            const float *HI = pick(d.h, outBuf ^ 1), *HUI = pick(d.hu, outBuf ^ 1), *HVI = pick(d.hv, outBuf ^ 1);
            HO[g] = HI[g]; HUO[g] = HUI[g]; HVO[g] = HVI[g];
        }
    }
    // corners come from the diagonal interior cell whatever the boundary type
    if (edgeX && edgeY) {
        for (int cxi = 0; cxi < 2; cxi++)
            for (int cyi = 0; cyi < 2; cyi++) {
                const int sx = cxi ? B.nx : 1, sy = cyi ? B.ny : 1;
                if (sx != x || sy != y) continue;
                const size_t g = size_t(B.base) + size_t(cxi ? B.nx + 1 : 0) * P + size_t(cyi ? B.ny + 1 : 0);
                HO[g] = h; HUO[g] = hu; HVO[g] = hv;
            }
    }
}

template <int S, int SEM, bool UPDATE>
__global__ void __launch_bounds__(kMaxTileRows, 4) sweepKernel(const DomainDev d) {
    // the update pass of the f-wave / HLLE unsplit step also records the
    // speed bounds of the bounded speed pass
    constexpr bool BOUNDS = UPDATE && SEM == SEM_UNSPLIT && (S == SOLVER_HLLE || S == SOLVER_FWAVE);
    __shared__ float sC[2][6][kMaxTileRows];   // y-direction cell quantities of column x
    __shared__ float sR[2][2][kMaxTileRows];   // right-going (h, hv) update into row t
    __shared__ float sBot[2][kMaxTileCols];    // right-going update into row y0 (bottom tile edge)
    __shared__ float sTop[2][kMaxTileCols];    // left-going update into row yTop (top tile edge)
    __shared__ float sRed[kMaxTileRows / 32];
    __shared__ int sLast;
    const bool bounds = BOUNDS && d.tileW != nullptr;
    // the static partition and the block descriptors are written only when
    // the domain is built (local time stepping's work lists are not: they
    // come from the previous kernel): bring the first segment's into L1 before waiting for the
    // previous kernel.  The update pass also prefetches the segment's first
    // columns into L2 from the buffer the group state names now (a hint only:
    // every value used is loaded after the wait).
    if (!d.ltsWork) {
        const int s0 = d.ctaSeg[blockIdx.x];
        if (s0 < d.ctaSeg[blockIdx.x + 1]) {
            const WorkUnit w0 = d.units[s0];
            const BlockDesc &B0 = d.blocks[w0.block];
            if (threadIdx.x == 0) prefetchL1(&B0);
            if (UPDATE) {
                const int y = w0.y0 + int(threadIdx.x);
                // through L2 only: no line of the group state may sit in L1
                // when the reads after the wait come
                const int c = __ldcg(&d.groups[B0.group].cur);
                const size_t P = size_t(B0.pitch);
                const float *f[4] = {pick(d.h, c), pick(d.hu, c), pick(d.hv, c), d.b};
                if (y <= B0.ny + 1) {
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        for (int x = w0.x0 - 1; x <= min(w0.x0 + 2, w0.x1); x++)
                            asm volatile("prefetch.global.L2 [%0];" ::"l"(f[k] + B0.base + size_t(x) * P + size_t(y)));
                }
                // the two cells of this thread's boundary y-edge (see below)
                const int XC0 = w0.x1 - w0.x0;
                if (int(threadIdx.x) < 2 * XC0) {
                    const bool top = int(threadIdx.x) >= XC0;
                    const int k = top ? int(threadIdx.x) - XC0 : int(threadIdx.x);
                    const int yl = top ? min(w0.y0 + int(blockDim.x) - 1, B0.ny) : w0.y0 - 1;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(f[q] + B0.base + size_t(w0.x0 + k) * P + size_t(yl)));
                }
            }
        }
    }
    pdlWaitAndRelease();

    const int t = threadIdx.x, TY = blockDim.x;
    // one segment: rows [wu.y0, wu.y0 + TY) x columns [wu.x0, wu.x1) of a block
    auto segment = [&](const WorkUnit wu, unsigned count, unsigned total) {
        const BlockDesc B = d.blocks[wu.block];
        // local time stepping: block k is dt group k, so the group's loads
        // need not wait for the block descriptor's
        GroupState *G = d.groups + (d.ltsWork ? wu.block : B.group);
        if (!groupActive(G)) return;
        const int cur = __ldg(&G->cur);
        const float *__restrict__ H = pick(d.h, cur) + B.base;
        const float *__restrict__ HU = pick(d.hu, cur) + B.base;
        const float *__restrict__ HV = pick(d.hv, cur) + B.base;
        const float *__restrict__ BT = d.b + B.base;
        const size_t P = size_t(B.pitch);
        const int x0 = wu.x0, x1 = wu.x1, XC = x1 - x0;
        const int y0 = wu.y0;
        const int y = y0 + t;
        const int yTop = min(y0 + TY - 1, B.ny);
        const bool active = y <= yTop;
        float smax = 0.f;
        float *__restrict__ HO = pick(d.h, cur ^ 1) + B.base;
        float *__restrict__ HUO = pick(d.hu, cur ^ 1) + B.base;
        float *__restrict__ HVO = pick(d.hv, cur ^ 1) + B.base;
        const bool rimRow = y == 1 || y == B.ny;
        // a rim row (y == 1 or y == ny) pushes the ghost below / above each of
        // its cells every column, as pushGhosts does it: one store per field at
        // rimGhost + x * rimPitch (offsets from the block's base).  Outflow and
        // intra-rank sides copy the cell, a wall negates hv, the other types
        // (and every side under local time stepping) keep the ghost's value
        // from the input buffer.  The block's first and last columns go
        // through pushGhosts (corners).  Inline, because the CTA's barrier makes
        // every warp wait for the rim row's warp each column.
        int rimMode = 0;  // 0: pushGhosts, 1: copy, 2: copy with -hv, 3: keep (local time stepping pushes none)
        long long rimGhost = 0;
        int rimPitch = 0;
        if (UPDATE && rimRow && B.ny > 1 && !d.lts) {
            const int side = (y == 1) ? 2 : 3;
            const int type = B.bnd[side];
            rimGhost = (side == 2) ? 0 : B.ny + 1;
            rimPitch = B.pitch;
            if (type == OUTFLOW || type == WALL) {
                rimMode = type == WALL ? 2 : 1;
            } else if (type == CONNECT_WITHIN_RANK) {
                const BlockDesc &N = d.blocks[B.nbr[side]];
                rimMode = 1;
                rimGhost = N.base - B.base + ((side == 2) ? N.ny + 1 : 0);
                rimPitch = N.pitch;
            } else {
                rimMode = 3;
            }
        }

        float dtdx = 0.f, dtdy = 0.f;
        if (UPDATE) {
            const float dt = __ldg(&G->dt);
            dtdx = dt / B.dx;
            dtdy = (SEM == SEM_SPLIT) ? dtdx : dt / B.dy;
        }

        __syncthreads();  // shared buffers of the previous segment are free
        // the tile's bottom (y0-1|y0) and top (yTop|yTop+1) y-edges of every column
        for (int i = t; i < 2 * XC; i += TY) {
            const bool top = i >= XC;
            const int k = top ? i - XC : i;
            const size_t o = size_t(x0 + k) * P + size_t(top ? yTop : y0 - 1);
            Cell L, R, dummy;
            cellQuantities<S>(H[o], HU[o], HV[o], BT[o], dummy, L);
            cellQuantities<S>(H[o + 1], HU[o + 1], HV[o + 1], BT[o + 1], dummy, R);
            if (UPDATE) {
                float aL, aR, auL, auR, s;
                // edgeSolve<S, true> leaves out the + 0 of the routing's
                // left-going parts (sTop here, aL/auL below): each is only ever
                // added to a right-going part, which is never -0, so every
                // sum keeps the reference's sign of zero
                edgeSolve<S, true>(L, R, aL, aR, auL, auR, s);
                if (top) {
                    sTop[0][k] = aL;
                    sTop[1][k] = auL;
                } else {
                    sBot[0][k] = aR;
                    sBot[1][k] = auR;
                }
            } else {
                smax = vmax(smax, edgeSpeed<S>(L, R));
            }
        }

        float nh = 0.f, nhu = 0.f, nhv = 0.f, nb = 0.f;
        if (active) {
            const unsigned o = unsigned(x0 - 1) * unsigned(P) + unsigned(y);
            nh = H[o]; nhu = HU[o]; nhv = HV[o]; nb = BT[o];
        }
        Cell prevX = makeCell(0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
        float pendH = 0.f, pendHU = 0.f;             // right-going x-update into cell x
        float oldH = 0.f, oldHU = 0.f, oldHV = 0.f;  // Q^n of cell x-1
        float syH = 0.f, syHV = 0.f;                 // y net-update sums of cell x-1
        bool bad = false;                            // a non-finite water height was produced
        float wmax = 0.f;                            // largest speed bound of this row's new cells
        int xarg = -1;                               // ... and its column

        for (int x = x0 - 1; x <= x1; ++x) {
            const float ch = nh, chu = nhu, chv = nhv, cb = nb;
            if (x < x1 && active) {
                const unsigned o = unsigned(x + 1) * unsigned(P) + unsigned(y);
                nh = H[o]; nhu = HU[o]; nhv = HV[o]; nb = BT[o];
            }
            Cell cx, cy;
            cellQuantities<S>(ch, chu, chv, cb, cx, cy);

            // x-edge (x-1 | x)
            if (x >= x0 && active) {
                if (UPDATE) {
                    float aL, aR, auL, auR, s;
                    edgeSolve<S, true>(prevX, cx, aL, aR, auL, auR, s);
                    if (x - 1 >= x0) {
                        float hn, hun, hvn;
                        if (SEM == SEM_UNSPLIT) {
                            const float sxH = pendH + aL, sxHU = pendHU + auL;
                            hn = oldH - (dtdx * sxH + dtdy * syH);
                            hun = oldHU - dtdx * sxHU;
                            hvn = oldHV - dtdy * syHV;
                            if (hn < 0.f) {
                                hn = 0.f; hun = 0.f; hvn = 0.f;
                            } else if (hn < 0.1f) {
                                hun = 0.f; hvn = 0.f;
                            }
                        } else {
                            const float sxH = aL + pendH, sxHU = auL + pendHU;
                            const float hStar = oldH - dtdx * sxH;
                            hn = hStar - dtdx * syH;
                            hun = oldHU - dtdx * sxHU;
                            hvn = oldHV - dtdx * syHV;
                        }
                        bad |= !(fabsf(hn) <= FLT_MAX);
                        if (BOUNDS && bounds) {  // (the bounds feed only the bounded speed pass)
                            const float w = cellSpeedBound(hn, hun, hvn);
                            if (w > wmax) {
                                wmax = w;
                                xarg = x - 1;
                            }
                        }
                        {
                            // per-block offsets fit in 32 bits
                            const unsigned o = unsigned(x - 1) * unsigned(P) + unsigned(y);
                            HO[o] = hn;
                            HUO[o] = hun;
                            HVO[o] = hvn;
                            // no ghost pushes under local time stepping: the
                            // next check carries the ring over and rebuilds it
                            if (!d.lts && (x - 1 == 1 || x - 1 == B.nx || rimRow)) {
                                if (rimMode != 0 && x - 1 != 1 && x - 1 != B.nx) {
                                    const long long g = rimGhost + (long long)(x - 1) * rimPitch;
                                    if (rimMode == 3) {
                                        HO[g] = H[g];
                                        HUO[g] = HU[g];
                                        HVO[g] = HV[g];
                                    } else {
                                        HO[g] = hn;
                                        HUO[g] = hun;
                                        HVO[g] = rimMode == 2 ? -hvn : hvn;
                                    }
                                } else {
                                    pushGhosts(d, B, cur ^ 1, P, x - 1, y, hn, hun, hvn);
                                }
                            }
                        }
                    }
                    pendH = aR;
                    pendHU = auR;
                } else {
                    smax = vmax(smax, edgeSpeed<S>(prevX, cx));
                }
            }
            // cell x-1 closed a column range of bound tiles, or the segment
            if (BOUNDS && bounds && x - 1 >= x0 && (((x - 2) & (kBoundTile - 1)) == kBoundTile - 1 || x == x1))
                boundFlush(d, B, cur ^ 1, x - 1, y0 + (t & ~31), yTop, y, wmax, xarg);
            prevX = cx;

            // y-edges of column x
            if (x >= x0 && x < x1) {
                const int buf = x & 1;
                sC[buf][0][t] = cy.h; sC[buf][1][t] = cy.hn; sC[buf][2][t] = cy.b;
                sC[buf][3][t] = cy.u; sC[buf][4][t] = cy.sq; sC[buf][5][t] = cy.c;
                __syncthreads();
                float bLh = 0.f, bLhv = 0.f;
                if (active && y < yTop) {
                    const Cell up = makeCell(sC[buf][0][t + 1], sC[buf][1][t + 1], sC[buf][2][t + 1],
                                             sC[buf][3][t + 1], sC[buf][4][t + 1], sC[buf][5][t + 1]);
                    if (UPDATE) {
                        float bR, bRhv, s;
                        edgeSolve<S, true>(cy, up, bLh, bR, bLhv, bRhv, s);
                        sR[buf][0][t + 1] = bR;
                        sR[buf][1][t + 1] = bRhv;
                    } else {
                        smax = vmax(smax, edgeSpeed<S>(cy, up));
                    }
                }
                if (UPDATE) {
                    __syncthreads();
                    if (active) {
                        if (y == yTop) {
                            bLh = sTop[0][x - x0];
                            bLhv = sTop[1][x - x0];
                        }
                        const float rH = (t == 0) ? sBot[0][x - x0] : sR[buf][0][t];
                        const float rHV = (t == 0) ? sBot[1][x - x0] : sR[buf][1][t];
                        if (SEM == SEM_UNSPLIT) {
                            syH = rH + bLh;
                            syHV = rHV + bLhv;
                        } else {
                            syH = bLh + rH;
                            syHV = bLhv + rHV;
                        }
                        oldH = ch; oldHU = chu; oldHV = chv;
                    }
                }
            }
        }
        if (UPDATE && __syncthreads_or(bad) && t == 0) atomicOr(&G->status, 2);
        segmentDone<UPDATE>(d, G, smax, sRed, &sLast, cur, count, total);
    };
    if (d.ltsWork) {
        ltsSegments<UPDATE>(d, TY, segment);
        if (UPDATE) {
            // the update pass's last CTA ends the iteration
            __syncthreads();
            if (t == 0)
                sLast = arriveAcqRel(reinterpret_cast<unsigned *>(d.ltsWork + kLwArrUpd), 1u) + 1u == gridDim.x;
            __syncthreads();
            if (sLast) {
                if (t == 0) d.ltsWork[kLwArrUpd] = 0;
                ltsEndIteration(d);
            }
        }
    } else {
        const int segEnd = d.ctaSeg[blockIdx.x + 1];
        for (int seg = d.ctaSeg[blockIdx.x]; seg < segEnd; ++seg) segment(d.units[seg], 1u, 0u);
    }
}

/// speed pass of the split block: x-edges (x|x+1), x = 0..nx, over every row
/// 0..ny+1 including the ghost rows (src/blocks/SWE_DimensionalSplitting.cpp:118-131)
template <int S> __global__ void __launch_bounds__(kMaxTileRows) speedSplitKernel(const DomainDev d) {
    __shared__ float sRed[kMaxTileRows / 32];
    __shared__ int sLast;
    const int TY = blockDim.x;
    const int segEnd = d.ctaSeg[blockIdx.x + 1];
    for (int seg = d.ctaSeg[blockIdx.x]; seg < segEnd; ++seg) {
        const WorkUnit wu = d.units[seg];
        const BlockDesc B = d.blocks[wu.block];
        GroupState *G = d.groups + B.group;
        if (!groupActive(G)) continue;
        const int cur = __ldg(&G->cur);
        const float *__restrict__ H = pick(d.h, cur) + B.base;
        const float *__restrict__ HU = pick(d.hu, cur) + B.base;
        const float *__restrict__ BT = d.b + B.base;
        const size_t P = size_t(B.pitch);
        const int yTop = min(wu.y0 + TY - 1, B.ny);
        const int rLo = (wu.y0 == 1) ? 0 : wu.y0;
        const int rHi = (yTop == B.ny) ? B.ny + 1 : yTop;
        float smax = 0.f;
        for (int r = rLo + int(threadIdx.x); r <= rHi; r += TY) {
            Cell prev, dummy;
            {
                const size_t o = size_t(wu.x0 - 1) * P + r;
                cellQuantities<S>(H[o], HU[o], 0.f, BT[o], prev, dummy);
            }
            for (int x = wu.x0; x <= wu.x1; ++x) {
                const size_t o = size_t(x) * P + r;
                Cell c;
                cellQuantities<S>(H[o], HU[o], 0.f, BT[o], c, dummy);
                smax = vmax(smax, edgeSpeed<S>(prev, c));
                prev = c;
            }
        }
        segmentDone<false>(d, G, smax, sRed, &sLast, cur);
    }
}

} // namespace swegb
