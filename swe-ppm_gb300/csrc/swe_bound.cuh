// Bounded speed pass of the f-wave / HLLE unsplit step.
//
// computeNumericalFluxes needs the maximum wave speed over all edges of the
// step (src/blocks/SWE_DimensionalSplittingMpi.cpp:391-456).  The full speed
// pass evaluates every edge for that.  This pass returns the same maximum,
// bit for bit, from far fewer edges:
//  - the previous update pass folded, for every bound tile (32 x 32 cells of
//    a block), the largest speed bound of its new cells (cellSpeedBound) and a
//    cell attaining it into the tile's entry;
//  - every edge a tile owns touches only the tile's cells and the cells across
//    its left / bottom (and, on the block's rim, right / top) side, so its
//    speed is at most the largest of those tiles' bounds (the ghosts of wall
//    and outflow sides copy the tile's own cells; other ghosts are unbounded);
//  - each warp takes one tile and evaluates exactly the edge at the tile's
//    largest bound, and the fastest edge of the last pass; the largest of
//    these exact speeds within the CTA is a lower bound T of the maximum;
//  - the tile's edges are evaluated only when its bound times a small margin
//    reaches T.
// Every skipped edge is slower than T, so the maximum over the evaluated
// edges is the maximum over all edges.  The last pass's fastest edge moves
// little between steps, so T is almost always within a few ulp of the new
// maximum and only the tiles that can reach it are evaluated.  Group state is
// read through the read-only path and the pass's atomics touch one key and
// one counter per CTA, so no cache line serialises the grid.
// Without valid bounds (first step, after an upload) every edge is evaluated.
//
// The pass also clears the other parity's tile entries for the update pass
// that follows (stale entries would only loosen the bounds).
#pragma once

#include "swe_sweep.cuh"

namespace swegb {

template <int S>
__device__ __forceinline__ void cellAt(const float *H, const float *HU, const float *HV, size_t o, Cell &cx, Cell &cy) {
    cellQuantities<S>(H[o], HU[o], HV[o], 0.f, cx, cy);
}

/// speed of the edge between the cells at element offsets oa (left / below)
/// and ob (right / above) of the current buffer; dir 0: x-edge, 1: y-edge
template <int S>
__device__ __forceinline__ float edgeSpeedAt(const float *H, const float *HU, const float *HV, long long oa,
                                             long long ob, int dir) {
    Cell ax, ay, bx, by;
    cellQuantities<S>(__ldg(H + oa), __ldg(HU + oa), __ldg(HV + oa), 0.f, ax, ay);
    cellQuantities<S>(__ldg(H + ob), __ldg(HU + ob), __ldg(HV + ob), 0.f, bx, by);
    return dir ? edgeSpeed<S>(ay, by) : edgeSpeed<S>(ax, bx);
}

/// code of the edge whose right / upper cell is (x, y) of bound tile `tile`
__device__ __forceinline__ unsigned int edgeCode(long long tile, const TileInfo &I, int x, int y, int dir) {
    return (unsigned(tile) << 13) | (unsigned(dir) << 12) | (unsigned(x - I.x0) << 6) | unsigned(y - I.y0);
}

/// the sample edge next to interior cell (x, y) of a block: the x-edge to its
/// left neighbour (right neighbour in column 1), else the y-edge below (above
/// in row 1); false for a 1 x 1 block.  Offsets include the block's base.
__device__ __forceinline__ bool sampleEdge(const TileInfo &I, long long tile, int x, int y, long long &oa,
                                           long long &ob, int &dir, unsigned int &code) {
    const long long P = I.pitch;
    int xb = x, yb = y;
    dir = 0;
    if (x > 1) {
    } else if (I.nx > 1) {
        xb = x + 1;
    } else if (y > 1) {
        dir = 1;
    } else if (I.ny > 1) {
        yb = y + 1;
        dir = 1;
    } else {
        return false;
    }
    ob = I.base + xb * P + yb;
    oa = dir ? ob - 1 : ob - P;
    code = edgeCode(tile, I, xb, yb, dir);
    return true;
}

__device__ __forceinline__ unsigned long long speedKey(float s, unsigned int code) {
    return ((unsigned long long)__float_as_uint(s) << 32) | code;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

/// exact speeds of the edges of columns [xa, xb) of a tile: x-edges (x-1|x)
/// and the y-edges of those columns (the block's top edge in the top rim
/// tile), plus (nx|nx+1) when xb = nx+1; lane = row y0 + lane, the loads of
/// all (at most NB) columns issued together.  An edge is solved only when the
/// larger speed bound of its two cells (cellSpeedBound, from the cells' own
/// values, ghosts included) reaches T, a speed some edge of the group has:
/// every skipped edge is slower than the maximum and cannot attain it.
/// Returns the lane's fastest edge as a speed key.
template <int S>
__device__ __forceinline__ unsigned long long tileColumnsSpeed(const float *H, const float *HU, const float *HV,
                                                               size_t P, const TileInfo &I, long long tile, int xa,
                                                               int xb, int lane, float T) {
    constexpr int NB = 4;
    const int y = I.y0 + lane;
    const bool active = y < I.y1;
    const bool top = y == I.ny && I.y1 == I.ny + 1;  // also owns (ny | ny+1)
    const int xEnd = xb == I.nx + 1 ? xb + 1 : xb;    // (nx | nx+1) on the right rim
    // columns xa-1 .. xa+NB: the left neighbour, up to NB tile columns and the
    // right ghost column
    float h[NB + 2], hu[NB + 2], hv[NB + 2];
#pragma unroll
    for (int k = 0; k <= NB + 1; k++) {
        const int x = xa - 1 + k;
        const size_t o = size_t(x) * P + size_t(y);
        h[k] = 0.f; hu[k] = 0.f; hv[k] = 0.f;
        if (x < xEnd && active) { h[k] = H[o]; hu[k] = HU[o]; hv[k] = HV[o]; }
    }
    // the cell below the tile's first row (lanes 0 .. NB-1, column xa + lane)
    // and, in the block's top rim tile, the ghost above its last row (lanes
    // NB .. 2NB-1): loaded once per lane, handed to lane 0 / the top lane by
    // shuffles (h and hv are all a y-edge needs)
    float eh = 0.f, ehv = 0.f;
    {
        const int x = xa + (lane & (NB - 1));
        if (x < xb) {
            if (lane < NB) {
                const size_t o = size_t(x) * P + size_t(I.y0 - 1);
                eh = H[o];
                ehv = HV[o];
            } else if (lane < 2 * NB && I.y1 == I.ny + 1) {
                const size_t o = size_t(x) * P + size_t(I.ny + 1);
                eh = H[o];
                ehv = HV[o];
            }
        }
    }
    unsigned long long best = 0ull;
    float wPrev = cellSpeedBound(h[0], hu[0], hv[0]);
#pragma unroll
    for (int k = 1; k <= NB + 1; k++) {
        const int x = xa - 1 + k;
        if (x >= xEnd) continue;  // warp-uniform
        const float w = cellSpeedBound(h[k], hu[k], hv[k]);
        // the cell below: the previous lane's, the tile's lower neighbour for lane 0
        float hBl = __shfl_up_sync(0xffffffffu, h[k], 1);
        float hvBl = __shfl_up_sync(0xffffffffu, hv[k], 1);
        float wBl = __shfl_up_sync(0xffffffffu, w, 1);
        const int kk = k <= NB ? k - 1 : 0;
        const float eB = __shfl_sync(0xffffffffu, eh, kk), eBv = __shfl_sync(0xffffffffu, ehv, kk);
        const float eT = __shfl_sync(0xffffffffu, eh, NB + kk), eTv = __shfl_sync(0xffffffffu, ehv, NB + kk);
        if (active) {
            if (!(vmax(wPrev, w) * kBoundMargin < T)) {  // x-edge (x-1 | x)
                Cell L, R, dummy;
                cellQuantities<S>(h[k - 1], hu[k - 1], hv[k - 1], 0.f, L, dummy);
                cellQuantities<S>(h[k], hu[k], hv[k], 0.f, R, dummy);
                const float sx = edgeSpeed<S>(L, R);
                if (sx > 0.f) best = umax64(best, speedKey(sx, edgeCode(tile, I, x, y, 0)));
            }
            if (k <= NB && x < xb) {                     // a column of the tile: its y-edges
                if (lane == 0) {
                    hBl = eB;
                    hvBl = eBv;
                    wBl = cellSpeedBound(hBl, 0.f, hvBl);
                }
                if (!(vmax(wBl, w) * kBoundMargin < T)) {
                    Cell L, R, dummy;
                    cellQuantities<S>(hBl, 0.f, hvBl, 0.f, dummy, L);
                    cellQuantities<S>(h[k], hu[k], hv[k], 0.f, dummy, R);
                    const float sy = edgeSpeed<S>(L, R);
                    if (sy > 0.f) best = umax64(best, speedKey(sy, edgeCode(tile, I, x, y, 1)));
                }
                if (top && !(vmax(w, cellSpeedBound(eT, 0.f, eTv)) * kBoundMargin < T)) {
                    Cell L, R, dummy;
                    cellQuantities<S>(h[k], hu[k], hv[k], 0.f, dummy, L);
                    cellQuantities<S>(eT, 0.f, eTv, 0.f, dummy, R);
                    const float st = edgeSpeed<S>(L, R);
                    if (st > 0.f) best = umax64(best, speedKey(st, edgeCode(tile, I, x, y + 1, 1)));
                }
            }
        }
        wPrev = w;
    }
    return best;
}

/// `count` more of the group's tiles are done, with their fastest edge `key`;
/// the last one sets maxTimestep (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456)
/// and remembers where the fastest edge was
__device__ __forceinline__ void boundTilesDone(const DomainDev &d, GroupState *G, unsigned long long key, int count) {
    if (key) atomicMax(&G->maxEdge, key);
    const unsigned prev = arriveAcqRel(&G->arrived, unsigned(count));
    if (prev + unsigned(count) == unsigned(G->tiles)) {
        // every CTA's key and candidate count, acquired by the arrival; the
        // state written here is read by the next kernel after this grid ends
        const unsigned long long k = __ldcg(&G->maxEdge);
        const int cands = __ldcg(&G->candidates);
        const float s = __uint_as_float(unsigned(k >> 32));  // every evaluated edge is in the key's maximum
        if (k) {
            const unsigned code = unsigned(k);
            const TileInfo I = d.tileInfo[code >> 13];
            const int dir = (code >> 12) & 1;
            const long long x = I.x0 + ((code >> 6) & 63), y = I.y0 + (code & 63);
            G->prevB = I.base + x * I.pitch + y;
            G->prevA = dir ? G->prevB - 1 : G->prevB - I.pitch;
            G->prevDir = dir;
            G->prevValid = 1;
        }
        const BlockDesc &F = d.blocks[G->firstBlock];
        G->speed = s;
        G->dt = groupTimestep(d, G, s, F.dx, F.dy);
        if (!(s == s)) G->status |= 1;
        G->lastCandidates = cands;
        G->candidates = 0;
        G->speedBits = 0u;
        G->maxEdge = 0ull;
        G->arrived = 0u;
    }
}

// One round = one tile per warp.  Lanes 0 and 1 of each warp evaluate, side
// by side, the tile's sample edge and the last pass's fastest edge; every warp
// compares its tile's bound with the CTA's largest sample in the same group.
// The CTA's candidate tiles are then evaluated by all its warps together, 4
// columns per warp.
template <int S> __global__ void __launch_bounds__(256, 4) speedBoundKernel(const DomainDev d) {
    __shared__ float sSamp[8], sW[8];
    __shared__ int sGrp[8], sCnt[8], sTileGrp[8];
    __shared__ unsigned long long sKey[8];
    __shared__ int sCand[8], sNCand;
    __shared__ float sCandT[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nwb = int(blockDim.x >> 5);
    {
        // tile records are written only when the domain is built: bring the
        // first round's into L1 before waiting for the previous kernel
        const long long slot = (long long)blockIdx.x + (long long)gridDim.x * wib;
        if (lane == 0 && slot < d.ntiles)
            prefetchL1(&d.tileInfo[(unsigned long long)slot * d.tileHashMul % (unsigned long long)d.ntiles]);
    }
    pdlWaitAndRelease();
    int grp = -1, cnt = 0;
    unsigned long long bkey = 0ull;  // lane 0: the warp's fastest edge so far (group grp)
    for (long long round = 0;; round++) {
        // consecutive tiles go to different CTAs
        const long long first = (long long)blockIdx.x + (long long)gridDim.x * (round * nwb);
        if (first >= d.ntiles) break;
        if (threadIdx.x == 0) sNCand = 0;
        const long long slot = first + (long long)gridDim.x * wib;
        // 1. bound and exact samples.  Tiles are dealt out by a multiplicative
        // hash so that neighbouring candidates land on different CTAs; the
        // loads of the bound, the key and the group state are issued together
        // (both parities, selected afterwards), so the chain is: tile record,
        // bounds and group state, sample cells.
        const long long it = slot < d.ntiles ? (long long)((unsigned long long)slot * d.tileHashMul % (unsigned long long)d.ntiles) : slot;
        int tgrp = -1;
        float W = INFINITY, samp = 0.f;
        if (slot < d.ntiles) {
            const TileInfo I = d.tileInfo[it];
            if (I.group != grp) {
                if (grp >= 0 && cnt > 0 && lane == 0) boundTilesDone(d, d.groups + grp, bkey, cnt);
                grp = I.group;
                cnt = 0;
                bkey = 0ull;
            }
            const GroupState *G = d.groups + grp;
            // group state (constant during the pass: read-only path, one L2
            // fetch per SM) and both parities of the tile entries at once
            const float gTime = __ldg(&G->time), gTarget = __ldg(&G->target);
            const int gEnabled = __ldg(&G->enabled);
            const int cur = __ldg(&G->cur), bv0 = __ldg(&G->boundsValid[0]), bv1 = __ldg(&G->boundsValid[1]);
            const int pValid = __ldg(&G->prevValid), pDir = __ldg(&G->prevDir);
            const long long pA = __ldg(&G->prevA), pB = __ldg(&G->prevB);
            float w0 = 0.f, w1 = 0.f;
            unsigned long long k0 = 0ull, k1 = 0ull;
            if (lane == 0) {
                w0 = __uint_as_float(__ldg(&d.tileW[it]));
                w1 = __uint_as_float(__ldg(&d.tileW[size_t(d.ntiles) + size_t(it)]));
                for (int sd = 0; sd < 4; sd++) {
                    const int n = I.nbr[sd];
                    if (n >= 0) {
                        w0 = vmax(w0, __uint_as_float(__ldg(&d.tileW[n])));
                        w1 = vmax(w1, __uint_as_float(__ldg(&d.tileW[size_t(d.ntiles) + size_t(n)])));
                    } else if (n == kNbrUnbounded) {
                        w0 = INFINITY;
                        w1 = INFINITY;
                    }
                }
                k0 = __ldg(&d.tileKey[it]);
                k1 = __ldg(&d.tileKey[size_t(d.ntiles) + size_t(it)]);
            }
            if (gTime < gTarget && gEnabled) {
                cnt++;
                tgrp = grp;
                long long oa = 0, ob = 0;
                int dir = 0;
                unsigned int code = 0;
                bool have = false;
                if (lane == 0) {
                    const bool valid = cur ? bv1 : bv0;
                    const unsigned long long key = valid ? (cur ? k1 : k0) : 0ull;
                    if (valid) W = cur ? w1 : w0;
                    // clear the entry the next update pass folds into
                    d.tileW[size_t(cur ^ 1) * size_t(d.ntiles) + size_t(it)] = 0u;
                    d.tileKey[size_t(cur ^ 1) * size_t(d.ntiles) + size_t(it)] = 0ull;
                    if (key) have = sampleEdge(I, it, int((key >> 16) & 0xffffull), int(key & 0xffffull), oa, ob, dir, code);
                } else if (lane == 1 && pValid) {
                    oa = pA;
                    ob = pB;
                    dir = pDir;
                    have = true;  // code 0: already known
                }
                float sp = 0.f;
                if (have)
                    sp = vmax(0.f, edgeSpeedAt<S>(pick(d.h, cur), pick(d.hu, cur), pick(d.hv, cur), oa, ob, dir));
                const float sp1 = __shfl_down_sync(0xffffffffu, sp, 1);
                if (lane == 0) {
                    samp = vmax(sp, sp1);
                    if (sp > 0.f) bkey = umax64(bkey, speedKey(sp, code));
                }
            }
        }
        if (lane == 0) {
            sSamp[wib] = samp;
            sW[wib] = W;
            sTileGrp[wib] = tgrp;
        }
        __syncthreads();
        // 2. the largest exact speed the CTA sampled in the tile's group (the
        // last pass's fastest edge among them) is a lower bound T
        if (lane == 0 && tgrp >= 0) {
            float T = 0.f;
            for (int v = 0; v < nwb; v++)
                if (sTileGrp[v] == tgrp) T = vmax(T, sSamp[v]);
            if (!(W * kBoundMargin < T)) {
                const int c = atomicAdd(&sNCand, 1);
                sCand[c] = wib;
                sCandT[c] = T;
            }
        }
        __syncthreads();
        // 3. the candidates of this round, all warps on each
        const int ncand = sNCand;
        for (int c = 0; c < ncand; c++) {
            const long long ct = (long long)((unsigned long long)(first + (long long)gridDim.x * sCand[c]) *
                                             d.tileHashMul % (unsigned long long)d.ntiles);
            const TileInfo I = d.tileInfo[ct];
            GroupState *G = d.groups + I.group;
            const int cur = __ldg(&G->cur);
            const int xa = I.x0 + 4 * wib;
            unsigned long long k = 0ull;
            if (xa < I.x1)
                k = tileColumnsSpeed<S>(pick(d.h, cur) + I.base, pick(d.hu, cur) + I.base, pick(d.hv, cur) + I.base,
                                        size_t(I.pitch), I, ct, xa, min(xa + 4, I.x1), lane, sCandT[c]);
            for (int o = 16; o > 0; o >>= 1) k = umax64(k, __shfl_xor_sync(0xffffffffu, k, o));
            if (lane == 0) sKey[wib] = k;
            __syncthreads();
            if (threadIdx.x == 0) {
                atomicAdd(&G->candidates, 1);
                unsigned long long kk = sKey[0];
                for (int w = 1; w < nwb; w++) kk = umax64(kk, sKey[w]);
                if (kk) atomicMax(&G->maxEdge, kk);
            }
            __syncthreads();
        }
    }
    // combine the warps of the CTA per group, one arrival per group
    if (lane == 0) {
        sKey[wib] = bkey;
        sGrp[wib] = grp;
        sCnt[wib] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < nwb; w++) {
            const int g = sGrp[w];
            if (g < 0 || sCnt[w] == 0) continue;
            unsigned long long kg = sKey[w];
            int cg = sCnt[w];
            for (int v = w + 1; v < nwb; v++)
                if (sGrp[v] == g && sCnt[v] > 0) {
                    kg = umax64(kg, sKey[v]);
                    cg += sCnt[v];
                    sCnt[v] = 0;
                }
            boundTilesDone(d, d.groups + g, kg, cg);
        }
    }
}

} // namespace swegb
