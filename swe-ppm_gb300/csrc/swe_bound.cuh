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
//  - each warp takes one tile: it evaluates exactly one edge at the tile's
//    largest bound and adds that speed to the group's running maximum at once;
//    the running maximum T read afterwards is the speed of some edge, hence a
//    lower bound of the step's maximum;
//  - the tile's edges are evaluated only when its bound times a small margin
//    reaches T.
// Every skipped edge is slower than T, so the maximum over the evaluated
// edges is the maximum over all edges, whatever order the warps run in.
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

/// exact speed of one edge next to interior cell (x, y) of a block: the
/// x-edge to its left neighbour (right neighbour in column 1), else the
/// y-edge below (above in row 1); -1 for a 1 x 1 block
template <int S>
__device__ __forceinline__ float sampleEdgeSpeed(const float *H, const float *HU, const float *HV, size_t P, int x,
                                                 int y, int nx, int ny) {
    int xa = x, ya = y, xb = x, yb = y;
    bool alongX = true;
    if (x > 1) xa = x - 1;
    else if (nx > 1) xb = x + 1;
    else if (y > 1) { ya = y - 1; alongX = false; }
    else if (ny > 1) { yb = y + 1; alongX = false; }
    else return -1.f;
    Cell ax, ay, bx, by;
    cellAt<S>(H, HU, HV, size_t(xa) * P + size_t(ya), ax, ay);
    cellAt<S>(H, HU, HV, size_t(xb) * P + size_t(yb), bx, by);
    return alongX ? edgeSpeed<S>(ax, bx) : edgeSpeed<S>(ay, by);
}

/// exact maximum speed of the edges of columns [xa, xb) of a tile: x-edges
/// (x-1|x) and the y-edges of those columns (the block's top edge in the top
/// rim tile), plus (nx|nx+1) when xb = nx+1; lane = row y0 + lane, the loads
/// of all (at most NB) columns issued together
template <int S>
__device__ __forceinline__ float tileColumnsSpeed(const float *H, const float *HU, const float *HV, size_t P,
                                                  const TileInfo &I, int xa, int xb, int lane) {
    constexpr int NB = 4;
    const int y = I.y0 + lane;
    const bool active = y < I.y1;
    const bool top = y == I.ny && I.y1 == I.ny + 1;  // also owns (ny | ny+1)
    const int xEnd = xb == I.nx + 1 ? xb + 1 : xb;    // (nx | nx+1) on the right rim
    // columns xa-1 .. xa+NB: the left neighbour, up to NB tile columns and the
    // right ghost column
    float h[NB + 2], hu[NB + 2], hv[NB + 2], hB[NB], hvB[NB], hT[NB], hvT[NB];
#pragma unroll
    for (int k = 0; k <= NB + 1; k++) {
        const int x = xa - 1 + k;
        const size_t o = size_t(x) * P + size_t(y);
        h[k] = 0.f; hu[k] = 0.f; hv[k] = 0.f;
        if (x < xEnd && active) { h[k] = H[o]; hu[k] = HU[o]; hv[k] = HV[o]; }
        if (k > 0 && k <= NB) {
            hB[k - 1] = 0.f; hvB[k - 1] = 0.f; hT[k - 1] = 0.f; hvT[k - 1] = 0.f;
            if (x < xb && active) {
                if (lane == 0) { hB[k - 1] = H[o - 1]; hvB[k - 1] = HV[o - 1]; }
                if (top) { hT[k - 1] = H[o + 1]; hvT[k - 1] = HV[o + 1]; }
            }
        }
    }
    float smax = 0.f;
    Cell prevX, dummy;
    cellQuantities<S>(h[0], hu[0], hv[0], 0.f, prevX, dummy);
#pragma unroll
    for (int k = 1; k <= NB + 1; k++) {
        const int x = xa - 1 + k;
        if (x >= xEnd) continue;  // warp-uniform
        Cell cx, cy, below;
        cellQuantities<S>(h[k], hu[k], hv[k], 0.f, cx, cy);
        below.h = __shfl_up_sync(0xffffffffu, cy.h, 1);
        below.hn = __shfl_up_sync(0xffffffffu, cy.hn, 1);
        below.u = __shfl_up_sync(0xffffffffu, cy.u, 1);
        below.sq = __shfl_up_sync(0xffffffffu, cy.sq, 1);
        below.c = __shfl_up_sync(0xffffffffu, cy.c, 1);
        below.b = 0.f;
        if (active) {
            smax = vmax(smax, edgeSpeed<S>(prevX, cx));  // x-edge (x-1 | x)
            if (k <= NB && x < xb) {                     // a column of the tile: its y-edges
                if (lane == 0) cellQuantities<S>(hB[k - 1], 0.f, hvB[k - 1], 0.f, dummy, below);
                smax = vmax(smax, edgeSpeed<S>(below, cy));
                if (top) {
                    Cell above;
                    cellQuantities<S>(hT[k - 1], 0.f, hvT[k - 1], 0.f, dummy, above);
                    smax = vmax(smax, edgeSpeed<S>(cy, above));
                }
            }
        }
        prevX = cx;
    }
    return smax;
}

/// the group's speed pass is done when `count` more tiles are: max speed ->
/// dt (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456)
__device__ __forceinline__ void boundTilesDone(const DomainDev &d, GroupState *G, float m, int count) {
    atomicMax(&G->speedBits, __float_as_uint(m));
    __threadfence();
    const unsigned prev = atomicAdd(&G->arrived, unsigned(count));
    if (prev + unsigned(count) == unsigned(G->tiles)) {
        __threadfence();
        const float s = __uint_as_float(atomicOr(&G->speedBits, 0u));
        const BlockDesc &F = d.blocks[G->firstBlock];
        G->speed = s;
        G->dt = timestepFromSpeed(s, F.dx, F.dy, SEM_UNSPLIT);
        if (!(s == s)) G->status |= 1;
        G->speedBits = 0u;
        G->arrived = 0u;
        __threadfence();
    }
}

// One round = one tile per warp.  Each warp reads its tile's bound, samples
// one exact edge speed and decides; the CTA's candidate tiles are then
// evaluated by all its warps together, 4 columns per warp, so that a
// candidate costs a couple of memory latencies instead of a lone warp's
// serial march over 32 columns.
template <int S> __global__ void __launch_bounds__(256, 4) speedBoundKernel(const DomainDev d) {
    __shared__ float sMax[8], sRed[8];
    __shared__ int sGrp[8], sCnt[8];
    __shared__ int sCand[8], sNCand;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nwb = int(blockDim.x >> 5);
    int grp = -1, cnt = 0;
    float smax = 0.f;
    for (long long round = 0;; round++) {
        // consecutive tiles go to different CTAs
        const long long first = (long long)blockIdx.x + (long long)gridDim.x * (round * nwb);
        if (first >= d.ntiles) break;
        if (threadIdx.x == 0) sNCand = 0;
        __syncthreads();
        const long long it = first + (long long)gridDim.x * wib;
        if (it < d.ntiles) {
            const TileInfo I = d.tileInfo[it];
            if (I.group != grp) {
                if (grp >= 0 && cnt > 0) {
                    float m = smax;
                    for (int o = 16; o > 0; o >>= 1) m = vmax(m, __shfl_xor_sync(0xffffffffu, m, o));
                    if (lane == 0) boundTilesDone(d, d.groups + grp, m, cnt);
                }
                grp = I.group;
                cnt = 0;
                smax = 0.f;
            }
            GroupState *G = d.groups + grp;
            if (groupActive(G)) {
                cnt++;
                const int cur = G->cur;
                const bool valid = G->boundsValid[cur] != 0;
                const unsigned int *Wp = d.tileW + size_t(cur) * size_t(d.ntiles);
                float W = INFINITY;
                unsigned long long key = 0ull;
                if (valid) {
                    W = __uint_as_float(Wp[it]);
                    for (int s = 0; s < 4; s++) {
                        const int n = I.nbr[s];
                        if (n >= 0) W = vmax(W, __uint_as_float(Wp[n]));
                        else if (n == kNbrUnbounded) W = INFINITY;
                    }
                    key = d.tileKey[size_t(cur) * size_t(d.ntiles) + size_t(it)];
                }
                if (lane == 0) {  // clear the entry the next update pass folds into
                    d.tileW[size_t(cur ^ 1) * size_t(d.ntiles) + size_t(it)] = 0u;
                    d.tileKey[size_t(cur ^ 1) * size_t(d.ntiles) + size_t(it)] = 0ull;
                    float T = 0.f;
                    if (key) {
                        const size_t P = size_t(I.pitch);
                        const float sp = sampleEdgeSpeed<S>(pick(d.h, cur) + I.base, pick(d.hu, cur) + I.base,
                                                            pick(d.hv, cur) + I.base, P, int((key >> 16) & 0xffffull),
                                                            int(key & 0xffffull), I.nx, I.ny);
                        if (sp > 0.f) {
                            smax = vmax(smax, sp);
                            // the running maximum after this sample: a lower bound
                            T = vmax(__uint_as_float(atomicMax(&G->speedBits, __float_as_uint(sp))), sp);
                        }
                    }
                    if (!(W * kBoundMargin < T)) sCand[atomicAdd(&sNCand, 1)] = int(it - first) / int(gridDim.x);
                }
            }
        }
        __syncthreads();
        // the candidates of this round, all warps on each
        const int ncand = sNCand;
        for (int c = 0; c < ncand; c++) {
            const long long ct = first + (long long)gridDim.x * sCand[c];
            const TileInfo I = d.tileInfo[ct];
            GroupState *G = d.groups + I.group;
            const int cur = G->cur;
            const int xa = I.x0 + 4 * wib;
            float m = 0.f;
            if (xa < I.x1) {
                const int xb = min(xa + 4, I.x1);
                m = tileColumnsSpeed<S>(pick(d.h, cur) + I.base, pick(d.hu, cur) + I.base, pick(d.hv, cur) + I.base,
                                        size_t(I.pitch), I, xa, xb, lane);
            }
            for (int o = 16; o > 0; o >>= 1) m = vmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) sRed[wib] = m;
            __syncthreads();
            if (threadIdx.x == 0) {
                float mm = sRed[0];
                for (int w = 1; w < nwb; w++) mm = vmax(mm, sRed[w]);
                atomicMax(&G->speedBits, __float_as_uint(mm));
            }
            __syncthreads();
        }
    }
    // combine the warps of the CTA per group, one arrival per group
    float m = smax;
    for (int o = 16; o > 0; o >>= 1) m = vmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
        sMax[wib] = m;
        sGrp[wib] = grp;
        sCnt[wib] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < nwb; w++) {
            const int g = sGrp[w];
            if (g < 0 || sCnt[w] == 0) continue;
            float mg = sMax[w];
            int cg = sCnt[w];
            for (int v = w + 1; v < nwb; v++)
                if (sGrp[v] == g && sCnt[v] > 0) {
                    mg = vmax(mg, sMax[v]);
                    cg += sCnt[v];
                    sCnt[v] = 0;
                }
            boundTilesDone(d, d.groups + g, mg, cg);
        }
    }
}

} // namespace swegb
