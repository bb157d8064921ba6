// Step kernels of the block step, templated on solver and semantics.
//
// One global time step of a group of blocks is three launches:
//   ghostKernel      setGhostLayer: boundary conditions + on-device halo copies
//                    between blocks (src/blocks/SWE_Block.hh:757-911,
//                    src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304)
//   sweepKernel<..., false>  speed pass: every edge's max wave speed, CTA max
//                    by warp shuffles, group max by atomicMax; the last CTA of
//                    the group turns it into maxTimestep
//                    (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-472)
//   sweepKernel<..., true>   fused pass: solves every edge again, sums the net
//                    updates per cell in registers and writes Q^{n+1} with the
//                    dry clamp (src/blocks/SWE_DimensionalSplittingMpi.cpp:484-518)
//                    or the split update (src/blocks/SWE_DimensionalSplitting.cpp:187-210)
// The speed pass is needed because dt depends on the same step's wave speeds;
// at 2048^2 the state (67 MB) stays in L2 between the two passes, so DRAM
// sees each input byte once.
//
// Tiling: a CTA owns TY = blockDim.x consecutive rows (one per thread, y is the
// contiguous direction) of an x-chunk [x0, x1) of one block and marches along
// x.  The x-edge (x-1|x) is solved from the previous column kept in registers;
// the y-edge (y|y+1) from the neighbouring thread's cell in shared memory; the
// tile's two boundary y-edges per column are solved up front.  Every cell's
// update is finished one column later, when its right edge is known.
#pragma once

#include "swe_device.cuh"

namespace swegb {

__device__ __forceinline__ float blockReduceMax(float v, float *sRed) {
    for (int o = 16; o > 0; o >>= 1) v = vmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
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

/// buffer p of a double-buffered field without dynamic indexing of the kernel parameter
__device__ __forceinline__ float *pick(float *const (&f)[2], int p) { return p ? f[1] : f[0]; }

__device__ __forceinline__ bool groupActive(const GroupState *G) {
    return *((volatile const float *)&G->time) < *((volatile const float *)&G->target);
}

template <int S> __device__ __forceinline__ void cellQuantities(float h, float hu, float hv, float b, Cell &cx, Cell &cy) {
    const bool wet = !(h < kDryTol);
    float sq = 0.f, c = 0.f, ux = 0.f, uy = 0.f;
    if (S != SOLVER_AUGRIE) {
        sq = sqrtf(h);
        if (S == SOLVER_HLLE) c = sqrtf(kG * h);
        ux = wet ? hu / h : 0.f;
        uy = wet ? hv / h : 0.f;
    }
    cx = makeCell(h, hu, b, ux, sq, c);
    cy = makeCell(h, hv, b, uy, sq, c);
}

template <int S, int SEM, bool UPDATE>
__global__ void __launch_bounds__(kMaxTileRows) sweepKernel(const DomainDev d) {
    __shared__ float sC[2][6][kMaxTileRows];   // y-direction cell quantities of column x
    __shared__ float sR[2][2][kMaxTileRows];   // right-going (h, hv) update into row t
    __shared__ float sBot[2][kMaxTileCols];    // right-going update into row y0 (bottom tile edge)
    __shared__ float sTop[2][kMaxTileCols];    // left-going update into row yTop (top tile edge)
    __shared__ float sRed[kMaxTileRows / 32];
    __shared__ int sLast;

    const WorkUnit wu = d.units[blockIdx.x];
    const BlockDesc B = d.blocks[wu.block];
    GroupState *G = d.groups + B.group;
    if (!groupActive(G)) return;
    const int cur = G->cur;
    const float *__restrict__ H = pick(d.h, cur) + B.base;
    const float *__restrict__ HU = pick(d.hu, cur) + B.base;
    const float *__restrict__ HV = pick(d.hv, cur) + B.base;
    const float *__restrict__ BT = d.b + B.base;
    const size_t P = size_t(B.pitch);
    const int t = threadIdx.x, TY = blockDim.x;
    const int x0 = wu.x0, x1 = wu.x1, XC = x1 - x0;
    const int y0 = wu.y0;
    const int y = y0 + t;
    const int yTop = min(y0 + TY - 1, B.ny);
    const bool active = y <= yTop;
    float smax = 0.f;

    float dtdx = 0.f, dtdy = 0.f;
    if (UPDATE) {
        const float dt = G->dt;
        dtdx = dt / B.dx;
        dtdy = (SEM == SEM_SPLIT) ? dtdx : dt / B.dy;
    }

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
            edgeSolve<S>(L, R, aL, aR, auL, auR, s);
            if (top) {
                sTop[0][k] = aL;
                sTop[1][k] = auL;
            } else {
                sBot[0][k] = aR;
                sBot[1][k] = auR;
            }
            // carry the ghost rows (set by this step's ghost layer) into the
            // output buffer, where the reference keeps them after the update
            const bool ghostRow = top ? (yTop == B.ny) : (y0 == 1);
            if (ghostRow) {
                const size_t g = top ? o + 1 : o;
                pick(d.h, cur ^ 1)[B.base + g] = H[g];
                pick(d.hu, cur ^ 1)[B.base + g] = HU[g];
                pick(d.hv, cur ^ 1)[B.base + g] = HV[g];
            }
        } else {
            smax = vmax(smax, edgeSpeed<S>(L, R));
        }
    }

    float *__restrict__ HO = UPDATE ? pick(d.h, cur ^ 1) + B.base : nullptr;
    float *__restrict__ HUO = UPDATE ? pick(d.hu, cur ^ 1) + B.base : nullptr;
    float *__restrict__ HVO = UPDATE ? pick(d.hv, cur ^ 1) + B.base : nullptr;
    if (UPDATE && t == 0) {  // corner ghosts of the block, carried over like the rest of the ring
        const int cx[2] = {0, B.nx + 1}, cyy[2] = {0, B.ny + 1};
        const bool hasX[2] = {x0 == 1, x1 == B.nx + 1}, hasY[2] = {y0 == 1, yTop == B.ny};
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                if (hasX[i] && hasY[j]) {
                    const size_t o = size_t(cx[i]) * P + size_t(cyy[j]);
                    HO[o] = H[o]; HUO[o] = HU[o]; HVO[o] = HV[o];
                }
    }

    float nh = 0.f, nhu = 0.f, nhv = 0.f, nb = 0.f;
    if (active) {
        const size_t o = size_t(x0 - 1) * P + y;
        nh = H[o]; nhu = HU[o]; nhv = HV[o]; nb = BT[o];
    }
    Cell prevX = makeCell(0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
    float pendH = 0.f, pendHU = 0.f;                 // right-going x-update into cell x
    float oldH = 0.f, oldHU = 0.f, oldHV = 0.f;      // Q^n of cell x-1
    float syH = 0.f, syHV = 0.f;                     // y net-update sums of cell x-1
    bool bad = false;                                // a non-finite water height was produced

    for (int x = x0 - 1; x <= x1; ++x) {
        const float ch = nh, chu = nhu, chv = nhv, cb = nb;
        if (x < x1 && active) {
            const size_t o = size_t(x + 1) * P + y;
            nh = H[o]; nhu = HU[o]; nhv = HV[o]; nb = BT[o];
        }
        Cell cx, cy;
        cellQuantities<S>(ch, chu, chv, cb, cx, cy);
        if (UPDATE && active && (x == 0 || x == B.nx + 1)) {  // ghost columns carried over
            const size_t o = size_t(x) * P + y;
            HO[o] = ch; HUO[o] = chu; HVO[o] = chv;
        }

        // x-edge (x-1 | x)
        if (x >= x0 && active) {
            if (UPDATE) {
                float aL, aR, auL, auR, s;
                edgeSolve<S>(prevX, cx, aL, aR, auL, auR, s);
                if (x - 1 >= x0) {
                    const size_t o = size_t(x - 1) * P + y;
                    if (SEM == SEM_UNSPLIT) {
                        const float sxH = pendH + aL, sxHU = pendHU + auL;
                        float hn = oldH - (dtdx * sxH + dtdy * syH);
                        float hun = oldHU - dtdx * sxHU;
                        float hvn = oldHV - dtdy * syHV;
                        if (hn < 0.f) {
                            hn = 0.f; hun = 0.f; hvn = 0.f;
                        } else if (hn < 0.1f) {
                            hun = 0.f; hvn = 0.f;
                        }
                        bad |= !(fabsf(hn) <= FLT_MAX);
                        HO[o] = hn; HUO[o] = hun; HVO[o] = hvn;
                    } else {
                        const float sxH = aL + pendH, sxHU = auL + pendHU;
                        const float hStar = oldH - dtdx * sxH;
                        const float hn = hStar - dtdx * syH;
                        bad |= !(fabsf(hn) <= FLT_MAX);
                        HO[o] = hn;
                        HUO[o] = oldHU - dtdx * sxHU;
                        HVO[o] = oldHV - dtdx * syHV;
                    }
                }
                pendH = aR;
                pendHU = auR;
            } else {
                smax = vmax(smax, edgeSpeed<S>(prevX, cx));
            }
        }
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
                    edgeSolve<S>(cy, up, bLh, bR, bLhv, bRhv, s);
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

    if (UPDATE) {
        // the last CTA of the group advances the group's clock and buffer
        if (__syncthreads_or(bad) && t == 0) atomicOr(&G->status, 2);
        if (t == 0) {
            __threadfence();
            const unsigned prev = atomicAdd(&G->arrived, 1u);
            sLast = (prev == unsigned(G->units) - 1u);
        }
        __syncthreads();
        if (sLast && t == 0) {
            __threadfence();
            G->arrived = 0u;
            G->time = G->time + G->dt;
            G->steps = G->steps + 1;
            G->cur = cur ^ 1;
            __threadfence();
        }
    } else {
        const float m = blockReduceMax(smax, sRed);
        if (t == 0) {
            atomicMax(&G->speedBits, __float_as_uint(m));
            __threadfence();
            const unsigned prev = atomicAdd(&G->arrived, 1u);
            sLast = (prev == unsigned(G->units) - 1u);
        }
        __syncthreads();
        if (sLast && t == 0) {
            __threadfence();
            float s = __uint_as_float(atomicOr(&G->speedBits, 0u));
            const BlockDesc &F = d.blocks[G->firstBlock];
            if (SEM == SEM_SPLIT && d.splitDtMode == SPLIT_DT_LAST_EDGE) {
                // speed of the last x-edge the serial loop solves: (nx | nx+1) in row ny+1
                const float *Hc = pick(d.h, cur) + F.base, *HUc = pick(d.hu, cur) + F.base, *Bc = d.b + F.base;
                const size_t o = size_t(F.nx) * size_t(F.pitch) + size_t(F.ny + 1);
                const size_t o2 = o + size_t(F.pitch);
                Cell L, R, dummy;
                cellQuantities<S>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                cellQuantities<S>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
                s = vmax(0.f, edgeSpeed<S>(L, R));
            }
            G->speed = s;
            G->dt = timestepFromSpeed(s, F.dx, F.dy, SEM);
            if (!(s == s)) G->status |= 1;  // NaN wave speed
            G->speedBits = 0u;
            G->arrived = 0u;
            __threadfence();
        }
    }
}

/// speed pass of the split block: x-edges (x|x+1), x = 0..nx, over every row
/// 0..ny+1 including the ghost rows (src/blocks/SWE_DimensionalSplitting.cpp:118-131)
template <int S> __global__ void __launch_bounds__(kMaxTileRows) speedSplitKernel(const DomainDev d) {
    __shared__ float sRed[kMaxTileRows / 32];
    __shared__ int sLast;
    const WorkUnit wu = d.units[blockIdx.x];
    const BlockDesc B = d.blocks[wu.block];
    GroupState *G = d.groups + B.group;
    if (!groupActive(G)) return;
    const int cur = G->cur;
    const float *__restrict__ H = pick(d.h, cur) + B.base;
    const float *__restrict__ HU = pick(d.hu, cur) + B.base;
    const float *__restrict__ BT = d.b + B.base;
    const size_t P = size_t(B.pitch);
    const int TY = blockDim.x;
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
    const float m = blockReduceMax(smax, sRed);
    if (threadIdx.x == 0) {
        atomicMax(&G->speedBits, __float_as_uint(m));
        __threadfence();
        const unsigned prev = atomicAdd(&G->arrived, 1u);
        sLast = (prev == unsigned(G->units) - 1u);
    }
    __syncthreads();
    if (sLast && threadIdx.x == 0) {
        __threadfence();
        float s = __uint_as_float(atomicOr(&G->speedBits, 0u));
        const BlockDesc &F = d.blocks[G->firstBlock];
        if (d.splitDtMode == SPLIT_DT_LAST_EDGE) {
            const float *Hc = pick(d.h, cur) + F.base, *HUc = pick(d.hu, cur) + F.base, *Bc = d.b + F.base;
            const size_t o = size_t(F.nx) * size_t(F.pitch) + size_t(F.ny + 1);
            const size_t o2 = o + size_t(F.pitch);
            Cell L, R, dummy;
            cellQuantities<S>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
            cellQuantities<S>(Hc[o2], HUc[o2], 0.f, Bc[o2], R, dummy);
            s = vmax(0.f, edgeSpeed<S>(L, R));
        }
        G->speed = s;
        G->dt = timestepFromSpeed(s, F.dx, F.dy, SEM_SPLIT);
        if (!(s == s)) G->status |= 1;
        G->speedBits = 0u;
        G->arrived = 0u;
        __threadfence();
    }
}

} // namespace swegb
