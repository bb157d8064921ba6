// Warp-synchronous step kernels (an alternative thread mapping of the sweep).
//
// Same two passes as swe_sweep.cuh (speed pass, fused solve + update with the
// ghost push), different mapping: every WARP owns a strip of 32*R consecutive
// rows (lane l holds rows y0 + R*l .. y0 + R*l + R-1, loaded with one 16-byte
// load per field when R = 4) of one block and marches along x over its column
// range.  Per column:
//   * x-edges (x-1|x): R solves against the previous column kept in registers;
//   * y-edges: R-1 edges inside the lane, one edge to lane l+1 (its cell via
//     __shfl_down), and the strip's bottom/top edges, which the warp solves up
//     front for 32 columns at a time (lane k for column c0+k) and hands out by
//     __shfl_sync;
// so the march needs no shared memory and no block-wide barrier.  A cell's
// update is finished one column later, when its right edge is known.
#pragma once

#include "swe_sweep.cuh"

namespace swegb {

template <int R> struct Quad {
    float v[R];
};

/// loads rows y .. y+R-1 of one column field (one 8- or 16-byte load when
/// aligned and fully inside the block, scalar loads of the valid rows otherwise)
template <int R>
__device__ __forceinline__ Quad<R> loadQuad(const float *__restrict__ f, size_t o, int validRows, bool vec) {
    Quad<R> q;
    if (vec && validRows == R) {
        if (R == 4) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(f + o));
            q.v[0] = t.x; q.v[1] = t.y; q.v[2] = t.z; q.v[3] = t.w;
        } else if (R == 2) {
            const float2 t = __ldg(reinterpret_cast<const float2 *>(f + o));
            q.v[0] = t.x; q.v[1] = t.y;
        } else {
#pragma unroll
            for (int r = 0; r < R; r++) q.v[r] = __ldg(f + o + r);
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; r++) q.v[r] = (r < validRows) ? __ldg(f + o + r) : 1.f;
    }
    return q;
}

/// stores R rows of one column field (one wide store when aligned)
template <int R> __device__ __forceinline__ void storeQuad(float *__restrict__ f, size_t o, const float *v) {
    if (R == 4) {
        *reinterpret_cast<float4 *>(f + o) = make_float4(v[0], v[1], v[2], v[3]);
    } else if (R == 2) {
        *reinterpret_cast<float2 *>(f + o) = make_float2(v[0], v[1]);
    } else {
#pragma unroll
        for (int r = 0; r < R; r++) f[o + r] = v[r];
    }
}

template <int S, int SEM, bool UPDATE, int R>
__global__ void __launch_bounds__(128) sweepWarpKernel(const DomainDev d) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);  // global warp id
    const int segEnd = d.ctaSeg[gw + 1];
    for (int seg = d.ctaSeg[gw]; seg < segEnd; ++seg) {
        const WorkUnit wu = d.units[seg];
        const BlockDesc B = d.blocks[wu.block];
        GroupState *G = d.groups + B.group;
        if (!groupActive(G)) continue;
        const int cur = G->cur;
        const float *__restrict__ H = pick(d.h, cur) + B.base;
        const float *__restrict__ HU = pick(d.hu, cur) + B.base;
        const float *__restrict__ HV = pick(d.hv, cur) + B.base;
        const float *__restrict__ BT = d.b + B.base;
        const size_t P = size_t(B.pitch);
        const int x0 = wu.x0, x1 = wu.x1;
        const int y0 = wu.y0;
        const int yTop = min(y0 + 32 * R - 1, B.ny);
        const int yl = y0 + R * lane;                    // first row of this lane
        const int valid = max(0, min(R, yTop - yl + 1));  // rows of this lane inside the strip
        // wide loads need the lane's first row on an R*4-byte boundary
        const bool vec = ((B.base + yl) % R) == 0 && (P % R) == 0;
        float dtdx = 0.f, dtdy = 0.f;
        if (UPDATE) {
            const float dt = G->dt;
            dtdx = dt / B.dx;
            dtdy = (SEM == SEM_SPLIT) ? dtdx : dt / B.dy;
        }
        float smax = 0.f;
        bool bad = false;

        Cell prevX[R];
        float pendH[R], pendHU[R], oldH[R], oldHU[R], oldHV[R], syH[R], syHV[R];
        // strip boundary edges of the current 32-column chunk (lane k: column c0 + k)
        float botH = 0.f, botHV = 0.f, topH = 0.f, topHV = 0.f;
        int chunk0 = -1;

        Quad<R> nh = loadQuad<R>(H, size_t(x0 - 1) * P + yl, valid, vec);
        Quad<R> nhu = loadQuad<R>(HU, size_t(x0 - 1) * P + yl, valid, vec);
        Quad<R> nhv = loadQuad<R>(HV, size_t(x0 - 1) * P + yl, valid, vec);
        Quad<R> nb = loadQuad<R>(BT, size_t(x0 - 1) * P + yl, valid, vec);
        // rows of this lane that need no ghost push (interior of the block in y)
        const bool innerRows = valid == R && yl > 1 && yl + R - 1 < B.ny;

        for (int x = x0 - 1; x <= x1; ++x) {
            const Quad<R> ch = nh, chu = nhu, chv = nhv, cb = nb;
            if (x < x1) {
                const size_t o = size_t(x + 1) * P + yl;
                nh = loadQuad<R>(H, o, valid, vec);
                nhu = loadQuad<R>(HU, o, valid, vec);
                nhv = loadQuad<R>(HV, o, valid, vec);
                nb = loadQuad<R>(BT, o, valid, vec);
            }
            // boundary y-edges of the strip for the next 32 columns
            if (x >= x0 && x < x1 && ((x - x0) & 31) == 0) {
                chunk0 = x;
                const int xc = x + lane;
                float bh = 0.f, bhv = 0.f, th = 0.f, thv = 0.f;
                if (xc < x1) {
                    const size_t ob = size_t(xc) * P + size_t(y0 - 1);
                    const size_t ot = size_t(xc) * P + size_t(yTop);
                    Cell L, Rr, dummy;
                    cellQuantities<S>(H[ob], HU[ob], HV[ob], BT[ob], dummy, L);
                    cellQuantities<S>(H[ob + 1], HU[ob + 1], HV[ob + 1], BT[ob + 1], dummy, Rr);
                    if (UPDATE) {
                        float a, b2, c, e, s;
                        edgeSolve<S>(L, Rr, a, b2, c, e, s);
                        bh = b2; bhv = e;  // right-going into row y0
                    } else {
                        smax = fmaxf(smax, edgeSpeed<S>(L, Rr));
                    }
                    cellQuantities<S>(H[ot], HU[ot], HV[ot], BT[ot], dummy, L);
                    cellQuantities<S>(H[ot + 1], HU[ot + 1], HV[ot + 1], BT[ot + 1], dummy, Rr);
                    if (UPDATE) {
                        float a, b2, c, e, s;
                        edgeSolve<S>(L, Rr, a, b2, c, e, s);
                        th = a; thv = c;  // left-going into row yTop
                    } else {
                        smax = fmaxf(smax, edgeSpeed<S>(L, Rr));
                    }
                }
                botH = bh; botHV = bhv; topH = th; topHV = thv;
            }

            Cell cx[R], cy[R];
#pragma unroll
            for (int r = 0; r < R; r++) cellQuantities<S>(ch.v[r], chu.v[r], chv.v[r], cb.v[r], cx[r], cy[r]);

            // x-edges (x-1 | x) and the finished cells of column x-1
            if (x >= x0) {
                float outH[R], outHU[R], outHV[R];
                const bool wide = UPDATE && vec && innerRows && x - 1 > 1 && x - 1 < B.nx && x - 1 >= x0;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    if (r >= valid) continue;
                    if (UPDATE) {
                        float aL, aR, auL, auR, s;
                        edgeSolve<S>(prevX[r], cx[r], aL, aR, auL, auR, s);
                        if (x - 1 >= x0) {
                            float hn, hun, hvn;
                            if (SEM == SEM_UNSPLIT) {
                                const float sxH = pendH[r] + aL, sxHU = pendHU[r] + auL;
                                hn = oldH[r] - (dtdx * sxH + dtdy * syH[r]);
                                hun = oldHU[r] - dtdx * sxHU;
                                hvn = oldHV[r] - dtdy * syHV[r];
                                if (hn < 0.f) {
                                    hn = 0.f; hun = 0.f; hvn = 0.f;
                                } else if (hn < 0.1f) {
                                    hun = 0.f; hvn = 0.f;
                                }
                            } else {
                                const float sxH = aL + pendH[r], sxHU = auL + pendHU[r];
                                const float hStar = oldH[r] - dtdx * sxH;
                                hn = hStar - dtdx * syH[r];
                                hun = oldHU[r] - dtdx * sxHU;
                                hvn = oldHV[r] - dtdx * syHV[r];
                            }
                            bad |= !(fabsf(hn) <= FLT_MAX);
                            outH[r] = hn; outHU[r] = hun; outHV[r] = hvn;
                            if (!wide) storeCell(d, B, cur ^ 1, P, x - 1, yl + r, hn, hun, hvn);
                        }
                        pendH[r] = aR;
                        pendHU[r] = auR;
                    } else {
                        smax = fmaxf(smax, edgeSpeed<S>(prevX[r], cx[r]));
                    }
                }
                if (wide) {
                    const size_t o = size_t(B.base) + size_t(x - 1) * P + size_t(yl);
                    storeQuad<R>(pick(d.h, cur ^ 1), o, outH);
                    storeQuad<R>(pick(d.hu, cur ^ 1), o, outHU);
                    storeQuad<R>(pick(d.hv, cur ^ 1), o, outHV);
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) prevX[r] = cx[r];

            // y-edges of column x
            if (x >= x0 && x < x1) {
                // the next lane's first cell (lane 31: the strip's top edge instead)
                Cell up;
                up.h = __shfl_down_sync(0xffffffffu, cy[0].h, 1);
                up.hn = __shfl_down_sync(0xffffffffu, cy[0].hn, 1);
                up.b = __shfl_down_sync(0xffffffffu, cy[0].b, 1);
                up.u = __shfl_down_sync(0xffffffffu, cy[0].u, 1);
                up.sq = __shfl_down_sync(0xffffffffu, cy[0].sq, 1);
                up.c = __shfl_down_sync(0xffffffffu, cy[0].c, 1);
                const int k = x - chunk0;
                const float tH = __shfl_sync(0xffffffffu, topH, k);
                const float tHV = __shfl_sync(0xffffffffu, topHV, k);
                const float bH = __shfl_sync(0xffffffffu, botH, k);
                const float bHV = __shfl_sync(0xffffffffu, botHV, k);
                float inL_H[R], inL_HV[R];    // left-going into row r from the edge above it
                float inR_H[R], inR_HV[R];    // right-going into row r from the edge below it
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int yr = yl + r;
                    const bool edgeInside = yr < yTop;  // edge (yr | yr+1) inside the strip
                    inL_H[r] = 0.f; inL_HV[r] = 0.f;
                    float oR = 0.f, oRHV = 0.f;
                    if (r < valid && edgeInside) {
                        const Cell &U = (r + 1 < R) ? cy[r + 1] : up;
                        if (UPDATE) {
                            float s;
                            edgeSolve<S>(cy[r], U, inL_H[r], oR, inL_HV[r], oRHV, s);
                        } else {
                            smax = fmaxf(smax, edgeSpeed<S>(cy[r], U));
                        }
                    }
                    if (UPDATE) {
                        if (r + 1 < R) {
                            inR_H[r + 1] = oR;
                            inR_HV[r + 1] = oRHV;
                        } else {
                            // hand the right-going part to the next lane's first row
                            inR_H[0] = __shfl_up_sync(0xffffffffu, oR, 1);
                            inR_HV[0] = __shfl_up_sync(0xffffffffu, oRHV, 1);
                        }
                        if (yr == yTop) {
                            inL_H[r] = tH;
                            inL_HV[r] = tHV;
                        }
                    }
                }
                if (UPDATE) {
                    if (lane == 0) {
                        inR_H[0] = bH;
                        inR_HV[0] = bHV;
                    }
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        if (SEM == SEM_UNSPLIT) {
                            syH[r] = inR_H[r] + inL_H[r];
                            syHV[r] = inR_HV[r] + inL_HV[r];
                        } else {
                            syH[r] = inL_H[r] + inR_H[r];
                            syHV[r] = inL_HV[r] + inR_HV[r];
                        }
                        oldH[r] = ch.v[r];
                        oldHU[r] = chu.v[r];
                        oldHV[r] = chv.v[r];
                    }
                }
            }
        }
        if (UPDATE) {
            if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&G->status, 2);
        }
        // segment done: warp-level reduction and arrival
        float m = smax;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        int last = 0;
        if (lane == 0) {
            if (!UPDATE) atomicMax(&G->speedBits, __float_as_uint(m));
            __threadfence();
            const unsigned prev = atomicAdd(&G->arrived, 1u);
            last = (prev == unsigned(UPDATE ? G->unitsUpd : G->units) - 1u);
            if (last) {
                __threadfence();
                if (UPDATE) {
                    G->arrived = 0u;
                    G->time = G->time + G->dt;
                    G->steps = G->steps + 1;
                    G->cur = cur ^ 1;
                    G->ghostsAhead = 1;
                } else {
                    const float s = __uint_as_float(atomicOr(&G->speedBits, 0u));
                    const BlockDesc &F = d.blocks[G->firstBlock];
                    G->speed = s;
                    G->dt = timestepFromSpeed(s, F.dx, F.dy, d.semantics);
                    if (!(s == s)) G->status |= 1;
                    G->speedBits = 0u;
                    G->arrived = 0u;
                }
                __threadfence();
            }
        }
        __syncwarp();
    }
}

} // namespace swegb

namespace swegb {

/// split-step speed pass on the warp mapping: x-edges (x-1|x), x = x0..x1, of
/// the strip's rows plus the ghost rows 0 and ny+1 at the block's bottom/top
/// (src/blocks/SWE_DimensionalSplitting.cpp:118-131); the last segment also
/// evaluates the LAST_EDGE reduction mode
template <int S, int R> __global__ void __launch_bounds__(128) speedSplitWarpKernel(const DomainDev d) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int segEnd = d.ctaSeg[gw + 1];
    for (int seg = d.ctaSeg[gw]; seg < segEnd; ++seg) {
        const WorkUnit wu = d.units[seg];
        const BlockDesc B = d.blocks[wu.block];
        GroupState *G = d.groups + B.group;
        if (!groupActive(G)) continue;
        const int cur = G->cur;
        const float *__restrict__ H = pick(d.h, cur) + B.base;
        const float *__restrict__ HU = pick(d.hu, cur) + B.base;
        const float *__restrict__ BT = d.b + B.base;
        const size_t P = size_t(B.pitch);
        const int yTop = min(wu.y0 + 32 * R - 1, B.ny);
        const int yl = wu.y0 + R * lane;
        float smax = 0.f;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int y = yl + r;
            if (y > yTop) continue;
            Cell prev, dummy;
            size_t o = size_t(wu.x0 - 1) * P + y;
            cellQuantities<S>(H[o], HU[o], 0.f, BT[o], prev, dummy);
            for (int x = wu.x0; x <= wu.x1; ++x) {
                o += P;
                Cell c;
                cellQuantities<S>(H[o], HU[o], 0.f, BT[o], c, dummy);
                smax = fmaxf(smax, edgeSpeed<S>(prev, c));
                prev = c;
            }
        }
        // ghost rows: lanes over columns
        for (int g = 0; g < 2; g++) {
            const bool has = g == 0 ? wu.y0 == 1 : yTop == B.ny;
            if (!has) continue;
            const int y = g == 0 ? 0 : B.ny + 1;
            for (int x = wu.x0 + lane; x <= wu.x1; x += 32) {
                Cell L, Rr, dummy;
                const size_t o = size_t(x) * P + y;
                cellQuantities<S>(H[o - P], HU[o - P], 0.f, BT[o - P], L, dummy);
                cellQuantities<S>(H[o], HU[o], 0.f, BT[o], Rr, dummy);
                smax = fmaxf(smax, edgeSpeed<S>(L, Rr));
            }
        }
        float m = smax;
        for (int o2 = 16; o2 > 0; o2 >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o2));
        if (lane == 0) {
            atomicMax(&G->speedBits, __float_as_uint(m));
            __threadfence();
            const unsigned prev = atomicAdd(&G->arrived, 1u);
            if (prev == unsigned(G->units) - 1u) {
                __threadfence();
                float s = __uint_as_float(atomicOr(&G->speedBits, 0u));
                const BlockDesc &F = d.blocks[G->firstBlock];
                if (d.splitDtMode == SPLIT_DT_LAST_EDGE) {
                    const float *Hc = pick(d.h, cur) + F.base, *HUc = pick(d.hu, cur) + F.base, *Bc = d.b + F.base;
                    const size_t o = size_t(F.nx) * size_t(F.pitch) + size_t(F.ny + 1);
                    const size_t o2 = o + size_t(F.pitch);
                    Cell L, Rr, dummy;
                    cellQuantities<S>(Hc[o], HUc[o], 0.f, Bc[o], L, dummy);
                    cellQuantities<S>(Hc[o2], HUc[o2], 0.f, Bc[o2], Rr, dummy);
                    s = fmaxf(0.f, edgeSpeed<S>(L, Rr));
                }
                G->speed = s;
                G->dt = timestepFromSpeed(s, F.dx, F.dy, SEM_SPLIT);
                if (!(s == s)) G->status |= 1;
                G->speedBits = 0u;
                G->arrived = 0u;
                __threadfence();
            }
        }
        __syncwarp();
    }
}

} // namespace swegb
