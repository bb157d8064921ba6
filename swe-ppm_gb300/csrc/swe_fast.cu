// Fast-arithmetic step of the f-wave / HLLE unsplit block step.
//
// The step of sweepKernel<S, SEM_UNSPLIT, true> -- the net updates of
// computeNumericalFluxes (src/blocks/SWE_DimensionalSplittingMpi.cpp:391-446)
// applied by updateUnknowns with the dry clamp (:484-518) -- computed with
// approximate reciprocal, reciprocal square root and square root and with
// contracted multiply-adds.  Results agree with the reference to FP32
// round-off, not bit for bit; this translation unit is compiled with
// -fmad=true and approximate division.
//
// One launch per time step:
//  - Column strips of h, hu, hv, b (a segment's rows plus a halo row on each
//    side) are staged into shared memory by bulk asynchronous copies
//    (cp.async.bulk) on a ring of kRing mbarrier slots, issued kRing columns
//    ahead of the sweep by one thread.
//  - Each thread owns R consecutive rows of a tile and marches along x.  The
//    x-edge (x-1|x) uses the previous column kept in registers, the y-edges
//    the thread's own rows and the staged row above them.  The right-going
//    part of a thread's top y-edge reaches the thread above through shared
//    memory; the tile's bottom y-edge of every column is solved up front.
//  - The next step's maximum wave speed (computeNumericalFluxes :391-456 on
//    Q^{n+1}) is evaluated while Q^{n+1} is produced: edges between two cells
//    of the segment as soon as both exist, edges to a ghost from the boundary
//    rule (outflow copy, wall mirror, kept ghost), and edges between cells of
//    two segments ("pieces") by the CTA of whichever of those segments
//    finishes last (an arrival counter per piece, no waiting).  The group's
//    last CTA turns the maximum into the next maxTimestep (:448-456), so a
//    step is this one kernel: no speed pass.
#include <cfloat>

#include "swe_fast.hpp"
#include "swe_launch.hpp"
#include "swe_sweep.cuh"

namespace swegb {
namespace fast {

constexpr int kRing = 6;                          // column strips in flight per CTA
constexpr int kHalo = 4;                          // staged rows below the tile (16-byte aligned start)
constexpr int kSlice = kMaxTileRows + 2 * kHalo;  // floats per field of one strip
constexpr int kSlotFloats = 4 * kSlice;           // h, hu, hv, b
constexpr unsigned kSpinLimit = 1u << 22;         // bound of every wait on a copy
constexpr size_t kRingBytes = sizeof(float) * kRing * kSlotFloats;

// ---------------------------------------------------------------------------
// approximate special functions (PTX .approx forms) and the copy ring
// ---------------------------------------------------------------------------
__device__ __forceinline__ float aRcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float aRsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float aSqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ unsigned smemAddr(const void *p) { return unsigned(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbarInit(unsigned a, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(unsigned a, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbarTryWait(unsigned a, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
/// bounded wait for the phase of parity `parity` of the mbarrier at `a`
__device__ __forceinline__ bool mbarWait(unsigned a, unsigned parity) {
    for (unsigned n = 0; n < kSpinLimit; ++n)
        if (mbarTryWait(a, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulkLoad(unsigned dst, const float *src, unsigned bytes, unsigned mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

// ---------------------------------------------------------------------------
// edges
// ---------------------------------------------------------------------------
/// A cell seen from one direction for the flux: h, normal momentum hn,
/// surface elevation eta = h + b, u = hn/h, sqrt(h), momentum flux m = hn u,
/// u - c and u + c.  The flux jump with the bathymetry source of the f-wave
/// and HLLE solvers, (phi_R - phi_L) + g/2 (h_L + h_R)(b_R - b_L) with
/// phi = hn u + g/2 h^2, equals (m_R - m_L) + g/2 (h_L + h_R)(eta_R - eta_L):
/// the same quantity without the difference of the two g/2 h^2 terms, whose
/// cancellation costs float32 digits in deep water.
struct FQ {
    float h, hn, eta, u, sq, m, lo, hi;
};

__device__ __forceinline__ FQ makeFQ(float h, float hn, float eta, float ih, float sq, float c) {
    FQ q;
    q.h = h;
    q.hn = hn;
    q.eta = eta;
    q.u = hn * ih;
    q.sq = sq;
    q.m = hn * q.u;
    q.lo = q.u - c;
    q.hi = q.u + c;
    return q;
}

/// the same from raw values (one reciprocal square root)
__device__ __forceinline__ FQ rawFQ(float h, float hn, float b) {
    const float r = aRsqrt(h);
    const float sq = h * r;
    return makeFQ(h, hn, h + b, r * r, sq, kSqrtG * sq);
}

__device__ __forceinline__ void routeFast(float s, float zh, float zhu, float &hL, float &hR, float &huL, float &huR) {
    if (s < -kZeroTol) {
        hL += zh;
        huL += zhu;
    } else if (s > kZeroTol) {
        hR += zh;
        huR += zhu;
    } else {
        const float a = 0.5f * zh, c = 0.5f * zhu;
        hL += a;
        huL += c;
        hR += a;
        huR += c;
    }
}

/// f-wave (Bale et al. 2002) or HLLE (Einfeldt 1988) waves of an edge whose
/// two sides are wet: Roe speeds (HLLE: with the Einfeldt bounds) and the
/// decomposition of the flux jump.  GENERAL: route each wave by its speed
/// (half to each side within zeroTol); otherwise the edge is taken as
/// subsonic (wave 1 left, wave 2 right) and `sub` receives min(-s1, s2),
/// which is above zeroTol exactly when it is.
template <int S, bool GENERAL>
__device__ __forceinline__ void waves(const FQ &L, const FQ &R, float &aL, float &aR, float &auL, float &auR,
                                      float &sub) {
    const float rs = aRcp(L.sq + R.sq);
    const float uRoe = fmaf(L.u, L.sq, R.u * R.sq) * rs;
    const float ghs = kHalfG * (L.h + R.h);
    const float cRoe = aSqrt(ghs);
    float s1 = uRoe - cRoe, s2 = uRoe + cRoe;
    if (S == SOLVER_HLLE) {
        s1 = fminf(L.lo, s1);
        s2 = fmaxf(R.hi, s2);
    }
    const float df1 = R.hn - L.hn;
    const float df2 = fmaf(ghs, R.eta - L.eta, R.m - L.m);
    const float rd = aRcp(s2 - s1);
    const float b1 = fmaf(s2, df1, -df2) * rd;
    const float b2 = fmaf(-s1, df1, df2) * rd;
    if (GENERAL) {
        aL = 0.f;
        aR = 0.f;
        auL = 0.f;
        auR = 0.f;
        routeFast(s1, b1, b1 * s1, aL, aR, auL, auR);
        routeFast(s2, b2, b2 * s2, aL, aR, auL, auR);
    } else {
        aL = b1;
        auL = b1 * s1;
        aR = b2;
        auR = b2 * s2;
        sub = fminf(sub, fminf(-s1, s2));
    }
}

__device__ __forceinline__ FQ mirrorFQ(const FQ &q) {
    FQ m = q;
    m.hn = -q.hn;
    m.u = -q.u;
    m.lo = -q.hi;
    m.hi = -q.lo;
    return m;
}

/// net updates of any edge (left h, right h, left hn, right hn): a dry side
/// becomes the wet side's mirror image (a wall) and takes no update, dry/dry
/// edges give nothing, waves are routed by their speeds
template <int S> __device__ __noinline__ float4 edgeGeneral(FQ L, FQ R) {
    const bool dL = L.h < kDryTol, dR = R.h < kDryTol;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (dL && dR) return o;
    if (dL) L = mirrorFQ(R);
    else if (dR) R = mirrorFQ(L);
    float sub = 0.f;
    waves<S, true>(L, R, o.x, o.y, o.z, o.w, sub);
    if (dL) {
        o.x = 0.f;
        o.z = 0.f;
    }
    if (dR) {
        o.y = 0.f;
        o.w = 0.f;
    }
    return o;
}

/// a new cell seen from one direction for its edges' wave speeds
struct SV {
    float h, u, sq, c;
};

__device__ __forceinline__ SV makeSV(float h, float hn, float r) {
    SV v;
    v.h = h;
    v.sq = h * r;
    v.u = hn * (r * r);
    v.c = kSqrtG * v.sq;
    return v;
}
__device__ __forceinline__ SV rawSV(float h, float hn) { return makeSV(h, hn, aRsqrt(h)); }

/// maximum wave speed of an edge with both sides wet, max(|s1|, |s2|) of the
/// solver's two waves: |uRoe| + cRoe for the f-wave solver, and for HLLE also
/// the Einfeldt bounds c_L - u_L and u_R + c_R
template <int S> __device__ __forceinline__ float wetSpeed(const SV &L, const SV &R) {
    const float rs = aRcp(L.sq + R.sq);
    const float uRoe = fmaf(L.u, L.sq, R.u * R.sq) * rs;
    const float cRoe = aSqrt(kHalfG * (L.h + R.h));
    float s = fabsf(uRoe) + cRoe;
    if (S == SOLVER_HLLE) s = fmaxf(s, fmaxf(L.c - L.u, R.u + R.c));
    return s;
}

/// the same for any edge: a dry side becomes the wet side's mirror image
template <int S> __device__ __noinline__ float speedGeneral(SV L, SV R) {
    const bool dL = L.h < kDryTol, dR = R.h < kDryTol;
    if (dL && dR) return 0.f;
    if (dL) {
        L = R;
        L.u = -R.u;
    } else if (dR) {
        R = L;
        R.u = -L.u;
    }
    return wetSpeed<S>(L, R);
}

/// maxTimestep from the maximum wave speed, IEEE operations as
/// src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456
__device__ __forceinline__ float dtFromSpeed(float s, float dx, float dy) {
    if (double(s) > 0.00001) {
        const float a = __fdiv_rn(dx, s), b = __fdiv_rn(dy, s);
        const float dt = (b < a) ? b : a;
        return __fmul_rn(dt, 0.4f);
    }
    return FLT_MAX;
}

/// A cell (x, y) of Q^{n+1} on its block's rim: pushes it into every ghost
/// the next setGhostLayer fills from it -- the boundary rule of
/// src/blocks/SWE_Block.hh:757-911 (outflow copy, wall with the normal
/// momentum negated, the other types keep the ghost's value), the
/// neighbour block's ghost for CONNECT_WITHIN_RANK (the on-device form of
/// src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304), and the
/// corners from the diagonal cell -- and returns the next state's wave speed
/// of its edges to ghosts of its own block: all of them for the f-wave
/// solver, the kept ones for HLLE (an outflow or wall ghost's edge is covered
/// by the cell's own speed bound).  Output / input pointers are the whole
/// field (block bases added here).
template <int S>
__device__ __noinline__ float rimCell(float *HO, float *HUO, float *HVO, const float *H, const float *HU,
                                      const float *HV, const BlockDesc *blocks, int blk, int x, int y, float h, float hu,
                                      float hv) {
    const BlockDesc &B = blocks[blk];
    const size_t P = size_t(B.pitch);
    const long long base = B.base;
    const float r = aRsqrt(h);
    const SV vx = makeSV(h, hu, r), vy = makeSV(h, hv, r);
    float s = 0.f;
    for (int side = 0; side < 4; side++) {
        const bool on = side == 0 ? x == 1 : side == 1 ? x == B.nx : side == 2 ? y == 1 : y == B.ny;
        if (!on) continue;
        const int type = B.bnd[side];
        const int gx = side == 0 ? 0 : side == 1 ? B.nx + 1 : x;
        const int gy = side == 2 ? 0 : side == 3 ? B.ny + 1 : y;
        const size_t g = size_t(base + gx * (long long)P + gy);
        if (type == CONNECT_WITHIN_RANK) {
            const BlockDesc &N = blocks[B.nbr[side]];
            const int nxg = side == 0 ? N.nx + 1 : side == 1 ? 0 : x;
            const int nyg = side == 2 ? N.ny + 1 : side == 3 ? 0 : y;
            const size_t gn = size_t(N.base + nxg * (long long)N.pitch + nyg);
            HO[gn] = h;
            HUO[gn] = hu;
            HVO[gn] = hv;
            continue;
        }
        float gh, ghu, ghv;
        if (type == OUTFLOW) {
            gh = h; ghu = hu; ghv = hv;
        } else if (type == WALL) {
            gh = h;
            ghu = side < 2 ? -hu : hu;
            ghv = side < 2 ? hv : -hv;
        } else {
            gh = H[g]; ghu = HU[g]; ghv = HV[g];
        }
        HO[g] = gh;
        HUO[g] = ghu;
        HVO[g] = ghv;
        if (S == SOLVER_FWAVE || (type != OUTFLOW && type != WALL)) {
            const SV gv = rawSV(gh, side < 2 ? ghu : ghv);
            const SV &cv = side < 2 ? vx : vy;
            s = fmaxf(s, (side == 0 || side == 2) ? speedGeneral<S>(gv, cv) : speedGeneral<S>(cv, gv));
        }
    }
    for (int cxi = 0; cxi < 2; cxi++)
        for (int cyi = 0; cyi < 2; cyi++) {
            if ((cxi ? B.nx : 1) != x || (cyi ? B.ny : 1) != y) continue;
            const size_t g = size_t(base + (cxi ? B.nx + 1 : 0) * (long long)P + (cyi ? B.ny + 1 : 0));
            HO[g] = h;
            HUO[g] = hu;
            HVO[g] = hv;
        }
    return s;
}

// ---------------------------------------------------------------------------
// the step kernel
// ---------------------------------------------------------------------------
/// HLLE: the next state's maximum wave speed is the largest cell speed
/// c + max(|u|, |v|) over its wet cells -- exactly, in exact arithmetic: every
/// edge speed is at most the larger cell speed of its two cells (|uRoe| is a
/// sqrt(h)-weighted mean of |u|, cRoe at most the same mean of c, and the
/// Einfeldt bounds are the cells' own u -/+ c), and every wet cell's u + c
/// and c - u are the Einfeldt bounds of its left and right edges (v likewise
/// in y; a dry neighbour's mirror image gives the same).  Only edges to
/// ghosts that keep their own values need their speed evaluated.  The f-wave
/// solver has no such identity: its edges are evaluated one by one, those
/// between two segments as pieces.
template <int S, int R, int MINB>
__global__ void __launch_bounds__(kMaxTileRows / R, MINB) fastStepKernel(const FastDev f) {
    constexpr int NT = kMaxTileRows / R;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr bool EDGES = S == SOLVER_FWAVE;  // next-state speeds edge by edge
    extern __shared__ __align__(128) float ring[];  // kRing strips of kSlotFloats
    __shared__ __align__(8) unsigned long long mbar[kRing];
    __shared__ int slotDone[kRing];  // warps done with the strip in a slot
    __shared__ float sRed[NT / 32];
    __shared__ int sLast, sNWon, sAbort;
    __shared__ int sWon[kMaxArrivals];

    const int t = threadIdx.x, lane = t & 31, nth = blockDim.x, nw = nth >> 5, TY = nth * R;
    // strips start as a state at rest (rows a partial tile never loads stay finite)
    for (int i = t; i < kRing * kSlotFloats; i += nth) ring[i] = ((i % kSlotFloats) < kSlice) ? 1.f : 0.f;
    if (t == 0) {
        for (int s = 0; s < kRing; s++) {
            mbarInit(smemAddr(&mbar[s]), 1u);
            slotDone[s] = 0;
        }
        sAbort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned phases = 0u;  // bit s: parity of slot s's next phase
    pdlWaitAndRelease();

    const unsigned ringAddr = smemAddr(ring);
    const int segEnd = f.ctaSeg[blockIdx.x + 1];
    for (int seg = f.ctaSeg[blockIdx.x]; seg < segEnd; ++seg) {
        const Unit wu = f.units[seg];
        const BlockDesc &B = f.d.blocks[wu.block];
        GroupState *G = f.d.groups + __ldg(&B.group);
        if (!groupActive(G)) continue;
        const int cur = __ldg(&G->cur);
        const unsigned P = unsigned(__ldg(&B.pitch));
        const long long base = __ldg(&B.base);
        const int nx = __ldg(&B.nx), ny = __ldg(&B.ny);
        const int x0 = wu.x0, x1 = wu.x1, XC = x1 - x0, ncol = XC + 2;  // columns x0-1 .. x1
        const int y0 = wu.y0, yTop = min(y0 + TY - 1, ny);
        const int rowStart = y0 - kHalo;
        const unsigned bytes = unsigned(((yTop + 2 - rowStart) + 3) & ~3) * 4u;
        float dtdx, dtdy;
        {
            const float dt = __ldg(&G->dt);
            dtdx = __fdiv_rn(dt, __ldg(&B.dx));
            dtdy = __fdiv_rn(dt, __ldg(&B.dy));
        }
        const float *__restrict__ Hin = pick(f.d.h, cur);
        const float *__restrict__ HUin = pick(f.d.hu, cur);
        const float *__restrict__ HVin = pick(f.d.hv, cur);
        float *__restrict__ HO = pick(f.d.h, cur ^ 1) + base;
        float *__restrict__ HUO = pick(f.d.hu, cur ^ 1) + base;
        float *__restrict__ HVO = pick(f.d.hv, cur ^ 1) + base;
        // the strip of column x0-1+k (rows rowStart ..) into slot k % kRing
        auto refill = [&](int k, int slot) {
            const unsigned mb = smemAddr(&mbar[slot]);
            mbarExpectTx(mb, 4u * bytes);
            const size_t col = size_t(base) + size_t(x0 - 1 + k) * P + size_t(rowStart);
            const unsigned dst = ringAddr + unsigned(slot * kSlotFloats) * 4u;
            bulkLoad(dst, Hin + col, bytes, mb);
            bulkLoad(dst + unsigned(kSlice) * 4u, HUin + col, bytes, mb);
            bulkLoad(dst + unsigned(2 * kSlice) * 4u, HVin + col, bytes, mb);
            bulkLoad(dst + unsigned(3 * kSlice) * 4u, f.d.b + col, bytes, mb);
        };

        __syncthreads();  // the previous segment is done with every slot and shared value
        if (t == 0) {
            sNWon = 0;
            for (int k = 0; k < min(kRing, ncol); k++) refill(k, k);
        }

        const int yA = y0 + R * t;                       // this thread's first row
        const int nAct = max(0, min(R, yTop - yA + 1));  // its rows inside the tile
        const bool fullTile = yTop - y0 + 1 == TY;       // every thread has R rows (CTA-uniform)
        const bool upIn = yA + R <= yTop;                // the next thread's first row is in the tile
        // rows on the block's rim (y == 1, y == ny): ghost below / above.
        // rimMode per row: 0 none, 1 copy, 2 copy with -hv, 3 kept ghost (its
        // edge speed is evaluated), 4 every ghost edge evaluated (f-wave)
        int rimMode[R];
        long long rimGhost[R];
        int rimPitch[R];
        bool rimAny = false;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int y = yA + r;
            rimMode[r] = 0;
            rimGhost[r] = 0;
            rimPitch[r] = 0;
            if (r < nAct && (y == 1 || y == ny)) {
                rimAny = true;
                const int side = (y == 1) ? 2 : 3;
                const int type = __ldg(&B.bnd[side]);
                rimGhost[r] = (side == 2) ? 0 : ny + 1;
                rimPitch[r] = int(P);
                if (ny == 1 || EDGES) {
                    rimMode[r] = 4;
                } else if (type == OUTFLOW || type == WALL) {
                    rimMode[r] = type == WALL ? 2 : 1;
                } else if (type == CONNECT_WITHIN_RANK) {
                    const BlockDesc &N = f.d.blocks[__ldg(&B.nbr[side])];
                    rimMode[r] = 1;
                    rimGhost[r] = __ldg(&N.base) - base + ((side == 2) ? __ldg(&N.ny) + 1 : 0);
                    rimPitch[r] = __ldg(&N.pitch);
                } else {
                    rimMode[r] = 3;
                }
            }
        }
        const bool rimWarp = __any_sync(FULL, rimAny);

        FQ prevX[R];
        float pendH[R], pendHU[R], oldHV[R], syH[R], syHV[R];
        SV nprev[R];
        float smax = 0.f;
        bool bad = false;
#pragma unroll
        for (int r = 0; r < R; r++) {
            pendH[r] = pendHU[r] = oldHV[r] = syH[r] = syHV[r] = 0.f;
            nprev[r] = SV{1.f, 0.f, 1.f, 0.f};
        }
        const int i0 = kHalo + R * t;  // strip index of this thread's first row
        int slot = 0;
        for (int k = 0; k < ncol; ++k) {
            // wait for the strip of column x = x0-1+k (bounded; a stalled copy
            // aborts the CTA, see below)
            {
                const unsigned a = smemAddr(&mbar[slot]), par = (phases >> slot) & 1u;
                bool ok = mbarTryWait(a, par);
                for (unsigned n = 0; !ok && n < kSpinLimit; ++n) {
                    if (*(volatile int *)&sAbort) break;
                    ok = mbarTryWait(a, par);
                }
                if (__any_sync(FULL, !ok)) {
                    if (lane == 0) *(volatile int *)&sAbort = 1;
                    break;
                }
                phases ^= 1u << slot;
            }
            const float *sl = ring + slot * kSlotFloats;
            // A. this thread's cells of column x
            float ch[R], chu[R], chv[R], cb[R];
            if (R == 4) {
                const float4 a = *reinterpret_cast<const float4 *>(sl + i0);
                const float4 bq = *reinterpret_cast<const float4 *>(sl + kSlice + i0);
                const float4 c = *reinterpret_cast<const float4 *>(sl + 2 * kSlice + i0);
                const float4 e = *reinterpret_cast<const float4 *>(sl + 3 * kSlice + i0);
                const float va[4] = {a.x, a.y, a.z, a.w}, vb[4] = {bq.x, bq.y, bq.z, bq.w};
                const float vc[4] = {c.x, c.y, c.z, c.w}, ve[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
                for (int r = 0; r < R; r++) {
                    ch[r] = va[r % 4]; chu[r] = vb[r % 4]; chv[r] = vc[r % 4]; cb[r] = ve[r % 4];
                }
            } else if (R == 2) {
                const float2 a = *reinterpret_cast<const float2 *>(sl + i0);
                const float2 bq = *reinterpret_cast<const float2 *>(sl + kSlice + i0);
                const float2 c = *reinterpret_cast<const float2 *>(sl + 2 * kSlice + i0);
                const float2 e = *reinterpret_cast<const float2 *>(sl + 3 * kSlice + i0);
                ch[0] = a.x; ch[R - 1] = a.y;
                chu[0] = bq.x; chu[R - 1] = bq.y;
                chv[0] = c.x; chv[R - 1] = c.y;
                cb[0] = e.x; cb[R - 1] = e.y;
            } else {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    ch[r] = sl[i0 + r];
                    chu[r] = sl[kSlice + i0 + r];
                    chv[r] = sl[2 * kSlice + i0 + r];
                    cb[r] = sl[3 * kSlice + i0 + r];
                }
            }
            FQ cx[R], cy[R];
            float minh = 3.0e38f;  // smallest depth the column's edges touch
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float rr = aRsqrt(ch[r]);
                const float sq = ch[r] * rr, ih = rr * rr, c = kSqrtG * sq, eta = ch[r] + cb[r];
                cx[r] = makeFQ(ch[r], chu[r], eta, ih, sq, c);
                cy[r] = makeFQ(ch[r], chv[r], eta, ih, sq, c);
                minh = fminf(minh, ch[r]);
            }
            const bool xcol = k >= 1, ycol = k >= 1 && k <= XC;
            // B. x-edges (x-1 | x); y-edges of column x: between this thread's
            // rows and the top one with the staged row above; lane 0 also the
            // one below its first row (its right-going part comes from no
            // other lane).  All taken as wet and subsonic first.
            float aLx[R], aRx[R], auLx[R], auRx[R], bLh[R], bLhv[R], bRh[R], bRhv[R], tRh = 0.f, tRhv = 0.f;
            float lowRh = 0.f, lowRhv = 0.f;
            float sub = 3.0e38f;
            FQ up, low;
            if (xcol) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    waves<S, false>(prevX[r], cx[r], aLx[r], aRx[r], auLx[r], auRx[r], sub);
                    minh = fminf(minh, prevX[r].h);
                }
            }
            if (ycol) {
                const int iu = i0 + R;
                up = rawFQ(sl[iu], sl[2 * kSlice + iu], sl[3 * kSlice + iu]);
#pragma unroll
                for (int r = 0; r + 1 < R; r++)
                    waves<S, false>(cy[r], cy[(r + 1) % R], bLh[r], bRh[(r + 1) % R], bLhv[r], bRhv[(r + 1) % R], sub);
                waves<S, false>(cy[R - 1], up, bLh[R - 1], tRh, bLhv[R - 1], tRhv, sub);
                minh = fminf(minh, up.h);
                if (lane == 0) {
                    low = rawFQ(sl[i0 - 1], sl[2 * kSlice + i0 - 1], sl[3 * kSlice + i0 - 1]);
                    float dl, dlv;
                    waves<S, false>(low, cy[0], dl, lowRh, dlv, lowRhv, sub);
                    minh = fminf(minh, low.h);
                }
            }
            // the strip is read: the warp that finishes it last refills the slot
            __syncwarp();
            if (lane == 0) {
                if (atomicAdd(&slotDone[slot], 1) == nw - 1) {
                    slotDone[slot] = 0;
                    if (k + kRing < ncol) refill(k + kRing, slot);
                }
            }
            slot = (slot + 1 == kRing) ? 0 : slot + 1;
            // C. a lane with a dry cell or an edge that is not subsonic solves
            // its edges again in full (rare: shorelines, fronts)
            const bool redo = xcol && (minh < kDryTol || !(sub > kZeroTol));
            if (__any_sync(FULL, redo)) {
                if (redo) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const float4 e = edgeGeneral<S>(prevX[r], cx[r]);
                        aLx[r] = e.x; aRx[r] = e.y; auLx[r] = e.z; auRx[r] = e.w;
                    }
                    if (ycol) {
#pragma unroll
                        for (int r = 0; r + 1 < R; r++) {
                            const float4 e = edgeGeneral<S>(cy[r], cy[(r + 1) % R]);
                            bLh[r] = e.x; bRh[(r + 1) % R] = e.y; bLhv[r] = e.z; bRhv[(r + 1) % R] = e.w;
                        }
                        const float4 e = edgeGeneral<S>(cy[R - 1], up);
                        bLh[R - 1] = e.x; tRh = e.y; bLhv[R - 1] = e.z; tRhv = e.w;
                        if (lane == 0) {
                            const float4 e0 = edgeGeneral<S>(low, cy[0]);
                            lowRh = e0.y;
                            lowRhv = e0.w;
                        }
                    }
                }
            }
            // D. cells (x-1, y): Q^{n+1} with the dry clamp, and their part
            // of the next maxTimestep
            if (k >= 2) {
                const int xc = x0 - 2 + k;
                float hn[R], hun[R], hvn[R];
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const float sxH = pendH[r] + aLx[r], sxHU = pendHU[r] + auLx[r];
                    float h_ = prevX[r].h - (dtdx * sxH + dtdy * syH[r]);
                    float hu_ = prevX[r].hn - dtdx * sxHU;
                    float hv_ = oldHV[r] - dtdy * syHV[r];
                    hu_ = (h_ < 0.1f) ? 0.f : hu_;
                    hv_ = (h_ < 0.1f) ? 0.f : hv_;
                    h_ = (h_ < 0.f) ? 0.f : h_;
                    hn[r] = h_;
                    hun[r] = hu_;
                    hvn[r] = hv_;
                    bad |= (r < nAct) && !(fabsf(h_) <= FLT_MAX);
                }
                const unsigned o = unsigned(xc) * P + unsigned(yA);
                if (R == 4 && fullTile) {
                    *reinterpret_cast<float4 *>(HO + o) = make_float4(hn[0], hn[1 % R], hn[2 % R], hn[3 % R]);
                    *reinterpret_cast<float4 *>(HUO + o) = make_float4(hun[0], hun[1 % R], hun[2 % R], hun[3 % R]);
                    *reinterpret_cast<float4 *>(HVO + o) = make_float4(hvn[0], hvn[1 % R], hvn[2 % R], hvn[3 % R]);
                } else if (R == 2 && fullTile) {
                    *reinterpret_cast<float2 *>(HO + o) = make_float2(hn[0], hn[R - 1]);
                    *reinterpret_cast<float2 *>(HUO + o) = make_float2(hun[0], hun[R - 1]);
                    *reinterpret_cast<float2 *>(HVO + o) = make_float2(hvn[0], hvn[R - 1]);
                } else {
#pragma unroll
                    for (int r = 0; r < R; r++)
                        if (r < nAct) {
                            HO[o + r] = hn[r];
                            HUO[o + r] = hun[r];
                            HVO[o + r] = hvn[r];
                        }
                }
                if (!EDGES) {
                    // HLLE: the wet new cells' speeds c + max(|u|, |v|)
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const float rn = aRsqrt(hn[r]);
                        const float w = fmaf(fmaxf(fabsf(hun[r]), fabsf(hvn[r])), rn * rn, kSqrtG * (hn[r] * rn));
                        smax = fmaxf(smax, (r < nAct && hn[r] >= kDryTol) ? w : 0.f);
                    }
                } else {
                    // f-wave: x-edge (x-2 | x-1), the y-edges between this
                    // thread's rows and the one to the next lane's first row
                    // (the last lane's goes to the pass after the sweep)
                    SV nxv[R], nyv[R];
                    float nminh = 3.0e38f;
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const float rn = aRsqrt(hn[r]);
                        nxv[r] = makeSV(hn[r], hun[r], rn);
                        nyv[r] = makeSV(hn[r], hvn[r], rn);
                        nminh = fminf(nminh, fminf(hn[r], nprev[r].h));
                    }
                    SV nu;
                    nu.h = __shfl_down_sync(FULL, nyv[0].h, 1);
                    nu.u = __shfl_down_sync(FULL, nyv[0].u, 1);
                    nu.sq = __shfl_down_sync(FULL, nyv[0].sq, 1);
                    nu.c = kSqrtG * nu.sq;
                    const bool nuIn = upIn && lane < 31;
                    nminh = fminf(nminh, nuIn ? nu.h : 1.f);
                    float sp[2 * R + 1];
#pragma unroll
                    for (int r = 0; r < R; r++) sp[r] = wetSpeed<S>(nprev[r], nxv[r]);
#pragma unroll
                    for (int r = 0; r + 1 < R; r++) sp[R + r] = wetSpeed<S>(nyv[r], nyv[(r + 1) % R]);
                    sp[2 * R] = wetSpeed<S>(nyv[R - 1], nu);
                    const bool nredo = nminh < kDryTol;
                    if (__any_sync(FULL, nredo)) {
                        if (nredo) {
#pragma unroll
                            for (int r = 0; r < R; r++) sp[r] = speedGeneral<S>(nprev[r], nxv[r]);
#pragma unroll
                            for (int r = 0; r + 1 < R; r++) sp[R + r] = speedGeneral<S>(nyv[r], nyv[(r + 1) % R]);
                            sp[2 * R] = speedGeneral<S>(nyv[R - 1], nu);
                        }
                    }
#pragma unroll
                    for (int r = 0; r < R; r++) smax = fmaxf(smax, (r < nAct && k >= 3) ? sp[r] : 0.f);
#pragma unroll
                    for (int r = 0; r + 1 < R; r++) smax = fmaxf(smax, (r + 1 < nAct) ? sp[R + r] : 0.f);
                    smax = fmaxf(smax, nuIn ? sp[2 * R] : 0.f);
#pragma unroll
                    for (int r = 0; r < R; r++) nprev[r] = nxv[r];
                }
                // the block's rim: ghost pushes, edges to the block's own ghosts
                if (xc == 1 || xc == nx) {
#pragma unroll
                    for (int r = 0; r < R; r++)
                        if (r < nAct)
                            smax = fmaxf(smax, rimCell<S>(pick(f.d.h, cur ^ 1), pick(f.d.hu, cur ^ 1), pick(f.d.hv, cur ^ 1),
                                                          Hin, HUin, HVin, f.d.blocks, wu.block, xc, yA + r, hn[r],
                                                          hun[r], hvn[r]));
                } else if (rimWarp) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        if (rimMode[r] == 0) continue;
                        if (rimMode[r] >= 3) {
                            smax = fmaxf(smax, rimCell<S>(pick(f.d.h, cur ^ 1), pick(f.d.hu, cur ^ 1), pick(f.d.hv, cur ^ 1),
                                                          Hin, HUin, HVin, f.d.blocks, wu.block, xc, yA + r, hn[r],
                                                          hun[r], hvn[r]));
                        } else {
                            const long long g = rimGhost[r] + (long long)xc * rimPitch[r];
                            HO[g] = hn[r];
                            HUO[g] = hun[r];
                            HVO[g] = rimMode[r] == 2 ? -hvn[r] : hvn[r];
                        }
                    }
                }
            }
            if (ycol) {
                // y-sums of column x: right-going part of the edge below the
                // first row from the lane below (lane 0: its own), left-going
                // parts from this lane's edges
                const float pH = __shfl_up_sync(FULL, tRh, 1), pHV = __shfl_up_sync(FULL, tRhv, 1);
                bRh[0] = (lane == 0) ? lowRh : pH;
                bRhv[0] = (lane == 0) ? lowRhv : pHV;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    syH[r] = bRh[r] + bLh[r];
                    syHV[r] = bRhv[r] + bLhv[r];
                    oldHV[r] = chv[r];
                }
            }
            if (xcol) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    pendH[r] = aRx[r];
                    pendHU[r] = auRx[r];
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) prevX[r] = cx[r];
        }
        __syncthreads();  // every warp's sweep is done: its stores are visible to the CTA
        if (sAbort) {
            // a copy did not arrive in time: wait (bounded) for the copies in
            // flight, flag the group and leave the kernel
            if (t == 0) {
                for (int s = 0; s < kRing; s++) mbarWait(smemAddr(&mbar[s]), (phases >> s) & 1u);
                atomicOr(&G->status, 4);
            }
            return;
        }
        if (__syncthreads_or(bad) && t == 0) atomicOr(&G->status, 2);

        if (EDGES) {
            // f-wave: the next state's y-edges between the warps' strips of rows
            const float *Ho = HO, *Vo = HVO;
            for (int i = t; i < (nw - 1) * XC; i += nth) {
                const int w = i / XC + 1, x = x0 + i % XC;
                const int y = y0 + w * 32 * R;  // first row of warp w
                if (y > yTop) continue;
                const unsigned ob = unsigned(x) * P + unsigned(y), oa = ob - 1u;
                const SV a = rawSV(__ldcg(Ho + oa), __ldcg(Vo + oa));
                const SV bq = rawSV(__ldcg(Ho + ob), __ldcg(Vo + ob));
                smax = fmaxf(smax, speedGeneral<S>(a, bq));
            }
            // pieces: arrive on every piece this segment's cells belong to; the
            // last arrival evaluates the piece's edges from the written state
            __threadfence();
            __syncthreads();
            const int narr = wu.arrEnd - wu.arrBegin;
            if (t < narr) {
                const int p = f.arr[wu.arrBegin + t];
                const unsigned old = arriveAcqRel(&f.pieceCnt[p], 1u);
                if (old + 1u == unsigned(f.pieces[p].need)) {
                    __threadfence();
                    sWon[atomicAdd(&sNWon, 1)] = p;
                }
            }
            __syncthreads();
            const int nwon = sNWon;
            for (int i = 0; i < nwon; i++) {
                const int p = sWon[i];
                const Piece pc = f.pieces[p];
                const BlockDesc &PB = f.d.blocks[pc.block];
                const float *Hp = pick(f.d.h, cur ^ 1) + PB.base;
                const float *Np = (pc.dir ? pick(f.d.hv, cur ^ 1) : pick(f.d.hu, cur ^ 1)) + PB.base;
                const unsigned PP = unsigned(PB.pitch);
                for (int j = t; j < pc.len; j += nth) {
                    unsigned ob, oa;
                    if (pc.dir == 0) {
                        ob = unsigned(pc.x0) * PP + unsigned(pc.y0 + j);
                        oa = ob - PP;
                    } else {
                        ob = unsigned(pc.x0 + j) * PP + unsigned(pc.y0);
                        oa = ob - 1u;
                    }
                    const SV a = rawSV(__ldcg(Hp + oa), __ldcg(Np + oa));
                    const SV bq = rawSV(__ldcg(Hp + ob), __ldcg(Np + ob));
                    smax = fmaxf(smax, speedGeneral<S>(a, bq));
                }
                if (t == 0) f.pieceCnt[p] = 0u;
            }
        }

        // the group: maximum speed and arrival; the last CTA finishes the step
        const float m = blockReduceMax(smax, sRed);
        __syncthreads();
        if (t == 0) {
            atomicMax(&G->speedBits, __float_as_uint(m));
            const unsigned prev = arriveAcqRel(&G->arrived, 1u);
            sLast = prev + 1u == unsigned(G->unitsFast);
        }
        __syncthreads();
        if (sLast && t == 0) {
            const float s = __uint_as_float(__ldcg(&G->speedBits));
            const BlockDesc &F = f.d.blocks[G->firstBlock];
            G->arrived = 0u;
            G->speedBits = 0u;
            G->time = G->time + G->dt;
            G->steps = G->steps + 1;
            G->cur = cur ^ 1;
            G->ghostsAhead = 1;
            G->boundsValid[0] = 0;
            G->boundsValid[1] = 0;
            G->speed = s;
            G->dt = dtFromSpeed(s, F.dx, F.dy);
            if (!(s == s)) G->status |= 1;
        }
    }
}

/// rows per thread of the step kernel and its resident CTAs per SM (two
/// rows: the second row's edges give each thread two independent chains;
/// four CTAs of 128 threads keep the loop free of spills)
constexpr int kRows = 2;
constexpr int kMinCtas = 4;

int fastRows() { return kRows; }

cudaError_t launchFastStep(const FastDev &f, int solver, int grid, int tileRows, cudaStream_t s) {
    const int threads = tileRows / kRows;
    const cudaError_t e =
        solver == SOLVER_FWAVE
            ? launchPdlSmem(fastStepKernel<SOLVER_FWAVE, kRows, kMinCtas>, dim3(grid), dim3(threads), kRingBytes, s, f)
            : launchPdlSmem(fastStepKernel<SOLVER_HLLE, kRows, kMinCtas>, dim3(grid), dim3(threads), kRingBytes, s, f);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int fastOccupancy(int solver, int tileRows) {
    int a = 0;
    const int threads = tileRows / kRows;
    if (solver == SOLVER_FWAVE)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fastStepKernel<SOLVER_FWAVE, kRows, kMinCtas>, threads,
                                                      kRingBytes);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fastStepKernel<SOLVER_HLLE, kRows, kMinCtas>, threads,
                                                      kRingBytes);
    return a;
}

} // namespace fast
} // namespace swegb
