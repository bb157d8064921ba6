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
//    (cp.async.bulk) on a ring of kRing mbarrier slots.  The warp that
//    releases a slot last issues the copy of the column kRing ahead.
//  - Each thread owns two consecutive rows of a tile, computed as packed
//    pairs (f32x2 add / mul / fma), and marches along x.  The x-edge (x-1|x)
//    uses the previous column kept in registers, the y-edges the thread's
//    own rows and the staged row above them.  The right-going part of a
//    thread's top y-edge reaches the thread above by a shuffle; lane 0
//    solves the warp's bottom y-edge itself.
//  - The next step's maximum wave speed (computeNumericalFluxes :391-456 on
//    Q^{n+1}) is evaluated while Q^{n+1} is produced: edges between two cells
//    of the segment as soon as both exist, edges to a ghost from the boundary
//    rule (outflow copy, wall mirror, kept ghost), and edges between cells of
//    two segments ("pieces") by the CTA of whichever of those segments
//    finishes last (an arrival counter per piece, no waiting).  The group's
//    last CTA turns the maximum into the next maxTimestep (:448-456), so a
//    step is this one kernel: no speed pass.
#include <cfloat>
#include <type_traits>

#include "swe_fast.hpp"
#include "swe_launch.hpp"
#include "swe_sweep.cuh"

namespace swegb {
namespace fast {

constexpr int kRing = 4;                          // column strips in flight per CTA (4 ran faster than 5, 6, 8)
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
// packed pairs: a thread's two rows, one f32x2 instruction per operation
// ---------------------------------------------------------------------------
#define SWE_F2_OP2(name, op)                                                                            \
    __device__ __forceinline__ float2 name(float2 a, float2 b) {                                        \
        float2 d;                                                                                       \
        asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t" op            \
            " d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"                                                    \
            : "=f"(d.x), "=f"(d.y)                                                                      \
            : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                                  \
        return d;                                                                                       \
    }
SWE_F2_OP2(add2, "add.rn.ftz.f32x2")
SWE_F2_OP2(sub2, "sub.rn.ftz.f32x2")
SWE_F2_OP2(mul2, "mul.rn.ftz.f32x2")
#undef SWE_F2_OP2
/// a * b + c, one rounding per lane
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 a, b, c, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tmov.b64 c, {%6, %7};\n\t"
        "fma.rn.ftz.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float2 pk(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 rsqrt2(float2 a) { return make_float2(aRsqrt(a.x), aRsqrt(a.y)); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(aRcp(a.x), aRcp(a.y)); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(aSqrt(a.x), aSqrt(a.y)); }

/// FQ of two cells, one per lane of the pair
struct FQ2 {
    float2 h, hn, eta, u, sq, m, lo, hi;
};
__device__ __forceinline__ FQ2 makeFQ2(float2 h, float2 hn, float2 eta, float2 ih, float2 sq, float2 c) {
    FQ2 q;
    q.h = h;
    q.hn = hn;
    q.eta = eta;
    q.u = mul2(hn, ih);
    q.sq = sq;
    q.m = mul2(hn, q.u);
    q.lo = sub2(q.u, c);
    q.hi = add2(q.u, c);
    return q;
}
__device__ __forceinline__ FQ laneX(const FQ2 &q) { return FQ{q.h.x, q.hn.x, q.eta.x, q.u.x, q.sq.x, q.m.x, q.lo.x, q.hi.x}; }
__device__ __forceinline__ FQ laneY(const FQ2 &q) { return FQ{q.h.y, q.hn.y, q.eta.y, q.u.y, q.sq.y, q.m.y, q.lo.y, q.hi.y}; }
/// the pair (a, b) of two single cells
__device__ __forceinline__ FQ2 pairFQ(const FQ &a, const FQ &b) {
    FQ2 q;
    q.h = make_float2(a.h, b.h);
    q.hn = make_float2(a.hn, b.hn);
    q.eta = make_float2(a.eta, b.eta);
    q.u = make_float2(a.u, b.u);
    q.sq = make_float2(a.sq, b.sq);
    q.m = make_float2(a.m, b.m);
    q.lo = make_float2(a.lo, b.lo);
    q.hi = make_float2(a.hi, b.hi);
    return q;
}

/// waves<S, false> of two edges at once, rounding as the single-edge form:
/// the flux jump enters negated (-df2) so that both wave strengths are one
/// fused multiply-add each, (s2 df1 - df2) / (s2 - s1) and
/// (s1 df1 - df2) / (s1 - s2)
template <int S>
__device__ __forceinline__ void waves2(const FQ2 &L, const FQ2 &R, float2 &aL, float2 &aR, float2 &auL, float2 &auR,
                                       float &sub) {
    const float2 rs = rcp2(add2(L.sq, R.sq));
    const float2 uRoe = mul2(fma2(L.u, L.sq, mul2(R.u, R.sq)), rs);
    const float2 ghs = mul2(pk(kHalfG), add2(L.h, R.h));
    const float2 cRoe = sqrt2(ghs);
    float2 s1 = sub2(uRoe, cRoe), s2 = add2(uRoe, cRoe);
    if (S == SOLVER_HLLE) {
        s1 = make_float2(fminf(L.lo.x, s1.x), fminf(L.lo.y, s1.y));
        s2 = make_float2(fmaxf(R.hi.x, s2.x), fmaxf(R.hi.y, s2.y));
    }
    const float2 df1 = sub2(R.hn, L.hn);
    const float2 ndf2 = fma2(ghs, sub2(L.eta, R.eta), sub2(L.m, R.m));  // -(flux jump)
    const float2 rd = rcp2(sub2(s2, s1));
    const float2 nrd = mul2(rd, pk(-1.f));
    aL = mul2(fma2(s2, df1, ndf2), rd);
    aR = mul2(fma2(s1, df1, ndf2), nrd);
    auL = mul2(aL, s1);
    auR = mul2(aR, s2);
    sub = fminf(sub, fminf(fminf(-s1.x, -s1.y), fminf(s2.x, s2.y)));
}

// ---------------------------------------------------------------------------
// the step kernel
// ---------------------------------------------------------------------------
/// Loads of a thread's R = 2 NP consecutive rows of one strip field as NP pairs.
template <int NP> __device__ __forceinline__ void loadRows(const float *p, float2 (&v)[NP]) {
    if constexpr (NP == 2) {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = make_float2(a.x, a.y);
        v[NP - 1] = make_float2(a.z, a.w);
    } else {
#pragma unroll
        for (int q = 0; q < NP; q++) v[q] = *reinterpret_cast<const float2 *>(p + 2 * q);
    }
}
/// Stores of NP pairs to R consecutive rows of a field.
template <int NP> __device__ __forceinline__ void storeRows(float *p, const float2 (&v)[NP]) {
    if constexpr (NP == 2) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0].x, v[0].y, v[NP - 1].x, v[NP - 1].y);
    } else {
#pragma unroll
        for (int q = 0; q < NP; q++) *reinterpret_cast<float2 *>(p + 2 * q) = v[q];
    }
}
__device__ __forceinline__ float lanePick(float2 v, int i) { return i ? v.y : v.x; }

/// HLLE: the next state's maximum wave speed is the largest cell speed
/// c + max(|u|, |v|) over its wet cells -- exactly, in exact arithmetic: every
/// edge speed is at most the larger cell speed of its two cells (|uRoe| is a
/// sqrt(h)-weighted mean of |u|, cRoe at most the same mean of c, and the
/// Einfeldt bounds are the cells' own u -/+ c), and every wet cell's u + c
/// and c - u are the Einfeldt bounds of its left and right edges (v likewise
/// in y; a dry neighbour's mirror image gives the same).  A dry cell
/// (h < dryTol, momenta cleared by the clamp) has c + 0 < sqrt(g dryTol), below
/// every wet cell's speed, so a thread keeps the largest cell speed of all
/// its cells and drops it when none of them was wet.  Only edges to ghosts
/// that keep their own values need their speed evaluated.  The f-wave solver
/// has no such identity: its edges are evaluated one by one, those between
/// two segments as pieces.
///
/// Each thread owns R = 2 NP consecutive rows, computed as NP packed pairs.
template <int S, int NP, int MINB>
__global__ void __launch_bounds__(kMaxTileRows / (2 * NP), MINB) fastStepKernel(const FastDev f) {
    constexpr int R = 2 * NP;
    constexpr int NT = kMaxTileRows / R;
    constexpr int NW = (NT + 31) / 32;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr bool EDGES = S == SOLVER_FWAVE;  // next-state speeds edge by edge
    using T_ = std::true_type;
    using F_ = std::false_type;
    extern __shared__ __align__(128) float ring[];  // kRing strips of kSlotFloats
    __shared__ __align__(8) unsigned long long mbar[kRing];
    __shared__ unsigned slotDone[kRing];  // releases of a slot so far (nw per column)
    __shared__ float sRed[NW];
    __shared__ long long sRimGhost[NT][R];  // rim rows: the ghost row's offset from the block's base
    __shared__ int sRimPitch[NT][R];        // and its pitch
    __shared__ int sLast, sNWon, sAbort;
    __shared__ int sWon[kMaxArrivals];

    const int t = threadIdx.x, lane = t & 31, nth = blockDim.x, nw = nth >> 5, TY = R * nth;
    // strips start as a state at rest (rows a partial tile never loads stay finite)
#pragma unroll
    for (int s = 0; s < kRing; s++)
#pragma unroll
        for (int q = 0; q < 4; q++)
            for (int i = t; i < kSlice; i += nth) ring[s * kSlotFloats + q * kSlice + i] = q == 0 ? 1.f : 0.f;
    // the partition and the block descriptors are written only when the
    // domain is built: bring the first segment's into L1 before the wait
    if (t == 0) {
        const int s0 = f.ctaSeg[blockIdx.x];
        if (s0 < f.ctaSeg[blockIdx.x + 1]) {
            prefetchL1(&f.units[s0]);
            prefetchL1(&f.d.blocks[f.units[s0].block]);
        }
    }
    if (t == 0) {
        for (int s = 0; s < kRing; s++) {
            mbarInit(smemAddr(&mbar[s]), 1u);
            slotDone[s] = 0u;
        }
        sAbort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // slot of the next column and the rotations so far (the slot's phase
    // parity); the rotation continues across segments
    int slot = 0;
    unsigned rnd = 0u;
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
        float2 dtdx, dtdy;
        {
            const float dt = __ldg(&G->dt);
            dtdx = pk(__fdiv_rn(dt, __ldg(&B.dx)));
            dtdy = pk(__fdiv_rn(dt, __ldg(&B.dy)));
        }
        const float *__restrict__ Hin = pick(f.d.h, cur);
        const float *__restrict__ HUin = pick(f.d.hu, cur);
        const float *__restrict__ HVin = pick(f.d.hv, cur);
        float *__restrict__ HO = pick(f.d.h, cur ^ 1) + base;
        float *__restrict__ HUO = pick(f.d.hu, cur ^ 1) + base;
        float *__restrict__ HVO = pick(f.d.hv, cur ^ 1) + base;
        const int slot0 = slot;
        // the strip of column x0-1+k (rows rowStart ..) into slot s
        auto refill = [&](int k, int s) {
            const unsigned mb = smemAddr(&mbar[s]);
            mbarExpectTx(mb, 4u * bytes);
            const size_t col = size_t(base) + size_t(x0 - 1 + k) * P + size_t(rowStart);
            const unsigned dst = ringAddr + unsigned(s * kSlotFloats) * 4u;
            bulkLoad(dst, Hin + col, bytes, mb);
            bulkLoad(dst + unsigned(kSlice) * 4u, HUin + col, bytes, mb);
            bulkLoad(dst + unsigned(2 * kSlice) * 4u, HVin + col, bytes, mb);
            bulkLoad(dst + unsigned(3 * kSlice) * 4u, f.d.b + col, bytes, mb);
        };

        __syncthreads();  // the previous segment is done with every slot and shared value
        if (t == 0) {
            sNWon = 0;
            for (int k = 0; k < min(kRing, ncol); k++) refill(k, slot0 + k < kRing ? slot0 + k : slot0 + k - kRing);
        }

        const int yA = y0 + R * t;                       // this thread's first row
        const int nAct = max(0, min(R, yTop - yA + 1));  // its rows inside the tile
        const bool fullTile = yTop - y0 + 1 == TY;       // every thread has R rows (CTA-uniform)
        const bool upIn = yA + R <= yTop;                // the next thread's first row is in the tile
        // rows on the block's rim (y == 1, y == ny): ghost below / above.
        // rimMode (3 bits per row): 0 none, 1 copy, 2 copy with -hv, 3 kept
        // ghost (its edge speed is evaluated), 4 every ghost edge evaluated
        // (f-wave); the ghost row's offset and pitch wait in shared memory
        int rimModes = 0;
        bool rimAny = false;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int y = yA + r;
            if (r < nAct && (y == 1 || y == ny)) {
                rimAny = true;
                const int side = (y == 1) ? 2 : 3;
                const int type = __ldg(&B.bnd[side]);
                long long ghost = (side == 2) ? 0 : ny + 1;
                int pitch = int(P), mode;
                if (ny == 1 || EDGES) {
                    mode = 4;
                } else if (type == OUTFLOW || type == WALL) {
                    mode = type == WALL ? 2 : 1;
                } else if (type == CONNECT_WITHIN_RANK) {
                    const BlockDesc &N = f.d.blocks[__ldg(&B.nbr[side])];
                    mode = 1;
                    ghost = __ldg(&N.base) - base + ((side == 2) ? __ldg(&N.ny) + 1 : 0);
                    pitch = __ldg(&N.pitch);
                } else {
                    mode = 3;
                }
                rimModes |= mode << (3 * r);
                sRimGhost[t][r] = ghost;
                sRimPitch[t][r] = pitch;
            }
        }
        const bool rimWarp = __any_sync(FULL, rimAny);

        FQ2 px[NP];                                      // the previous column's cells (x direction)
        float2 pendH[NP], pendHU[NP];                    // right-going parts of their left x-edges
        float2 syH[NP], syHV[NP], oldHV[NP];             // their y sums and hv
        float2 hsum = pk(0.f);                           // new depths (not finite: a non-finite cell)
        float smax = 0.f, wmax = 0.f, hmax = 0.f;        // edge speeds; HLLE cell speeds and depths
        SV nprev[R];
#pragma unroll
        for (int q = 0; q < NP; q++) pendH[q] = pendHU[q] = syH[q] = syHV[q] = oldHV[q] = pk(0.f);
#pragma unroll
        for (int r = 0; r < R; r++) nprev[r] = SV{1.f, 0.f, 1.f, 0.f};
        const int i0 = kHalo + R * t;  // strip index of this thread's first row
        unsigned oldPrev = 0u;         // lane 0: the previous column's release count

        // one column x = x0-1+k: XCOL its x-edges (x-1 | x), YCOL its y-edges,
        // UPD the update of column x-1, RIMX column x-1 may be on the block's
        // left or right rim.  False: a copy did not arrive in time.
        auto column = [&](int k, auto xcolT, auto ycolT, auto updT, auto rimxT) -> bool {
            constexpr bool XCOL = decltype(xcolT)::value, YCOL = decltype(ycolT)::value;
            constexpr bool UPD = decltype(updT)::value, RIMX = decltype(rimxT)::value;
            // wait for the strip (bounded; a stalled copy aborts the CTA)
            {
                const unsigned a = smemAddr(&mbar[slot]);
                const unsigned par = rnd & 1u;
                if (!__all_sync(FULL, mbarTryWait(a, par))) {
                    bool ok = false;
                    for (unsigned n = 0; !ok && n < kSpinLimit; ++n) {
                        if (*(volatile int *)&sAbort) break;
                        ok = __all_sync(FULL, mbarTryWait(a, par));
                    }
                    if (!ok) {
                        if (lane == 0) *(volatile int *)&sAbort = 1;
                        return false;
                    }
                }
            }
            const float *sl = ring + slot * kSlotFloats;
            float2 ch[NP], chu[NP], chv[NP], cb[NP];
            loadRows<NP>(sl + i0, ch);
            loadRows<NP>(sl + kSlice + i0, chu);
            loadRows<NP>(sl + 2 * kSlice + i0, chv);
            loadRows<NP>(sl + 3 * kSlice + i0, cb);
            float uh = 0.f, uhv = 0.f, ub = 0.f, lh = 0.f, lhv = 0.f, lb = 0.f;
            if (YCOL) {
                uh = sl[i0 + R];
                uhv = sl[2 * kSlice + i0 + R];
                ub = sl[3 * kSlice + i0 + R];
                if (lane == 0) {  // the cell below the warp's first row
                    lh = sl[i0 - 1];
                    lhv = sl[2 * kSlice + i0 - 1];
                    lb = sl[3 * kSlice + i0 - 1];
                }
            }
            // A. this thread's cells of column x, the cell above its rows and
            // (lane 0) the one below
            FQ2 cx[NP], cy[NP];
#pragma unroll
            for (int q = 0; q < NP; q++) {
                const float2 rr = rsqrt2(ch[q]);
                const float2 sq = mul2(ch[q], rr), ih = mul2(rr, rr), c = mul2(pk(kSqrtG), sq);
                const float2 eta = add2(ch[q], cb[q]);
                cx[q] = makeFQ2(ch[q], chu[q], eta, ih, sq, c);
                cy[q] = makeFQ2(ch[q], chv[q], eta, ih, sq, c);
            }
            FQ up{}, low{};
            if (YCOL) {
                up = rawFQ(uh, uhv, ub);
                if (lane == 0) low = rawFQ(lh, lhv, lb);
            }
            // the strip's values are in use, so its reads are complete:
            // release it.  The slot's last releaser refills it; lane 0 reads
            // its count one column later, so no warp waits on the atomic.
            __syncwarp();
            if (lane == 0) {
                if (k >= 1 && k - 1 + kRing < ncol) {
                    const int sp = slot == 0 ? kRing - 1 : slot - 1;
                    const unsigned rp = slot == 0 ? rnd - 1u : rnd;
                    if (oldPrev + 1u == unsigned(nw) * (rp + 1u)) refill(k - 1 + kRing, sp);
                }
                unsigned old;
                asm volatile("atom.shared::cta.add.u32 %0, [%1], 1;"
                             : "=r"(old)
                             : "r"(smemAddr(&slotDone[slot])), "f"(cx[0].m.x), "f"(cx[0].m.y), "f"(cy[0].m.x),
                               "f"(cy[0].m.y), "f"(cx[0].eta.x), "f"(cx[0].eta.y), "f"(up.m), "f"(up.eta), "f"(low.m),
                               "f"(low.eta)
                             : "memory");
                oldPrev = old;
            }
            if (++slot == kRing) {
                slot = 0;
                ++rnd;
            }
            // B. x-edges (x-1 | x) and the y-edges between this thread's rows
            // and from its last row to the staged row above (lane 0: also the
            // one below its first row), all taken as wet and subsonic first
            float2 aLx[NP], aRx[NP], auLx[NP], auRx[NP], aLy[NP], aRy[NP], auLy[NP], auRy[NP];
            float sub = 3.0e38f, minh = 3.0e38f;
#pragma unroll
            for (int q = 0; q < NP; q++) minh = fminf(minh, fminf(ch[q].x, ch[q].y));
            if (XCOL) {
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    waves2<S>(px[q], cx[q], aLx[q], aRx[q], auLx[q], auRx[q], sub);
                    minh = fminf(minh, fminf(px[q].h.x, px[q].h.y));
                }
            }
            float lowRh = 0.f, lowRhv = 0.f;
            if (YCOL) {
#pragma unroll
                for (int q = 0; q < NP; q++)
                    waves2<S>(cy[q], pairFQ(laneY(cy[q]), q + 1 < NP ? laneX(cy[(q + 1) % NP]) : up), aLy[q], aRy[q],
                              auLy[q], auRy[q], sub);
                minh = fminf(minh, up.h);
                if (lane == 0) {
                    float dl, dlv;
                    waves<S, false>(low, laneX(cy[0]), dl, lowRh, dlv, lowRhv, sub);
                    minh = fminf(minh, low.h);
                }
            }
            // C. a lane with a dry cell or an edge that is not subsonic solves
            // its edges again in full (rare: shorelines, fronts)
            if (XCOL || YCOL) {
                const bool redo = minh < kDryTol || !(sub > kZeroTol);
                if (__any_sync(FULL, redo)) {
                    if (redo) {
                        if (XCOL) {
#pragma unroll
                            for (int q = 0; q < NP; q++) {
                                const float4 e0 = edgeGeneral<S>(laneX(px[q]), laneX(cx[q]));
                                const float4 e1 = edgeGeneral<S>(laneY(px[q]), laneY(cx[q]));
                                aLx[q] = make_float2(e0.x, e1.x);
                                aRx[q] = make_float2(e0.y, e1.y);
                                auLx[q] = make_float2(e0.z, e1.z);
                                auRx[q] = make_float2(e0.w, e1.w);
                            }
                        }
                        if (YCOL) {
#pragma unroll
                            for (int q = 0; q < NP; q++) {
                                const float4 e0 = edgeGeneral<S>(laneX(cy[q]), laneY(cy[q]));
                                const float4 e1 =
                                    edgeGeneral<S>(laneY(cy[q]), q + 1 < NP ? laneX(cy[(q + 1) % NP]) : up);
                                aLy[q] = make_float2(e0.x, e1.x);
                                aRy[q] = make_float2(e0.y, e1.y);
                                auLy[q] = make_float2(e0.z, e1.z);
                                auRy[q] = make_float2(e0.w, e1.w);
                            }
                            if (lane == 0) {
                                const float4 e2 = edgeGeneral<S>(low, laneX(cy[0]));
                                lowRh = e2.y;
                                lowRhv = e2.w;
                            }
                        }
                    }
                }
            }
            // D. cells (x-1, y): Q^{n+1} with the dry clamp, and their part
            // of the next maxTimestep
            if (UPD) {
                const int xc = x0 - 2 + k;
                float2 hn[NP], hun[NP], hvn[NP];
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    hn[q] = sub2(px[q].h, fma2(dtdx, add2(pendH[q], aLx[q]), mul2(dtdy, syH[q])));
                    hun[q] = sub2(px[q].hn, mul2(dtdx, add2(pendHU[q], auLx[q])));
                    hvn[q] = sub2(oldHV[q], mul2(dtdy, syHV[q]));
                    if (fullTile) {
                        hsum = add2(hsum, hn[q]);
                    } else {
                        hsum.x += 2 * q < nAct ? hn[q].x : 0.f;
                        hsum.y += 2 * q + 1 < nAct ? hn[q].y : 0.f;
                    }
                    hun[q].x = (hn[q].x < 0.1f) ? 0.f : hun[q].x;
                    hvn[q].x = (hn[q].x < 0.1f) ? 0.f : hvn[q].x;
                    hun[q].y = (hn[q].y < 0.1f) ? 0.f : hun[q].y;
                    hvn[q].y = (hn[q].y < 0.1f) ? 0.f : hvn[q].y;
                    hn[q].x = fmaxf(hn[q].x, 0.f);
                    hn[q].y = fmaxf(hn[q].y, 0.f);
                }
                const unsigned o = unsigned(xc) * P + unsigned(yA);
                if (fullTile) {
                    storeRows<NP>(HO + o, hn);
                    storeRows<NP>(HUO + o, hun);
                    storeRows<NP>(HVO + o, hvn);
                } else {
#pragma unroll
                    for (int r = 0; r < R; r++)
                        if (r < nAct) {
                            HO[o + r] = lanePick(hn[r / 2], r & 1);
                            HUO[o + r] = lanePick(hun[r / 2], r & 1);
                            HVO[o + r] = lanePick(hvn[r / 2], r & 1);
                        }
                }
                float2 rn[NP];
#pragma unroll
                for (int q = 0; q < NP; q++) rn[q] = rsqrt2(hn[q]);
                if (!EDGES) {
                    // HLLE: cell speeds c + max(|u|, |v|) (a dry cell: NaN for
                    // h = 0, below every wet cell's speed otherwise)
#pragma unroll
                    for (int q = 0; q < NP; q++) {
                        const float2 vmax = make_float2(fmaxf(fabsf(hun[q].x), fabsf(hvn[q].x)),
                                                        fmaxf(fabsf(hun[q].y), fabsf(hvn[q].y)));
                        const float2 w = fma2(vmax, mul2(rn[q], rn[q]), mul2(pk(kSqrtG), mul2(hn[q], rn[q])));
                        if (fullTile) {
                            wmax = fmaxf(wmax, fmaxf(w.x, w.y));
                            hmax = fmaxf(hmax, fmaxf(hn[q].x, hn[q].y));
                        } else {
                            wmax = fmaxf(wmax, fmaxf(2 * q < nAct ? w.x : 0.f, 2 * q + 1 < nAct ? w.y : 0.f));
                            hmax = fmaxf(hmax, fmaxf(2 * q < nAct ? hn[q].x : 0.f, 2 * q + 1 < nAct ? hn[q].y : 0.f));
                        }
                    }
                } else {
                    // f-wave: x-edges (x-2 | x-1), the y-edges between this
                    // thread's rows and the one to the next lane's first row
                    // (the last lane's goes to the pass after the sweep)
                    SV nxv[R], nyv[R];
                    float nminh = 3.0e38f;
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const float hr = lanePick(hn[r / 2], r & 1), rr2 = lanePick(rn[r / 2], r & 1);
                        nxv[r] = makeSV(hr, lanePick(hun[r / 2], r & 1), rr2);
                        nyv[r] = makeSV(hr, lanePick(hvn[r / 2], r & 1), rr2);
                        nminh = fminf(nminh, fminf(hr, nprev[r].h));
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
                    for (int r = 0; r + 1 < R; r++) sp[R + r] = wetSpeed<S>(nyv[r], nyv[r + 1]);
                    sp[2 * R] = wetSpeed<S>(nyv[R - 1], nu);
                    const bool nredo = nminh < kDryTol;
                    if (__any_sync(FULL, nredo)) {
                        if (nredo) {
#pragma unroll
                            for (int r = 0; r < R; r++) sp[r] = speedGeneral<S>(nprev[r], nxv[r]);
#pragma unroll
                            for (int r = 0; r + 1 < R; r++) sp[R + r] = speedGeneral<S>(nyv[r], nyv[r + 1]);
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
                if (RIMX && (xc == 1 || xc == nx)) {
#pragma unroll
                    for (int r = 0; r < R; r++)
                        if (r < nAct)
                            smax = fmaxf(smax, rimCell<S>(pick(f.d.h, cur ^ 1), pick(f.d.hu, cur ^ 1), pick(f.d.hv, cur ^ 1),
                                                          Hin, HUin, HVin, f.d.blocks, wu.block, xc, yA + r,
                                                          lanePick(hn[r / 2], r & 1), lanePick(hun[r / 2], r & 1),
                                                          lanePick(hvn[r / 2], r & 1)));
                } else if (rimWarp) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const int mode = (rimModes >> (3 * r)) & 7;
                        if (mode == 0) continue;
                        const float hr = lanePick(hn[r / 2], r & 1), ur = lanePick(hun[r / 2], r & 1),
                                    vr = lanePick(hvn[r / 2], r & 1);
                        if (mode >= 3) {
                            smax = fmaxf(smax, rimCell<S>(pick(f.d.h, cur ^ 1), pick(f.d.hu, cur ^ 1), pick(f.d.hv, cur ^ 1),
                                                          Hin, HUin, HVin, f.d.blocks, wu.block, xc, yA + r, hr, ur, vr));
                        } else {
                            const long long g = sRimGhost[t][r] + (long long)xc * sRimPitch[t][r];
                            HO[g] = hr;
                            HUO[g] = ur;
                            HVO[g] = mode == 2 ? -vr : vr;
                        }
                    }
                }
            }
            if (YCOL) {
                // y-sums of column x: the first row's bottom edge from the
                // lane below (lane 0: its own), the rest from this lane's edges
                const float pH = __shfl_up_sync(FULL, aRy[NP - 1].y, 1), pHV = __shfl_up_sync(FULL, auRy[NP - 1].y, 1);
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    const float bH = q == 0 ? (lane == 0 ? lowRh : pH) : aRy[(q + NP - 1) % NP].y;
                    const float bHV = q == 0 ? (lane == 0 ? lowRhv : pHV) : auRy[(q + NP - 1) % NP].y;
                    syH[q] = add2(make_float2(bH, aRy[q].x), aLy[q]);
                    syHV[q] = add2(make_float2(bHV, auRy[q].x), auLy[q]);
                    oldHV[q] = chv[q];
                }
            }
#pragma unroll
            for (int q = 0; q < NP; q++) {
                if (XCOL) {
                    pendH[q] = aRx[q];
                    pendHU[q] = auRx[q];
                }
                px[q] = cx[q];
            }
            return true;
        };

        bool ok = column(0, F_{}, F_{}, F_{}, F_{}) && column(1, T_{}, T_{}, F_{}, F_{});
        if (ok && XC >= 2) {
            ok = column(2, T_{}, T_{}, T_{}, T_{});
            for (int k = 3; ok && k <= XC; ++k) ok = column(k, T_{}, T_{}, T_{}, F_{});
        }
        if (ok) ok = column(XC + 1, T_{}, F_{}, T_{}, T_{});
        if (!EDGES) smax = fmaxf(smax, hmax >= kDryTol ? wmax : 0.f);
        const bool bad = !(fabsf(hsum.x + hsum.y) <= FLT_MAX);
        __syncthreads();  // every warp's sweep is done: its stores are visible to the CTA
        if (sAbort) {
            // a copy did not arrive in time: wait (bounded) for the copies in
            // flight, flag the group and leave the kernel
            if (t == 0) {
                for (int s = 0; s < kRing; s++) mbarWait(smemAddr(&mbar[s]), (s < slot ? rnd + 1u : rnd) & 1u);
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

/// Packed row pairs per thread of the step kernel and its resident CTAs per
/// SM.  One pair at four CTAs of 128 threads: 128 registers, no spills, 16
/// warps per SM.  The kernel is latency-bound, so warps count for more than
/// instructions: two pairs issue 25% fewer instructions but need 216
/// registers (8 warps per SM) and run 6% slower; one pair at five CTAs
/// spills.
constexpr int kPairs = 1;
constexpr int kMinCtas = 4;

int fastRows() { return 2 * kPairs; }

cudaError_t launchFastStep(const FastDev &f, int solver, int grid, int tileRows, cudaStream_t s) {
    const int threads = tileRows / (2 * kPairs);
    const cudaError_t e =
        solver == SOLVER_FWAVE
            ? launchPdlSmem(fastStepKernel<SOLVER_FWAVE, kPairs, kMinCtas>, dim3(grid), dim3(threads), kRingBytes, s, f)
            : launchPdlSmem(fastStepKernel<SOLVER_HLLE, kPairs, kMinCtas>, dim3(grid), dim3(threads), kRingBytes, s, f);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int fastOccupancy(int solver, int tileRows) {
    int a = 0;
    const int threads = tileRows / (2 * kPairs);
    if (solver == SOLVER_FWAVE)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fastStepKernel<SOLVER_FWAVE, kPairs, kMinCtas>, threads,
                                                      kRingBytes);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fastStepKernel<SOLVER_HLLE, kPairs, kMinCtas>, threads,
                                                      kRingBytes);
    return a;
}

} // namespace fast
} // namespace swegb
