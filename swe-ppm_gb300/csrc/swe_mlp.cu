// MLP surrogate of the augmented Riemann solver on fifth-generation tensor
// cores (tcgen05; primitives in swe_tc.cuh).
//
// The surrogate is an f-wave solver whose two wave speeds are the Roe speeds
// plus corrections predicted by a 6 -> 64 -> 64 -> 64 -> 4 SiLU network.  The
// strengths follow from the speeds by the f-wave closure, so the waves sum to
// the flux difference and mass is conserved by construction.  The network also
// predicts the two strengths; their distance to the closure's is the gate that
// sends an edge back to the augmented solver, as do dry or shallow sides
// (< 0.1 m: the switch depth of the reference's hybrid solver, whose call
// sites are src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410).
//
// Tensor-core mapping: a tile is 128 edges, one per thread and one per TMEM
// lane.  Every layer is one M = 128 GEMM with BF16 operands in shared memory
// (weights staged once per CTA) and the FP32 accumulator in TMEM; the
// epilogue (bias, SiLU, BF16 rounding) is done by the thread that owns the
// edge's lane and writes the next layer's operand row.  Training runs the
// backward pass in the same kernel: dA = dZ W reads the weights through the
// transposed (MN-major) descriptor, and the weight gradients dW = dZ^T A read
// the stored dZ and activation buffers transposed, with K running over the
// tile's edges; they accumulate in TMEM over all tiles of the CTA, the bias
// gradients as dZ^T times a block of ones.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "../../include/swe_gb300_mlp.h"
#include "swe_device.cuh"
#include "swe_mlp_launch.hpp"
#include "swe_sweep.cuh"
#include "swe_tc.cuh"

namespace swegb {
namespace mlp {

constexpr int kIn = 6, kHid = 64, kOut = 4;
constexpr int kInPad = 16, kOutPad = 16;  // K of layer 1 and N of layer 4, padded to the MMA minimum
constexpr int kTile = 128;                // edges per tile
// flat FP32 parameter vector: W1[64][6], b1, W2[64][64], b2, W3[64][64], b3, W4[4][64], b4
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kHid * kHid, oW4 = oB3 + kHid, oB4 = oW4 + kOut * kHid, kNParams = oB4 + kOut;
static_assert(kNParams == SWE_MLP_NPARAMS, "parameter count");
// packed image: BF16 weights in the core-matrix layout (K-major, one row per
// output neuron), then the FP32 biases b1 | b2 | b3 | b4 (b4 padded to 16)
constexpr int pW1 = 0, pW2 = pW1 + kHid * kInPad * 2, pW3 = pW2 + kHid * kHid * 2, pW4 = pW3 + kHid * kHid * 2,
              pBias = pW4 + kOutPad * kHid * 2, kBiasFloats = 3 * kHid + 16, kImageBytes = pBias + kBiasFloats * 4;
constexpr int kImageSmem = (kImageBytes + 255) / 256 * 256;
constexpr int kX0Bytes = kTile * kInPad * 2, kActBytes = kTile * kHid * 2, kOnesBytes = 16 * kTile * 2;
constexpr int kPartStride = kNParams + 4;  // per-CTA partial gradient, then the loss sum

// surrogate constants (gate and training)
constexpr float kWet = 0.1f;          // both sides at least this deep
constexpr float kClip = 8.f;          // feature clip
constexpr float kLambda = 0.1f;       // weight of the strength-consistency term
constexpr float kGateTau = 0.25f;     // |strengths - closure| <= tau (|closure|) + 1e-3 h c
constexpr float kMinSpread = 0.5f;    // s2 - s1 >= 0.5 c to use the surrogate
constexpr float kTrainSpread = 0.1f;  // s2 - s1 < 0.1 c: no gradient

// forward (inference) kernel: shared memory and TMEM columns
constexpr int kFwdX0 = kImageSmem, kFwdAct = kFwdX0 + kX0Bytes, kFwdSmem = kFwdAct + kActBytes;
constexpr uint32_t kFwdCols = 64;
// training kernel: shared memory ...
constexpr int kTrOnes = kImageSmem, kTrX0 = kTrOnes + kOnesBytes, kTrA1 = kTrX0 + kX0Bytes, kTrA2 = kTrA1 + kActBytes,
              kTrA3 = kTrA2 + kActBytes, kTrDZ4 = kTrA3 + kActBytes, kTrDZ = kTrDZ4 + kX0Bytes,
              kTrGuard = kTrDZ + kActBytes, kTrEnd = kTrGuard + 2048;
// ... requested larger than half an SM's shared memory, so one CTA owns the SM's 512 TMEM columns
constexpr int kTrSmem = 120 * 1024;
static_assert(kTrEnd <= kTrSmem, "training shared memory");
// ... and TMEM columns: pre-activations Z1..Z3, outputs O, dA, and the
// gradient accumulators (rows = output neurons of the layer, except gW4T)
constexpr uint32_t cZ1 = 0, cZ2 = 64, cZ3 = 128, cO = 192, cGW1 = 208, cGW4 = 224, cDB1 = 240, cDA = 256, cGW2 = 320,
                   cGW3 = 384, cDB2 = 448, cDB3 = 464, cDB4 = 480, kTrCols = 512;

// Over-reads of the padded (garbage) accumulator rows: an MN-major A operand
// with 64 (16) valid rows is read as 128 rows, i.e. up to 1024 (1792) bytes
// past its buffer -- A3 into dZ4, dZ4 into dZ, dZ into the guard.  Those rows
// of D are never read back.
static_assert(kTrDZ4 == kTrA3 + kActBytes && kTrDZ == kTrDZ4 + kX0Bytes && kTrGuard == kTrDZ + kActBytes, "");

__device__ __forceinline__ float tanhApprox(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
/// SiLU z * sigmoid(z) = h + h tanh(h), h = z / 2
__device__ __forceinline__ float silu(float z) {
    const float h = 0.5f * z;
    return fmaf(h, tanhApprox(h), h);
}
/// the same from h = z / 2
__device__ __forceinline__ float siluHalf(float h) { return fmaf(h, tanhApprox(h), h); }
/// d SiLU / dz = s (1 + z (1 - s)), s = sigmoid(z) = (1 + tanh(z / 2)) / 2
__device__ __forceinline__ float dsilu(float z) {
    const float s = fmaf(0.5f, tanhApprox(0.5f * z), 0.5f);
    return s * fmaf(z, 1.f - s, 1.f);
}
__device__ __forceinline__ uint32_t packBf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

/// the edge quantities the surrogate needs
struct EdgeFeat {
    float x[kIn];
    float hm, c, s10, s20, dF1, dF2;
    bool wet;
};

__device__ __forceinline__ void edgeFeatures(float hL, float hR, float huL, float huR, float bL, float bR, EdgeFeat &f) {
    f.hm = 0.5f * (hL + hR);
    f.c = sqrtf(kG * f.hm);
    const float rhm = 1.f / f.hm, rc = 1.f / f.c;
    const float uL = huL / hL, uR = huR / hR;
    f.x[0] = (hL - f.hm) * rhm;
    f.x[1] = (hR - f.hm) * rhm;
    f.x[2] = uL * rc;
    f.x[3] = uR * rc;
    f.x[4] = (bR - bL) * rhm;
    f.x[5] = ((hL + bL) - (hR + bR)) * rhm;
    const float sqL = sqrtf(hL), sqR = sqrtf(hR);
    const float uRoe = (uL * sqL + uR * sqR) / (sqL + sqR);
    f.s10 = uRoe - f.c;
    f.s20 = uRoe + f.c;
    f.dF1 = huR - huL;
    f.dF2 = ((huR * uR + kHalfG * hR * hR) - (huL * uL + kHalfG * hL * hL)) + kHalfG * (hL + hR) * (bR - bL);
    f.wet = hL >= kWet && hR >= kWet;
#pragma unroll
    for (int k = 0; k < kIn; k++) f.x[k] = f.wet ? fminf(fmaxf(f.x[k], -kClip), kClip) : 0.f;
}

/// speeds, closure strengths, predicted strengths and net updates of the surrogate
struct Waves {
    float s1, s2, D, b1, b2, bh1, bh2, w1, w2, U[4];
    bool finite;
};

__device__ __forceinline__ void surrogateWaves(const float o[4], const EdgeFeat &f, Waves &w) {
    w.s1 = fmaf(f.c, o[0], f.s10);
    w.s2 = fmaf(f.c, o[1], f.s20);
    w.D = w.s2 - w.s1;
    const float rD = 1.f / w.D;
    w.b1 = fmaf(w.s2, f.dF1, -f.dF2) * rD;
    w.b2 = fmaf(-w.s1, f.dF1, f.dF2) * rD;
    const float hc = f.hm * f.c;
    w.bh1 = o[2] * hc;
    w.bh2 = o[3] * hc;
    w.w1 = leftShare(w.s1);
    w.w2 = leftShare(w.s2);
    const float z1 = w.b1 * w.s1, z2 = w.b2 * w.s2;
    w.U[0] = fmaf(w.w2, w.b2, w.w1 * w.b1);
    w.U[1] = fmaf(1.f - w.w2, w.b2, (1.f - w.w1) * w.b1);
    w.U[2] = fmaf(w.w2, z2, w.w1 * z1);
    w.U[3] = fmaf(1.f - w.w2, z2, (1.f - w.w1) * z1);
    w.finite = isfinite(w.U[0]) && isfinite(w.U[1]) && isfinite(w.U[2]) && isfinite(w.U[3]);
}

__device__ __forceinline__ bool surrogateGate(const EdgeFeat &f, const Waves &w) {
    const float hc = f.hm * f.c;
    const float err = fabsf(w.bh1 - w.b1) + fabsf(w.bh2 - w.b2);
    return f.wet && w.finite && w.D >= kMinSpread * f.c && err <= fmaf(kGateTau, fabsf(w.b1) + fabsf(w.b2), 1e-3f * hc);
}

/// loss of one edge and dLoss/dOutputs (already divided by the batch size)
__device__ __forceinline__ float edgeLoss(const float o[4], const EdgeFeat &f, const float T[4], float invN, bool valid,
                                          float dO[4]) {
    Waves w;
    surrogateWaves(o, f, w);
    dO[0] = dO[1] = dO[2] = dO[3] = 0.f;
    if (!(valid && f.wet && w.finite && w.D >= kTrainSpread * f.c)) return 0.f;
    const float hc = f.hm * f.c, hcc = hc * f.c;
    const float ish = 1.f / (hc * hc), ishu = 1.f / (hcc * hcc);
    float e[4];
#pragma unroll
    for (int k = 0; k < 4; k++) e[k] = w.U[k] - T[k];
    const float db1 = w.bh1 - w.b1, db2 = w.bh2 - w.b2;
    const float L = (e[0] * e[0] + e[1] * e[1]) * ish + (e[2] * e[2] + e[3] * e[3]) * ishu +
                    kLambda * (db1 * db1 + db2 * db2) * ish;
    const float gh = 2.f * ish * invN, ghu = 2.f * ishu * invN;
    const float g0 = e[0] * gh, g1 = e[1] * gh, g2 = e[2] * ghu, g3 = e[3] * ghu;
    const float gl1 = kLambda * db1 * gh, gl2 = kLambda * db2 * gh;
    const float v1 = 1.f - w.w1, v2 = 1.f - w.w2;
    const float gb1 = g0 * w.w1 + g1 * v1 + (g2 * w.w1 + g3 * v1) * w.s1 - gl1;
    const float gb2 = g0 * w.w2 + g1 * v2 + (g2 * w.w2 + g3 * v2) * w.s2 - gl2;
    const float q = (gb1 - gb2) / w.D;
    const float gs1 = (g2 * w.w1 + g3 * v1) * w.b1 + q * w.b1;
    const float gs2 = (g2 * w.w2 + g3 * v2) * w.b2 + q * w.b2;
    dO[0] = gs1 * f.c;
    dO[1] = gs2 * f.c;
    dO[2] = gl1 * hc;
    dO[3] = gl2 * hc;
    return L;
}

// ---------------------------------------------------------------------------
// shared-memory operand rows
// ---------------------------------------------------------------------------
/// BF16 feature row of edge `row` (K = 16, features 6..15 zero)
__device__ __forceinline__ void storeX0(uint8_t *sX, int row, const float x[kIn]) {
    uint4 lo = make_uint4(packBf16(x[0], x[1]), packBf16(x[2], x[3]), packBf16(x[4], x[5]), 0u);
    *reinterpret_cast<uint4 *>(sX + tc::coreOffset(row, 0, kInPad)) = lo;
    *reinterpret_cast<uint4 *>(sX + tc::coreOffset(row, 8, kInPad)) = make_uint4(0u, 0u, 0u, 0u);
}
/// BF16 dZ4 row (4 valid columns of 16)
__device__ __forceinline__ void storeDZ4(uint8_t *s, int row, const float d[4]) {
    *reinterpret_cast<uint4 *>(s + tc::coreOffset(row, 0, kOutPad)) =
        make_uint4(packBf16(d[0], d[1]), packBf16(d[2], d[3]), 0u, 0u);
    *reinterpret_cast<uint4 *>(s + tc::coreOffset(row, 8, kOutPad)) = make_uint4(0u, 0u, 0u, 0u);
}
/// 16 columns (two core matrices) of a 64-wide BF16 row
__device__ __forceinline__ void store16(uint8_t *s, int row, int c, const uint32_t p[8]) {
    *reinterpret_cast<uint4 *>(s + tc::coreOffset(row, c, kHid)) = make_uint4(p[0], p[1], p[2], p[3]);
    *reinterpret_cast<uint4 *>(s + tc::coreOffset(row, c + 8, kHid)) = make_uint4(p[4], p[5], p[6], p[7]);
}

/// epilogue of a hidden layer: A = bf16(silu(Z + b)) for this thread's row;
/// hbias = b / 2, so h = (Z + b) / 2 is one fused multiply-add, rounded as
/// 0.5 (Z + b)
__device__ __forceinline__ void epilogueSilu(uint32_t tz, const float *hbias, uint8_t *dst, int row) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tc::load16(tz, c, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; j++)
            p[j] = packBf16(siluHalf(fmaf(0.5f, v[2 * j], hbias[c + 2 * j])),
                            siluHalf(fmaf(0.5f, v[2 * j + 1], hbias[c + 2 * j + 1])));
        store16(dst, row, c, p);
    }
}
/// backward epilogue: dZ = bf16(dA * silu'(Z + b)) for this thread's row
__device__ __forceinline__ void epilogueDsilu(uint32_t tda, uint32_t tz, const float *bias, uint8_t *dst, int row) {
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
        float g[16], z[16];
        tc::load16(tda, c, g);
        tc::load16(tz, c, z);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; j++)
            p[j] = packBf16(g[2 * j] * dsilu(z[2 * j] + bias[c + 2 * j]), g[2 * j + 1] * dsilu(z[2 * j + 1] + bias[c + 2 * j + 1]));
        store16(dst, row, c, p);
    }
}

/// all threads: make this thread's shared-memory writes and TMEM reads
/// ordered before MMAs that one thread issues after the barrier
__device__ __forceinline__ void publishToMma() {
    tc::fenceSmemForMma();
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
}
/// all threads: wait for the committed MMAs; false (everywhere) on time-out
__device__ __forceinline__ bool awaitMma(uint64_t *mbar, uint32_t &phase) {
    const bool ok = __syncthreads_and(tc::mbarWait(mbar, phase));
    phase ^= 1u;
    tc::fenceAfterSync();
    return ok;
}

/// stage the packed weights (and biases) into shared memory, and the hidden
/// layers' halved biases (the SiLU epilogue works on (Z + b) / 2)
__device__ __forceinline__ void stageImage(const uint8_t *image, uint8_t *s, float *hbias) {
    const int4 *src = reinterpret_cast<const int4 *>(image);
    int4 *dst = reinterpret_cast<int4 *>(s);
    for (int i = threadIdx.x; i < kImageBytes / 16; i += blockDim.x) dst[i] = __ldg(src + i);
    const float *b = reinterpret_cast<const float *>(image + pBias);
    for (int i = threadIdx.x; i < 3 * kHid; i += blockDim.x) hbias[i] = 0.5f * __ldg(b + i);
}

/// the four forward GEMMs of one tile, with the epilogues between them; on
/// return the raw outputs sit in TMEM columns oCol.. (without b4).  act[l] is
/// the shared-memory buffer of layer l's output activations, zc[l] the TMEM
/// columns of its pre-activations.
__device__ __forceinline__ bool forwardTile(uint32_t tm, const uint8_t *sW, const float *hbias, const uint8_t *sX0,
                                            uint8_t *const act[3], const uint32_t zc[3], uint32_t oCol, uint64_t *mbar,
                                            uint32_t &phase) {
    const int t = threadIdx.x;
    publishToMma();
    if (t == 0) {
        tc::mma(tm + zc[0], tc::smemDesc(sX0, 0, kInPad), tc::smemDesc(sW + pW1, 0, kInPad), tc::idescBf16(128, kHid), false);
        tc::commit(mbar);
    }
    if (!awaitMma(mbar, phase)) return false;
    epilogueSilu(tm + zc[0], hbias, act[0], t);
    const int pw[2] = {pW2, pW3};
#pragma unroll
    for (int l = 0; l < 2; l++) {
        publishToMma();
        if (t == 0) {
#pragma unroll
            for (int kk = 0; kk < kHid / 16; kk++)
                tc::mma(tm + zc[l + 1], tc::smemDesc(act[l], kk * 16, kHid), tc::smemDesc(sW + pw[l], kk * 16, kHid),
                        tc::idescBf16(128, kHid), kk > 0);
            tc::commit(mbar);
        }
        if (!awaitMma(mbar, phase)) return false;
        epilogueSilu(tm + zc[l + 1], hbias + kHid * (l + 1), act[l + 1], t);
    }
    publishToMma();
    if (t == 0) {
#pragma unroll
        for (int kk = 0; kk < kHid / 16; kk++)
            tc::mma(tm + oCol, tc::smemDesc(act[2], kk * 16, kHid), tc::smemDesc(sW + pW4, kk * 16, kHid),
                    tc::idescBf16(128, kOutPad), kk > 0);
        tc::commit(mbar);
    }
    return awaitMma(mbar, phase);
}

/// edges in structure-of-arrays form: quantity k of edge e at v[k * stride + idx(e)]
struct EdgeBatch {
    const float *v;        // hL, hR, huL, huR, bL, bR
    const float *targets;  // hUpdL, hUpdR, huUpdL, huUpdR (training)
    const int *perm;       // optional index map
    long long stride;
    int offset, count;
    __device__ __forceinline__ long long index(int i) const { return perm ? (long long)perm[offset + i] : (long long)(offset + i); }
};

enum FwdMode { FWD_OUTPUTS = 0, FWD_SOLVE = 1 };

/// inference: outputs (FWD_OUTPUTS: raw network outputs o, 4 x n) or the
/// surrogate solve (FWD_SOLVE: net updates 4 x n, speed, used flag per edge)
template <int MODE>
__global__ void __launch_bounds__(128) forwardKernel(const uint8_t *image, EdgeBatch in, float *out, float *speed,
                                                     uint8_t *used, long long ostride, int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ float sHb[3 * kHid];  // halved hidden-layer biases
    const int t = threadIdx.x;
    uint8_t *sW = smem, *sX0 = smem + kFwdX0, *sAct = smem + kFwdAct;
    stageImage(image, sW, sHb);
    if (t == 0) tc::mbarInit(&mbar, 1);
    if (t < 32) tc::tmemAlloc(&tslot, kFwdCols);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tm = tslot;
    const float *bias = reinterpret_cast<const float *>(sW + pBias);
    uint8_t *const act[3] = {sAct, sAct, sAct};
    const uint32_t zc[3] = {0, 0, 0};
    uint32_t phase = 0;
    bool ok = true;
    const int ntiles = (in.count + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * kTile + t;
        const bool valid = i < in.count;
        float q[6] = {1.f, 1.f, 0.f, 0.f, 0.f, 0.f};
        long long e = 0;
        if (valid) {
            e = in.index(i);
#pragma unroll
            for (int k = 0; k < 6; k++) q[k] = __ldg(in.v + k * in.stride + e);
        }
        EdgeFeat f;
        edgeFeatures(q[0], q[1], q[2], q[3], q[4], q[5], f);
        storeX0(sX0, t, f.x);
        if (!(ok = forwardTile(tm, sW, sHb, sX0, act, zc, 0, &mbar, phase))) break;
        float v[16];
        tc::load16(tm, 0, v);
        float o[4];
#pragma unroll
        for (int k = 0; k < 4; k++) o[k] = v[k] + bias[3 * kHid + k];
        if (!valid) continue;
        if (MODE == FWD_OUTPUTS) {
#pragma unroll
            for (int k = 0; k < 4; k++) out[k * ostride + i] = o[k];
        } else {
            Waves w;
            surrogateWaves(o, f, w);
            float u[4], s;
            const bool use = surrogateGate(f, w);
            if (use) {
#pragma unroll
                for (int k = 0; k < 4; k++) u[k] = w.U[k];
                s = fmaxf(fabsf(w.s1), fabsf(w.s2));
            } else {
                edgeAugRie(q[0], q[1], q[2], q[3], q[4], q[5], u[0], u[1], u[2], u[3], s);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) out[k * ostride + i] = u[k];
            speed[i] = s;
            used[i] = use ? 1 : 0;
        }
    }
    if (!ok) {
        if (t == 0) atomicOr(err, 1);
        tc::mbarWait(&mbar, phase);  // bounded: let an MMA still in flight finish before the columns go
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t < 32) tc::tmemFree(tm, kFwdCols);
}

/// training: forward, loss and backward over the batch's tiles; each CTA
/// accumulates its weight and bias gradients in TMEM and writes them, with
/// its loss sum, to partials[blockIdx.x]
__global__ void __launch_bounds__(128, 1) trainKernel(const uint8_t *image, EdgeBatch in, float invN, float *partials,
                                                      int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ float sHb[3 * kHid];  // halved hidden-layer biases
    __shared__ float warpLoss[4];
    const int t = threadIdx.x;
    uint8_t *sW = smem, *sOnes = smem + kTrOnes, *sX0 = smem + kTrX0, *sDZ4 = smem + kTrDZ4, *sDZ = smem + kTrDZ;
    uint8_t *const act[3] = {smem + kTrA1, smem + kTrA2, smem + kTrA3};
    stageImage(image, sW, sHb);
    for (int i = t; i < kOnesBytes / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sOnes)[i] = 0x3F803F80u;  // BF16 1.0
    for (int i = t; i < (kTrEnd - kTrDZ4) / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sDZ4)[i] = 0u;
    if (t == 0) tc::mbarInit(&mbar, 1);
    if (t < 32) tc::tmemAlloc(&tslot, kTrCols);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tm = tslot;
    const float *bias = reinterpret_cast<const float *>(sW + pBias);
    const uint32_t zc[3] = {cZ1, cZ2, cZ3};
    uint32_t phase = 0;
    bool ok = true, first = true;
    float lossSum = 0.f;
    const int ntiles = (in.count + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * kTile + t;
        const bool valid = i < in.count;
        float q[6] = {1.f, 1.f, 0.f, 0.f, 0.f, 0.f}, T[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid) {
            const long long e = in.index(i);
#pragma unroll
            for (int k = 0; k < 6; k++) q[k] = __ldg(in.v + k * in.stride + e);
#pragma unroll
            for (int k = 0; k < 4; k++) T[k] = __ldg(in.targets + k * in.stride + e);
        }
        EdgeFeat f;
        edgeFeatures(q[0], q[1], q[2], q[3], q[4], q[5], f);
        storeX0(sX0, t, f.x);
        if (!(ok = forwardTile(tm, sW, sHb, sX0, act, zc, cO, &mbar, phase))) break;
        // loss and dLoss/dO
        {
            float v[16];
            tc::load16(tm + cO, 0, v);
            float o[4], dO[4];
#pragma unroll
            for (int k = 0; k < 4; k++) o[k] = v[k] + bias[3 * kHid + k];
            lossSum += edgeLoss(o, f, T, invN, valid, dO);
            storeDZ4(sDZ4, t, dO);
        }
        // layer 4: dA3 = dZ4 W4; gW4^T += A3^T dZ4; db4 += dZ4^T 1
        publishToMma();
        if (t == 0) {
            tc::mma(tm + cDA, tc::smemDesc(sDZ4, 0, kOutPad), tc::smemDescMN(sW + pW4, 0, kHid),
                    tc::idescBf16(128, kHid, false, true), false);
#pragma unroll
            for (int kk = 0; kk < kTile / 16; kk++) {
                const bool acc = !(first && kk == 0);
                tc::mma(tm + cGW4, tc::smemDescMN(act[2], kk * 16, kHid), tc::smemDescMN(sDZ4, kk * 16, kOutPad),
                        tc::idescBf16(128, kOutPad, true, true), acc);
                tc::mma(tm + cDB4, tc::smemDescMN(sDZ4, kk * 16, kOutPad), tc::smemDesc(sOnes, kk * 16, kTile),
                        tc::idescBf16(128, 16, true, false), acc);
            }
            tc::commit(&mbar);
        }
        if (!(ok = awaitMma(&mbar, phase))) break;
        // layers 3, 2, 1: dZ_l = dA_l * silu'(Z_l); dA_{l-1} = dZ_l W_l; gW_l += dZ_l^T A_{l-1}; db_l += dZ_l^T 1
        const int pw[3] = {pW1, pW2, pW3};
        const uint32_t cgw[3] = {cGW1, cGW2, cGW3}, cdb[3] = {cDB1, cDB2, cDB3};
#pragma unroll
        for (int l = 2; l >= 0; l--) {
            epilogueDsilu(tm + cDA, tm + zc[l], bias + kHid * l, sDZ, t);
            publishToMma();
            if (t == 0) {
                if (l > 0) {
#pragma unroll
                    for (int kk = 0; kk < kHid / 16; kk++)
                        tc::mma(tm + cDA, tc::smemDesc(sDZ, kk * 16, kHid), tc::smemDescMN(sW + pw[l], kk * 16, kHid),
                                tc::idescBf16(128, kHid, false, true), kk > 0);
                }
                const uint8_t *prev = l > 0 ? act[l - 1] : sX0;
                const int pwid = l > 0 ? kHid : kInPad;
#pragma unroll
                for (int kk = 0; kk < kTile / 16; kk++) {
                    const bool acc = !(first && kk == 0);
                    tc::mma(tm + cgw[l], tc::smemDescMN(sDZ, kk * 16, kHid), tc::smemDescMN(prev, kk * 16, pwid),
                            tc::idescBf16(128, pwid, true, true), acc);
                    tc::mma(tm + cdb[l], tc::smemDescMN(sDZ, kk * 16, kHid), tc::smemDesc(sOnes, kk * 16, kTile),
                            tc::idescBf16(128, 16, true, false), acc);
                }
                tc::commit(&mbar);
            }
            if (!(ok = awaitMma(&mbar, phase))) break;
        }
        if (!ok) break;
        first = false;
    }
    // per-CTA partial gradients: rows 0..63 of the accumulators live in the lanes of warps 0 and 1
    float *P = partials + (long long)blockIdx.x * kPartStride;
    if (ok && t < 64) {
        float v[16];
        if (first) {
            for (int k = 0; k < 16; k++) v[k] = 0.f;
        }
        if (!first) tc::load16(tm + cGW1, 0, v);
        for (int k = 0; k < kIn; k++) P[oW1 + t * kIn + k] = v[k];
        for (int l = 0; l < 2; l++) {
            const uint32_t col = l == 0 ? cGW2 : cGW3;
            const int off = l == 0 ? oW2 : oW3;
            for (int c = 0; c < kHid; c += 16) {
                if (!first) tc::load16(tm + col, c, v);
                for (int k = 0; k < 16; k++) P[off + t * kHid + c + k] = v[k];
            }
        }
        if (!first) tc::load16(tm + cGW4, 0, v);
        for (int k = 0; k < kOut; k++) P[oW4 + k * kHid + t] = v[k];
        const uint32_t cdb[4] = {cDB1, cDB2, cDB3, cDB4};
        const int odb[4] = {oB1, oB2, oB3, oB4};
        for (int l = 0; l < 4; l++) {
            if (!first) tc::load16(tm + cdb[l], 0, v);
            if (l < 3 || t < kOut) P[odb[l] + t] = v[0];
        }
    }
    // loss: fixed-order reduction
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, m);
    if ((t & 31) == 0) warpLoss[t >> 5] = lossSum;
    if (!ok) {
        if (t == 0) atomicOr(err, 1);
        tc::mbarWait(&mbar, phase);  // bounded
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t == 0) P[kNParams] = ((warpLoss[0] + warpLoss[1]) + warpLoss[2]) + warpLoss[3];
    if (t < 32) tc::tmemFree(tm, kTrCols);
}

/// sum of the per-CTA partials (fixed order); optional Adam step (Kingma & Ba
/// 2015) on the FP32 master parameters
__global__ void reduceAdamKernel(const float *partials, int nparts, float *grad, float *lossOut, float *p, float *m,
                                 float *v, float lr, float beta1, float beta2, float eps, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > kNParams) return;
    float g = 0.f;
    for (int c = 0; c < nparts; c++) g += partials[(long long)c * kPartStride + i];
    if (i == kNParams) {
        if (lossOut) *lossOut = g;
        return;
    }
    if (grad) grad[i] = g;
    if (lr > 0.f) {
        const float mi = fmaf(beta1, m[i], (1.f - beta1) * g);
        const float vi = fmaf(beta2, v[i], (1.f - beta2) * g * g);
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

/// FP32 master parameters -> packed image (BF16 weights in the core layout, FP32 biases)
__global__ void packKernel(const float *p, uint8_t *image) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int n1 = kHid * kInPad, n2 = kHid * kHid, n4 = kOutPad * kHid;
    if (i < n1) {
        const int r = i / kInPad, k = i % kInPad;
        *reinterpret_cast<__nv_bfloat16 *>(image + pW1 + tc::coreOffset(r, k, kInPad)) =
            __float2bfloat16_rn(k < kIn ? p[oW1 + r * kIn + k] : 0.f);
    } else if (i < n1 + 2 * n2) {
        const int j = i - n1, l = j / n2, r = (j % n2) / kHid, k = j % kHid;
        *reinterpret_cast<__nv_bfloat16 *>(image + (l ? pW3 : pW2) + tc::coreOffset(r, k, kHid)) =
            __float2bfloat16_rn(p[(l ? oW3 : oW2) + r * kHid + k]);
    } else if (i < n1 + 2 * n2 + n4) {
        const int j = i - n1 - 2 * n2, r = j / kHid, k = j % kHid;
        *reinterpret_cast<__nv_bfloat16 *>(image + pW4 + tc::coreOffset(r, k, kHid)) =
            __float2bfloat16_rn(r < kOut ? p[oW4 + r * kHid + k] : 0.f);
    } else if (i < n1 + 2 * n2 + n4 + kBiasFloats) {
        const int j = i - n1 - 2 * n2 - n4;
        float b = 0.f;
        if (j < kHid) b = p[oB1 + j];
        else if (j < 2 * kHid) b = p[oB2 + j - kHid];
        else if (j < 3 * kHid) b = p[oB3 + j - 2 * kHid];
        else if (j < 3 * kHid + kOut) b = p[oB4 + j - 3 * kHid];
        reinterpret_cast<float *>(image + pBias)[j] = b;
    }
}
constexpr int kPackThreads = kHid * kInPad + 2 * kHid * kHid + kOutPad * kHid + kBiasFloats;

// ---------------------------------------------------------------------------
// descriptor self-checks (one CTA): the operand readings the kernels use
// ---------------------------------------------------------------------------
enum CheckMode { CHECK_KMAJOR = 0, CHECK_WGRAD = 1, CHECK_DGRAD = 2 };

/// CHECK_KMAJOR: D[128 x w2] = X[128 x w1] Y[w2 x w1]^T (both K-major)
/// CHECK_WGRAD:  D[w1 x w2] = X[128 x w1]^T Y[128 x w2] (both read MN-major, K = 128 rows)
/// CHECK_DGRAD:  D[128 x w2] = X[128 x w1] Y[w1 x w2] (Y read MN-major)
__global__ void __launch_bounds__(128) gemmCheckKernel(int mode, const __nv_bfloat16 *X, const __nv_bfloat16 *Y,
                                                       float *D, int w1, int w2, int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x;
    const int yRows = mode == CHECK_KMAJOR ? w2 : (mode == CHECK_WGRAD ? 128 : w1);
    const int yCols = mode == CHECK_KMAJOR ? w1 : w2;
    uint8_t *sX = smem, *sY = smem + 128 * w1 * 2 + 2048;  // 2 KB guard for the padded-row over-read
    for (int i = t; i < (128 * w1 * 2 + 2048) / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(smem)[i] = 0u;
    __syncthreads();
    for (int i = t; i < 128 * w1; i += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sX + tc::coreOffset(i / w1, i % w1, w1)) = X[i];
    for (int i = t; i < yRows * yCols; i += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sY + tc::coreOffset(i / yCols, i % yCols, yCols)) = Y[i];
    if (t == 0) tc::mbarInit(&mbar, 1);
    if (t < 32) tc::tmemAlloc(&tslot, 128);
    tc::fenceSmemForMma();
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t taddr = tslot;
    if (t == 0) {
        if (mode == CHECK_KMAJOR) {
            for (int kk = 0; kk < w1 / 16; kk++)
                tc::mma(taddr, tc::smemDesc(sX, kk * 16, w1), tc::smemDesc(sY, kk * 16, w1), tc::idescBf16(128, w2), kk > 0);
        } else if (mode == CHECK_WGRAD) {
            for (int kk = 0; kk < 128 / 16; kk++)
                tc::mma(taddr, tc::smemDescMN(sX, kk * 16, w1), tc::smemDescMN(sY, kk * 16, w2),
                        tc::idescBf16(128, w2, true, true), kk > 0);
        } else {
            for (int kk = 0; kk < w1 / 16; kk++)
                tc::mma(taddr, tc::smemDesc(sX, kk * 16, w1), tc::smemDescMN(sY, kk * 16, w2),
                        tc::idescBf16(128, w2, false, true), kk > 0);
        }
        tc::commit(&mbar);
    }
    const bool ok = __syncthreads_and(tc::mbarWait(&mbar, 0));
    tc::fenceAfterSync();
    if (ok) {
        for (int c = 0; c < w2; c += 16) {
            float v[16];
            tc::load16(taddr, c, v);
            for (int j = 0; j < 16; j++) D[t * w2 + c + j] = v[j];
        }
    } else {
        if (t == 0) atomicOr(err, 1);
        tc::mbarWait(&mbar, 0);
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t < 32) tc::tmemFree(taddr, 128);
}


// ---------------------------------------------------------------------------
// surrogate step of a domain: edge pass, dt, cell update, finish
// ---------------------------------------------------------------------------
/// the six edge inputs of edge (tile, t) in the current buffer; false past the tile's end
__device__ __forceinline__ bool loadDomainEdge(const DomainDev &d, const EdgeTile &T, const BlockDesc &B, int cur, int t,
                                               float q[6], long long &oL) {
    const long long P = B.pitch;
    oL = B.base + (long long)T.col * P + (T.j0 + t);
    if (t >= T.count) return false;
    const long long oR = T.dir ? oL + 1 : oL + P;
    const float *H = pick(d.h, cur);
    const float *N = T.dir ? pick(d.hv, cur) : pick(d.hu, cur);
    q[0] = H[oL];
    q[1] = H[oR];
    q[2] = N[oL];
    q[3] = N[oR];
    q[4] = d.b[oL];
    q[5] = d.b[oR];
    return true;
}

/// the CTA's running max wave speed goes to its group
__device__ __forceinline__ void flushSpeed(const DomainDev &d, int group, float &smax, float *sMax) {
    float v = smax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = vmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sMax[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        const float m = vmax(vmax(sMax[0], sMax[1]), vmax(sMax[2], sMax[3]));
        atomicMax(&d.groups[group].speedBits, __float_as_uint(m));
    }
    __syncthreads();
    smax = 0.f;
}

/// edge pass over a contiguous range of tiles per CTA (so the group changes
/// rarely within a CTA).  SURR: surrogate with the gate, else the augmented
/// solver on every edge (the default step of augmented-solver domains).
/// Groups whose time reached their target (or that sit the step out) are
/// skipped, in this and the following kernels of the step.
template <bool SURR>
__global__ void __launch_bounds__(128) surrogateEdgeKernel(const DomainDev d, const uint8_t *image, const EdgeTile *tiles,
                                                           int ntiles, EdgeUpdates u, unsigned long long *usedCount,
                                                           int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ float sHb[3 * kHid];  // halved hidden-layer biases
    __shared__ float sMax[4];
    const int t = threadIdx.x;
    uint8_t *sW = smem, *sX0 = smem + kFwdX0, *sAct = smem + kFwdAct;
    uint32_t tm = 0;
    if (SURR) {
        stageImage(image, sW, sHb);
        if (t == 0) tc::mbarInit(&mbar, 1);
        if (t < 32) tc::tmemAlloc(&tslot, kFwdCols);
        tc::fenceBeforeSync();
        __syncthreads();
        tc::fenceAfterSync();
        tm = tslot;
    }
    const float *bias = reinterpret_cast<const float *>(sW + pBias);
    uint8_t *const act[3] = {sAct, sAct, sAct};
    const uint32_t zc[3] = {0, 0, 0};
    uint32_t phase = 0;
    bool ok = true;
    float smax = 0.f;
    unsigned usedLocal = 0;
    const int first = int((long long)ntiles * blockIdx.x / gridDim.x);
    const int last = int((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
    int group = -1;
    for (int tile = first; tile < last; tile++) {
        const EdgeTile T = tiles[tile];
        const BlockDesc &B = d.blocks[T.block];
        if (B.group != group) {
            if (group >= 0) flushSpeed(d, group, smax, sMax);
            group = B.group;
        }
        if (!groupActive(d.groups + group)) continue;  // the group reached its target (CTA-uniform)
        const int cur = d.groups[group].cur;
        float q[6] = {1.f, 1.f, 0.f, 0.f, 0.f, 0.f};
        long long oL;
        const bool valid = loadDomainEdge(d, T, B, cur, t, q, oL);
        float upd[4], s = 0.f;
        bool use = false;
        if (SURR) {
            EdgeFeat f;
            edgeFeatures(q[0], q[1], q[2], q[3], q[4], q[5], f);
            storeX0(sX0, t, f.x);
            if (!(ok = forwardTile(tm, sW, sHb, sX0, act, zc, 0, &mbar, phase))) break;
            float v[16];
            tc::load16(tm, 0, v);
            float o[4];
#pragma unroll
            for (int k = 0; k < 4; k++) o[k] = v[k] + bias[3 * kHid + k];
            Waves w;
            surrogateWaves(o, f, w);
            use = valid && surrogateGate(f, w);
            if (use) {
#pragma unroll
                for (int k = 0; k < 4; k++) upd[k] = w.U[k];
                s = fmaxf(fabsf(w.s1), fabsf(w.s2));
            }
        }
        if (valid) {
            if (!use) edgeAugRie(q[0], q[1], q[2], q[3], q[4], q[5], upd[0], upd[1], upd[2], upd[3], s);
            float *const *dst = T.dir ? u.y : u.x;
#pragma unroll
            for (int k = 0; k < 4; k++) dst[k][oL] = upd[k];
            smax = vmax(smax, s);
            usedLocal += use ? 1u : 0u;
        }
    }
    if (ok && group >= 0) flushSpeed(d, group, smax, sMax);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) usedLocal += __shfl_xor_sync(0xffffffffu, usedLocal, o);
    if ((t & 31) == 0 && usedLocal) atomicAdd(usedCount, (unsigned long long)usedLocal);
    if (SURR) {
        if (!ok) {
            if (t == 0) atomicOr(err, 1);
            tc::mbarWait(&mbar, phase);  // bounded
        }
        tc::fenceBeforeSync();
        __syncthreads();
        if (t < 32) tc::tmemFree(tm, kFwdCols);
    }
}

/// maxTimestep of every group from the edge pass's max wave speed
/// (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456)
__global__ void surrogateDtKernel(const DomainDev d, int ngroups) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    GroupState *G = d.groups + g;
    if (!groupActive(G)) return;
    const float s = __uint_as_float(G->speedBits);
    const BlockDesc &F = d.blocks[G->firstBlock];
    G->speed = s;
    G->dt = timestepFromSpeed(s, F.dx, F.dy, SEM_UNSPLIT);
    if (!(s == s)) G->status |= 1;
    G->speedBits = 0u;
}

/// the unsplit cell update (src/blocks/SWE_DimensionalSplittingMpi.cpp:458-492)
/// from the stored net updates: Q^{n+1} of interior cell (i, j) into the other buffer
__global__ void surrogateApplyKernel(const DomainDev d, EdgeUpdates u) {
    const BlockDesc B = d.blocks[blockIdx.y];
    GroupState *G = d.groups + B.group;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)B.nx * B.ny || !groupActive(G)) return;
    const int i = int(idx / B.ny) + 1, j = int(idx % B.ny) + 1;
    const int cur = G->cur;
    const float dt = G->dt;
    const float dtdx = dt / B.dx, dtdy = dt / B.dy;
    const long long P = B.pitch;
    const long long o = B.base + (long long)i * P + j;
    const float sxH = u.x[1][o - P] + u.x[0][o];
    const float sxHU = u.x[3][o - P] + u.x[2][o];
    const float syH = u.y[1][o - 1] + u.y[0][o];
    const float syHV = u.y[3][o - 1] + u.y[2][o];
    float hn = pick(d.h, cur)[o] - (dtdx * sxH + dtdy * syH);
    float hun = pick(d.hu, cur)[o] - dtdx * sxHU;
    float hvn = pick(d.hv, cur)[o] - dtdy * syHV;
    if (hn < 0.f) {
        hn = 0.f; hun = 0.f; hvn = 0.f;
    } else if (hn < 0.1f) {
        hun = 0.f; hvn = 0.f;
    }
    pick(d.h, cur ^ 1)[o] = hn;
    pick(d.hu, cur ^ 1)[o] = hun;
    pick(d.hv, cur ^ 1)[o] = hvn;
    if (!(fabsf(hn) <= FLT_MAX)) atomicOr(&G->status, 2);
}

__global__ void surrogateFinishKernel(const DomainDev d, int ngroups) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    GroupState *G = d.groups + g;
    if (!groupActive(G)) return;
    G->time = G->time + G->dt;
    G->steps = G->steps + 1;
    G->cur = G->cur ^ 1;
    G->ghostsAhead = 1;  // the next ghost kernel (mode 2) fills the new buffer's ring; the old ring stays readable
    G->boundsValid[0] = 0;
    G->boundsValid[1] = 0;
}

/// edge-state logger: inputs and augmented-solver net updates of every
/// stride-th edge into fixed slots (deterministic, whatever the launch shape)
__global__ void logEdgesKernel(const DomainDev d, const EdgeTile *tiles, int ntiles, int stride, float *slots,
                               long long nslots) {
    const int tile = blockIdx.x;
    if (tile >= ntiles) return;
    const long long e = (long long)tile * kTile + threadIdx.x;
    if (e % stride) return;
    const long long slot = e / stride;
    if (slot >= nslots) return;
    const EdgeTile T = tiles[tile];
    const BlockDesc &B = d.blocks[T.block];
    const int cur = d.groups[B.group].cur;
    float q[6];
    long long oL;
    float wet = 0.f;
    float r[4] = {0.f, 0.f, 0.f, 0.f};
    if (loadDomainEdge(d, T, B, cur, threadIdx.x, q, oL)) {
        float s;
        edgeAugRie(q[0], q[1], q[2], q[3], q[4], q[5], r[0], r[1], r[2], r[3], s);
        wet = (q[0] >= kWet && q[1] >= kWet) ? 1.f : 0.f;
    } else {
        for (int k = 0; k < 6; k++) q[k] = 0.f;
    }
    for (int k = 0; k < 6; k++) slots[k * nslots + slot] = q[k];
    for (int k = 0; k < 4; k++) slots[(6 + k) * nslots + slot] = r[k];
    slots[10 * nslots + slot] = wet;
}

} // namespace mlp
} // namespace swegb

using namespace swegb;
using namespace swegb::mlp;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

thread_local std::string g_mlpError;

int mlpFail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_mlpError = buf;
    return code;
}

#define MLP_TRY(call)                                                                                      \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return mlpFail(SWE_GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
/// uniform in [0, 1) with 24 random bits
float uniform01(uint64_t &s) { return float(splitmix(s) >> 40) * 0x1p-24f; }

} // namespace

struct swe_mlp {
    int device = 0;
    int sms = 0;
    int fwdBlocksPerSm = 1;
    float *p = nullptr, *m = nullptr, *v = nullptr;
    uint8_t *image = nullptr;
    float *partials = nullptr;  // [sms][kPartStride]
    float *grad = nullptr;      // reduced gradient and loss
    float *losses = nullptr;    // one loss sum per training batch
    size_t lossCap = 0;
    int *err = nullptr;
    long long adamSteps = 0;
    float *buf = nullptr;  // host-API staging
    size_t bufFloats = 0;
    int *perm = nullptr;
    size_t permCap = 0;

    int reserve(size_t floats) {
        if (floats <= bufFloats) return SWE_GPU_OK;
        cudaFree(buf);
        buf = nullptr;
        bufFloats = 0;
        MLP_TRY(cudaMalloc(&buf, floats * sizeof(float)));
        bufFloats = floats;
        return SWE_GPU_OK;
    }
    int checkErr(const char *what) {
        int h = 0;
        MLP_TRY(cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) {
            cudaMemset(err, 0, sizeof(int));
            return mlpFail(SWE_GPU_ERR_DEVICE, "%s: a tensor-core wait ran out of its iteration limit", what);
        }
        return SWE_GPU_OK;
    }
    int pack() {
        packKernel<<<(kPackThreads + 255) / 256, 256>>>(p, image);
        MLP_TRY(cudaGetLastError());
        return SWE_GPU_OK;
    }
    /// gradient (and optionally an Adam step) of the batch; loss sum to *lossDst (device)
    int trainBatch(const EdgeBatch &b, float invN, float lr, float *gradDst, float *lossDst) {
        const int ntiles = (b.count + kTile - 1) / kTile;
        const int grid = std::max(1, std::min(ntiles, sms));
        trainKernel<<<grid, 128, kTrSmem>>>(image, b, invN, partials, err);
        MLP_TRY(cudaGetLastError());
        float bc1 = 1.f, bc2 = 1.f;
        if (lr > 0.f) {
            adamSteps++;
            bc1 = 1.f - std::pow(0.9f, float(adamSteps));
            bc2 = 1.f - std::pow(0.999f, float(adamSteps));
        }
        reduceAdamKernel<<<(kNParams + 1 + 255) / 256, 256>>>(partials, grid, gradDst, lossDst, p, m, v, lr, 0.9f, 0.999f,
                                                               1e-8f, bc1, bc2);
        MLP_TRY(cudaGetLastError());
        if (lr > 0.f) return pack();
        return SWE_GPU_OK;
    }
};

namespace {

int checkEdges(swe_mlp *m, int n, const float *edges) {
    if (!m) return mlpFail(SWE_GPU_ERR_INVALID, "null handle");
    if (n < 0) return mlpFail(SWE_GPU_ERR_INVALID, "negative edge count");
    if (n > 0 && !edges) return mlpFail(SWE_GPU_ERR_INVALID, "null edge array");
    return SWE_GPU_OK;
}

void destroy(swe_mlp *m) {
    if (!m) return;
    cudaFree(m->p);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->image);
    cudaFree(m->partials);
    cudaFree(m->grad);
    cudaFree(m->losses);
    cudaFree(m->err);
    cudaFree(m->buf);
    cudaFree(m->perm);
    delete m;
}

} // namespace

extern "C" {

const char *swe_mlp_last_error(void) { return g_mlpError.c_str(); }

int swe_mlp_param_count(void) { return kNParams; }

int swe_mlp_launch_shape(swe_mlp *m, int *sms, int *forward_ctas_per_sm) {
    if (!m || !sms || !forward_ctas_per_sm) return mlpFail(SWE_GPU_ERR_INVALID, "null argument");
    *sms = m->sms;
    *forward_ctas_per_sm = m->fwdBlocksPerSm;
    return SWE_GPU_OK;
}

int swe_mlp_create(unsigned long long seed, swe_mlp **out) {
    if (!out) return mlpFail(SWE_GPU_ERR_INVALID, "null output pointer");
    *out = nullptr;
    swe_mlp *m = new swe_mlp();
    auto bail = [&](int rc) {
        destroy(m);
        return rc;
    };
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device);
    // shared memory: the largest carveout, so several forward CTAs share an SM
    auto smemAttr = [&](const void *f, int bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    };
    smemAttr((const void *)trainKernel, kTrSmem);
    smemAttr((const void *)forwardKernel<FWD_OUTPUTS>, kFwdSmem);
    smemAttr((const void *)forwardKernel<FWD_SOLVE>, kFwdSmem);
    smemAttr((const void *)surrogateEdgeKernel<true>, kFwdSmem);
    // resident inference CTAs per SM from their shared-memory footprint (the
    // CTA's static and dynamic shared memory plus the 1 KB the SM reserves per
    // CTA) and registers; TMEM: every resident CTA holds kFwdCols of the SM's
    // 512 columns.  Extra CTAs of a grid only queue.
    int smemSm = 0, regsSm = 0;
    cudaFuncAttributes fa{}, ea{};
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smemSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, m->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&regsSm, cudaDevAttrMaxRegistersPerMultiprocessor, m->device);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, forwardKernel<FWD_SOLVE>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&ea, surrogateEdgeKernel<true>);
    if (e != cudaSuccess) return bail(mlpFail(SWE_GPU_ERR_CUDA, "create: %s", cudaGetErrorString(e)));
    const int staticSmem = int(std::max(fa.sharedSizeBytes, ea.sharedSizeBytes));
    const int regs = std::max(fa.numRegs, ea.numRegs);
    const int bySmem = smemSm / (kFwdSmem + staticSmem + 1024);
    const int byRegs = regs > 0 ? regsSm / (regs * 128) : 8;
    m->fwdBlocksPerSm = std::max(1, std::min(std::min(bySmem, byRegs), int(512 / kFwdCols)));
    const size_t pb = kNParams * sizeof(float);
    e = cudaMalloc(&m->p, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->m, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->v, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->image, kImageSmem);
    if (e == cudaSuccess) e = cudaMalloc(&m->partials, size_t(m->sms) * kPartStride * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->grad, (kNParams + 4) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(m->image, 0, kImageSmem);
    if (e != cudaSuccess) return bail(mlpFail(SWE_GPU_ERR_CUDA, "create: %s", cudaGetErrorString(e)));
    // Glorot-uniform weights, zero biases, zero last layer: the untrained
    // surrogate is the f-wave solver with Roe speeds
    std::vector<float> p(kNParams, 0.f);
    uint64_t s = seed;
    auto glorot = [&](int off, int rows, int cols) {
        const float lim = std::sqrt(6.f / float(rows + cols));
        for (int i = 0; i < rows * cols; i++) p[off + i] = (2.f * uniform01(s) - 1.f) * lim;
    };
    glorot(oW1, kHid, kIn);
    glorot(oW2, kHid, kHid);
    glorot(oW3, kHid, kHid);
    int rc = swe_mlp_set_params(m, p.data());
    if (rc) return bail(rc);
    *out = m;
    return SWE_GPU_OK;
}

void swe_mlp_destroy(swe_mlp *m) { destroy(m); }

int swe_mlp_get_params(swe_mlp *m, float *params) {
    if (!m || !params) return mlpFail(SWE_GPU_ERR_INVALID, "null argument");
    MLP_TRY(cudaMemcpy(params, m->p, kNParams * sizeof(float), cudaMemcpyDeviceToHost));
    return SWE_GPU_OK;
}

int swe_mlp_set_params(swe_mlp *m, const float *params) {
    if (!m || !params) return mlpFail(SWE_GPU_ERR_INVALID, "null argument");
    MLP_TRY(cudaMemcpy(m->p, params, kNParams * sizeof(float), cudaMemcpyHostToDevice));
    MLP_TRY(cudaMemset(m->m, 0, kNParams * sizeof(float)));
    MLP_TRY(cudaMemset(m->v, 0, kNParams * sizeof(float)));
    m->adamSteps = 0;
    int rc = m->pack();
    if (rc) return rc;
    MLP_TRY(cudaDeviceSynchronize());
    return SWE_GPU_OK;
}

int swe_mlp_forward(swe_mlp *m, int n, const float *edges, float *out) {
    int rc = checkEdges(m, n, edges);
    if (rc) return rc;
    if (n > 0 && !out) return mlpFail(SWE_GPU_ERR_INVALID, "null output array");
    if (n == 0) return SWE_GPU_OK;
    if ((rc = m->reserve(size_t(10) * n))) return rc;
    MLP_TRY(cudaMemcpy(m->buf, edges, size_t(6) * n * sizeof(float), cudaMemcpyHostToDevice));
    float *dOut = m->buf + size_t(6) * n;
    EdgeBatch b{m->buf, nullptr, nullptr, n, 0, n};
    const int ntiles = (n + kTile - 1) / kTile;
    const int grid = std::min(ntiles, m->sms * m->fwdBlocksPerSm);
    forwardKernel<FWD_OUTPUTS><<<grid, 128, kFwdSmem>>>(m->image, b, dOut, nullptr, nullptr, n, m->err);
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaMemcpy(out, dOut, size_t(4) * n * sizeof(float), cudaMemcpyDeviceToHost));
    return m->checkErr("forward");
}

int swe_mlp_solve(swe_mlp *m, int n, const float *edges, float *updates, float *speed, unsigned char *used) {
    int rc = checkEdges(m, n, edges);
    if (rc) return rc;
    if (n > 0 && (!updates || !speed || !used)) return mlpFail(SWE_GPU_ERR_INVALID, "null output array");
    if (n == 0) return SWE_GPU_OK;
    if ((rc = m->reserve(size_t(12) * n))) return rc;
    MLP_TRY(cudaMemcpy(m->buf, edges, size_t(6) * n * sizeof(float), cudaMemcpyHostToDevice));
    float *dU = m->buf + size_t(6) * n, *dS = dU + size_t(4) * n;
    uint8_t *dUsed = reinterpret_cast<uint8_t *>(dS + n);
    EdgeBatch b{m->buf, nullptr, nullptr, n, 0, n};
    const int ntiles = (n + kTile - 1) / kTile;
    const int grid = std::min(ntiles, m->sms * m->fwdBlocksPerSm);
    forwardKernel<FWD_SOLVE><<<grid, 128, kFwdSmem>>>(m->image, b, dU, dS, dUsed, n, m->err);
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaMemcpy(updates, dU, size_t(4) * n * sizeof(float), cudaMemcpyDeviceToHost));
    MLP_TRY(cudaMemcpy(speed, dS, size_t(n) * sizeof(float), cudaMemcpyDeviceToHost));
    MLP_TRY(cudaMemcpy(used, dUsed, size_t(n), cudaMemcpyDeviceToHost));
    return m->checkErr("solve");
}

int swe_mlp_loss_grad(swe_mlp *m, int n, const float *edges, const float *targets, float *loss, float *grad) {
    int rc = checkEdges(m, n, edges);
    if (rc) return rc;
    if (n < 1 || !targets || !loss || !grad) return mlpFail(SWE_GPU_ERR_INVALID, "need n >= 1 and all arrays");
    if ((rc = m->reserve(size_t(10) * n))) return rc;
    MLP_TRY(cudaMemcpy(m->buf, edges, size_t(6) * n * sizeof(float), cudaMemcpyHostToDevice));
    MLP_TRY(cudaMemcpy(m->buf + size_t(6) * n, targets, size_t(4) * n * sizeof(float), cudaMemcpyHostToDevice));
    EdgeBatch b{m->buf, m->buf + size_t(6) * n, nullptr, n, 0, n};
    if ((rc = m->trainBatch(b, 1.f / float(n), 0.f, m->grad, m->grad + kNParams))) return rc;
    MLP_TRY(cudaMemcpy(grad, m->grad, kNParams * sizeof(float), cudaMemcpyDeviceToHost));
    float sum = 0.f;
    MLP_TRY(cudaMemcpy(&sum, m->grad + kNParams, sizeof(float), cudaMemcpyDeviceToHost));
    *loss = sum / float(n);
    return m->checkErr("loss_grad");
}

int swe_mlp_train(swe_mlp *m, int n, const float *edges, const float *targets, int epochs, int batch, float lr,
                  unsigned long long seed, float *epochLoss) {
    int rc = checkEdges(m, n, edges);
    if (rc) return rc;
    if (n < 1 || !targets || epochs < 1 || batch < 1 || !(lr > 0.f))
        return mlpFail(SWE_GPU_ERR_INVALID, "need n, epochs, batch >= 1, lr > 0 and the target array");
    if ((rc = m->reserve(size_t(10) * n))) return rc;
    MLP_TRY(cudaMemcpy(m->buf, edges, size_t(6) * n * sizeof(float), cudaMemcpyHostToDevice));
    MLP_TRY(cudaMemcpy(m->buf + size_t(6) * n, targets, size_t(4) * n * sizeof(float), cudaMemcpyHostToDevice));
    if (size_t(n) > m->permCap) {
        cudaFree(m->perm);
        m->perm = nullptr;
        m->permCap = 0;
        MLP_TRY(cudaMalloc(&m->perm, size_t(n) * sizeof(int)));
        m->permCap = n;
    }
    const int nb = (n + batch - 1) / batch;
    if (size_t(nb) * epochs > m->lossCap) {
        cudaFree(m->losses);
        m->losses = nullptr;
        m->lossCap = 0;
        MLP_TRY(cudaMalloc(&m->losses, size_t(nb) * epochs * sizeof(float)));
        m->lossCap = size_t(nb) * epochs;
    }
    std::vector<int> perm(n);
    uint64_t s = seed;
    for (int ep = 0; ep < epochs; ep++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[int(splitmix(s) % uint64_t(i + 1))]);
        MLP_TRY(cudaMemcpy(m->perm, perm.data(), size_t(n) * sizeof(int), cudaMemcpyHostToDevice));
        for (int k = 0; k < nb; k++) {
            const int off = k * batch, cnt = std::min(batch, n - off);
            EdgeBatch b{m->buf, m->buf + size_t(6) * n, m->perm, n, off, cnt};
            if ((rc = m->trainBatch(b, 1.f / float(cnt), lr, nullptr, m->losses + size_t(ep) * nb + k))) return rc;
        }
    }
    std::vector<float> bl(size_t(nb) * epochs);
    MLP_TRY(cudaMemcpy(bl.data(), m->losses, bl.size() * sizeof(float), cudaMemcpyDeviceToHost));
    if (epochLoss) {
        for (int ep = 0; ep < epochs; ep++) {
            double sum = 0.0;
            for (int k = 0; k < nb; k++) sum += bl[size_t(ep) * nb + k];
            epochLoss[ep] = float(sum / double(n));
        }
    }
    return m->checkErr("train");
}

int swe_mlp_gemm_check(int mode, int w1, int w2, const float *x, const float *y, float *d) {
    if (!x || !y || !d) return mlpFail(SWE_GPU_ERR_INVALID, "null argument");
    const bool okw = (w1 == 16 || w1 == 32 || w1 == 64) && w2 >= 16 && w2 <= 128 && w2 % 16 == 0;
    if (mode < CHECK_KMAJOR || mode > CHECK_DGRAD || !okw)
        return mlpFail(SWE_GPU_ERR_INVALID, "mode 0..2, w1 in {16, 32, 64}, w2 16..128 in steps of 16");
    const int yRows = mode == CHECK_KMAJOR ? w2 : (mode == CHECK_WGRAD ? 128 : w1);
    const int yCols = mode == CHECK_KMAJOR ? w1 : w2;
    std::vector<__nv_bfloat16> hx(size_t(128) * w1), hy(size_t(yRows) * yCols);
    for (size_t i = 0; i < hx.size(); i++) hx[i] = __float2bfloat16_rn(x[i]);
    for (size_t i = 0; i < hy.size(); i++) hy[i] = __float2bfloat16_rn(y[i]);
    __nv_bfloat16 *dX = nullptr, *dY = nullptr;
    float *dD = nullptr;
    int *dErr = nullptr;
    auto release = [&]() {
        cudaFree(dX);
        cudaFree(dY);
        cudaFree(dD);
        cudaFree(dErr);
    };
    const size_t smem = size_t(128) * w1 * 2 + 2048 + size_t(yRows) * yCols * 2;
    cudaError_t e = cudaMalloc(&dX, hx.size() * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&dY, hy.size() * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&dD, sizeof(float) * 128 * w2);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dX, hx.data(), hx.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dY, hy.data(), hy.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gemmCheckKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess) {
        gemmCheckKernel<<<1, 128, smem>>>(mode, dX, dY, dD, w1, w2, dErr);
        e = cudaGetLastError();
    }
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(d, dD, sizeof(float) * 128 * w2, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&err, dErr, sizeof(int), cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return mlpFail(SWE_GPU_ERR_CUDA, "gemm check: %s", cudaGetErrorString(e));
    if (err) return mlpFail(SWE_GPU_ERR_DEVICE, "gemm check: the MMA did not complete in time");
    return SWE_GPU_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// launchers of the domain kernels (swe_mlp_launch.hpp)
// ---------------------------------------------------------------------------
namespace swegb {
namespace mlp {

cudaError_t launchSurrogateEdges(const DomainDev &d, const swe_mlp *m, const EdgeTile *tiles, int ntiles, EdgeUpdates u,
                                 unsigned long long *used, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (m) {
        const int grid = std::min(ntiles, m->sms * m->fwdBlocksPerSm);
        surrogateEdgeKernel<true><<<grid, 128, kFwdSmem, s>>>(d, m->image, tiles, ntiles, u, used, m->err);
    } else {
        // the augmented solver alone: as many resident CTAs as registers allow
        // (latency hiding for its long dependency chains), looked up once per device
        static int perSm[64] = {0}, smCount[64] = {0};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64) dev = 0;
        if (!perSm[dev]) {
            cudaDeviceGetAttribute(&smCount[dev], cudaDevAttrMultiProcessorCount, dev);
            int occ = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, surrogateEdgeKernel<false>, 128, 0);
            perSm[dev] = std::max(1, occ);
        }
        const int grid = std::min(ntiles, smCount[dev] * perSm[dev]);
        surrogateEdgeKernel<false><<<grid, 128, 0, s>>>(d, nullptr, tiles, ntiles, u, used, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launchSurrogateDt(const DomainDev &d, int ngroups, cudaStream_t s) {
    surrogateDtKernel<<<(ngroups + 127) / 128, 128, 0, s>>>(d, ngroups);
    return cudaGetLastError();
}

cudaError_t launchSurrogateApply(const DomainDev &d, EdgeUpdates u, int nblocks, long long maxCells, cudaStream_t s) {
    const dim3 grid(unsigned((maxCells + 255) / 256), unsigned(nblocks));
    surrogateApplyKernel<<<grid, 256, 0, s>>>(d, u);
    return cudaGetLastError();
}

cudaError_t launchSurrogateFinish(const DomainDev &d, int ngroups, cudaStream_t s) {
    surrogateFinishKernel<<<(ngroups + 127) / 128, 128, 0, s>>>(d, ngroups);
    return cudaGetLastError();
}

cudaError_t launchLogEdges(const DomainDev &d, const EdgeTile *tiles, int ntiles, int stride, float *slots,
                           long long nslots, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    logEdgesKernel<<<ntiles, kTile, 0, s>>>(d, tiles, ntiles, stride, slots, nslots);
    return cudaGetLastError();
}

int checkDeviceError(swe_mlp *m, const char *what) { return m ? m->checkErr(what) : SWE_GPU_OK; }
int deviceOf(const swe_mlp *m) { return m ? m->device : -1; }

} // namespace mlp
} // namespace swegb
