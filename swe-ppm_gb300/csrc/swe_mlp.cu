// MLP surrogate of the augmented Riemann solver on fifth-generation tensor
// cores (tcgen05): see swe_tc.cuh for the primitives.  This file holds the
// tensor-core GEMM self-check used by the tests.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "swe_tc.cuh"

using namespace swegb;

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

#define MLP_TRY(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return mlpFail(SWE_GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

/// one CTA of 128 threads: D[128 x N] = A[128 x K] * B[N x K]^T, BF16 in, FP32 out
__global__ void __launch_bounds__(128) gemmCheckKernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D, int N,
                                                       int K, int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    uint8_t *sA = smem, *sB = smem + 128 * K * 2;
    const int t = threadIdx.x;
    for (int i = t; i < 128 * K; i += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sA + tc::coreOffset(i / K, i % K, K)) = A[i];
    for (int i = t; i < N * K; i += blockDim.x)
        *reinterpret_cast<__nv_bfloat16 *>(sB + tc::coreOffset(i / K, i % K, K)) = B[i];
    if (t == 0) tc::mbarInit(&mbar, 1);
    if (t < 32) tc::tmemAlloc(&tslot, 128);
    tc::fenceSmemForMma();
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t taddr = tslot;
    if (t == 0) {
        for (int kk = 0; kk < K / 16; kk++)
            tc::mma(taddr, tc::smemDesc(sA, kk * 16, K), tc::smemDesc(sB, kk * 16, K), tc::idescBf16(128, N), kk > 0);
        tc::commit(&mbar);
    }
    const bool ok = __syncthreads_and(tc::mbarWait(&mbar, 0));
    tc::fenceAfterSync();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tc::load16(taddr, c, v);
            for (int j = 0; j < 16; j++) D[t * N + c + j] = v[j];
        }
    } else if (t == 0) {
        atomicOr(err, 1);
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t < 32) tc::tmemFree(taddr, 128);
}

} // namespace

extern "C" {

const char *swe_mlp_last_error(void) { return g_mlpError.c_str(); }

int swe_mlp_gemm_check(int n, int k, const float *a, const float *b, float *d) {
    if (!a || !b || !d) return mlpFail(SWE_GPU_ERR_INVALID, "null argument");
    if (n < 16 || n > 128 || n % 16 || k < 16 || k > 64 || k % 16)
        return mlpFail(SWE_GPU_ERR_INVALID, "n must be 16..128 and k 16..64, multiples of 16");
    std::vector<__nv_bfloat16> ha(size_t(128) * k), hb(size_t(n) * k);
    for (size_t i = 0; i < ha.size(); i++) ha[i] = __float2bfloat16_rn(a[i]);
    for (size_t i = 0; i < hb.size(); i++) hb[i] = __float2bfloat16_rn(b[i]);
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    int *dErr = nullptr;
    auto release = [&]() {
        cudaFree(dA);
        cudaFree(dB);
        cudaFree(dD);
        cudaFree(dErr);
    };
    cudaError_t e = cudaMalloc(&dA, ha.size() * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&dB, hb.size() * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&dD, sizeof(float) * 128 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dA, ha.data(), ha.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, hb.data(), hb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
    if (e == cudaSuccess) {
        gemmCheckKernel<<<1, 128, size_t(128 + n) * k * 2>>>(dA, dB, dD, n, k, dErr);
        e = cudaGetLastError();
    }
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(d, dD, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&err, dErr, sizeof(int), cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return mlpFail(SWE_GPU_ERR_CUDA, "gemm check: %s", cudaGetErrorString(e));
    if (err) return mlpFail(SWE_GPU_ERR_DEVICE, "gemm check: the MMA did not complete in time");
    return SWE_GPU_OK;
}

} // extern "C"
