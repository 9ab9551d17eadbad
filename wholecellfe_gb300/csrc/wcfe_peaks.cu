// wcfe_peaks.cu — the rates of the pipes the step's kernels are measured against, taken on
// the GPU that runs them, for the roofline denominators the driver's peak file does not
// hold:
//  - TF32 on the 5th-generation tensor cores: one CTA per SM issues tcgen05.mma kind::tf32
//    (M = 128, N = 256, K = 8, the shape of the LU's widest trailing update) back to back
//    from operands resident in shared memory into two TMEM accumulators, so no operand
//    traffic limits it;
//  - FP64 and FP32 fused multiply-add: every thread runs eight independent FMA chains.
// Every wait is bounded; a timeout is reported as a negative rate.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/wcfe.h"
#include "wcfe_tc.cuh"

namespace wcfe {
int set_error(const char* msg, int code);   // wcfe_engine.cu: the thread's wcfe_last_error message
namespace {

constexpr int kPkThreads = 128;
constexpr uint32_t kPkA = 128u * 128u;   // 128 rows x 32 fp32 (one swizzle atom column)
constexpr uint32_t kPkB = 256u * 128u;   // 256 rows x 32 fp32
// more than half of an SM's shared memory, so that each SM runs one CTA (and its 512 TMEM columns)
constexpr size_t kPkSmem = 120 * 1024;
constexpr long long kPkWait = 4000000000ll;   // SM clocks before the final wait gives up

__global__ void __launch_bounds__(kPkThreads, 1) k_peak_tf32(int iters, int* status) {
    extern __shared__ uint8_t pk_raw[];
    uint8_t* sm = pk_raw + ((1024u - (smem_addr(pk_raw) & 1023u)) & 1023u);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kPkA + kPkB);
    uint32_t* tbase_s = reinterpret_cast<uint32_t*>(bar + 1);
    // operands: small finite values (their bit layout does not change the work)
    float* f = reinterpret_cast<float*>(sm);
    for (uint32_t i = threadIdx.x; i < (kPkA + kPkB) / 4; i += kPkThreads) f[i] = 1.0f + 1e-3f * (float)(i & 255u);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    fence_proxy_async_smem();
    if (threadIdx.x < 32) {
        tc_alloc(tbase_s, 512);
        tc_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tbase_s;
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc_idesc_tf32(128, 256);
        const uint32_t sa = smem_addr(sm);
        const uint64_t da = tc_desc_k_sw128(sa), db = tc_desc_k_sw128(sa + kPkA);
        for (int it = 0; it < iters; ++it) {
            const uint32_t d = tbase + (uint32_t)((it & 1) * 256);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                tc_mma_tf32(d, da + 2u * (uint32_t)k, db + 2u * (uint32_t)k, idesc, (uint32_t)((it >> 1) | k));
        }
        tc_commit(bar);   // arrives once every MMA above has completed
        if (!mbar_wait_bounded(bar, 0u, kPkWait)) atomicExch(status, 1);
    }
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tc_dealloc(tbase, 512);
}

template <class T>
__global__ void __launch_bounds__(256) k_peak_fma(int iters, T* sink) {
    T a[8], b = (T)1.0000001, c = (T)1e-7;
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = (T)(threadIdx.x + j);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = a[j] * b + c;
    T s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == (T)-1.2345) sink[0] = s;   // keeps the chains alive; never true
}

}  // namespace
}  // namespace wcfe

extern "C" int wcfe_debug_pipe_rates(double* tf32_tflops, double* fp64_tflops, double* fp32_tflops) {
    using namespace wcfe;
    if (!tf32_tflops || !fp64_tflops || !fp32_tflops) return set_error("bad argument", WCFE_ERR_ARG);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return set_error("no CUDA device", WCFE_ERR_NODEVICE);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int* status = nullptr;
    double* sink = nullptr;
    int rc = WCFE_OK;
    auto timed = [&](auto launch, int reps) -> float {
        launch();   // warm-up
        cudaEventRecord(e0);
        for (int r = 0; r < reps; ++r) launch();
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms / reps;
    };
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
        cudaMalloc(&status, sizeof(int)) != cudaSuccess || cudaMalloc(&sink, sizeof(double)) != cudaSuccess ||
        cudaMemset(status, 0, sizeof(int)) != cudaSuccess ||
        cudaFuncSetAttribute((const void*)k_peak_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPkSmem) !=
            cudaSuccess) {
        cudaGetLastError();
        rc = set_error("pipe-rate set-up failed", WCFE_ERR_CUDA);
    }
    if (rc == WCFE_OK) {
        const int iters = 20000;
        const float ms = timed([&] { k_peak_tf32<<<sms, kPkThreads, kPkSmem>>>(iters, status); }, 5);
        int st = 0;
        cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
        const double flop = 2.0 * 128 * 256 * 8 * 4.0 * iters * sms;
        *tf32_tflops = st ? -1.0 : flop / (ms * 1e-3) / 1e12;
        const int fi = 4096, blocks = sms * 8;
        const float md = timed([&] { k_peak_fma<double><<<blocks, 256>>>(fi, sink); }, 3);
        *fp64_tflops = 2.0 * 8 * fi * (double)blocks * 256 / (md * 1e-3) / 1e12;
        const float mf = timed([&] { k_peak_fma<float><<<blocks, 256>>>(fi * 8, reinterpret_cast<float*>(sink)); }, 3);
        *fp32_tflops = 2.0 * 8 * (fi * 8.0) * (double)blocks * 256 / (mf * 1e-3) / 1e12;
        if (cudaGetLastError() != cudaSuccess) rc = set_error("pipe-rate kernels failed", WCFE_ERR_CUDA);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (status) cudaFree(status);
    if (sink) cudaFree(sink);
    return rc;
}
