// wcfe_noalloc.cu — the cell's total area and area-weighted centroid
// (calculateAreaTot, cellBP/UL_growth_explicit.cpp:1662-1688) for callers that
// cannot allocate device memory.
//
// The engine computes the same quantity inside its step with a per-cell block
// of partial sums that it allocates.  Some host codes may not allocate at all
// while they run: a solver that reserves all of its device memory up front and
// treats any later cudaMalloc as an error, or one that must not pay the
// implicit device synchronisation a cudaMalloc/cudaFree brings in the middle of
// its time loop.  For them, wcfe_area_tot_noalloc keeps its scratch in the
// file-scope array below instead.  Every GPU that loads this library holds
// the array (128 KiB) until the process exits.
//
// Contract:
//  - inputs and output are the caller's device memory: positions double[n][3],
//    triangles int32[t][3], the result double[4] = {area, cx, cy, cz};
//  - at most kNaMaxBlocks * kNaElems = 4,194,304 triangles (larger: WCFE_ERR_LIMIT,
//    nothing launched);
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current.  Make that first call
//    before any stream capture;
//  - all calls share the one array, and each call overwrites the slots it uses
//    before reading them.  Calls that overlap on the GPU (two streams, or two
//    host threads) race on it: serialise them.
//  - a triangle index outside [0, n) makes the result NaN;
//  - a CUDA error already pending on the calling thread when the call starts is
//    left in place (not cleared) and the call returns WCFE_ERR_CUDA without
//    launching, so the status this call returns is always about its own launches;
//  - the device address is kept for the life of the process: after a
//    cudaDeviceReset of a device this entry point must not be called on it again.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/wcfe.h"

namespace wcfe {
int set_error(const char* msg, int code);   // wcfe_engine.cu: the thread's wcfe_last_error message
}

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaElems = 1024;                 // triangles per block
constexpr int kNaMaxBlocks = 4096;             // 4096 x 1024 = 4,194,304 triangles
constexpr int kNaMaxDevices = 64;

// scratch: per-block partial sums {area, area*cx, area*cy, area*cz}
static __device__ __align__(256) double g_na_part[kNaMaxBlocks * 4];

std::mutex g_na_mu;
double* g_na_addr[kNaMaxDevices] = {};

__device__ __forceinline__ void warp_sum4(double v[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

__global__ void __launch_bounds__(kNaThreads) k_na_partials(const double* __restrict__ x, int nv,
                                                           const int* __restrict__ tri, int nt,
                                                           double* __restrict__ part) {
    __shared__ double red[4 * (kNaThreads / 32)];
    double acc[4] = {0, 0, 0, 0};
    const int e0 = blockIdx.x * kNaElems;
    const int e1 = min(nt, e0 + kNaElems);
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const int a = tri[3 * e], b = tri[3 * e + 1], c = tri[3 * e + 2];
        if (a < 0 || a >= nv || b < 0 || b >= nv || c < 0 || c >= nv) {
            acc[0] = __longlong_as_double(0x7ff8000000000000ll);  // NaN marks a bad index
            continue;
        }
        const double* p1 = x + 3 * (size_t)a;
        const double* p2 = x + 3 * (size_t)b;
        const double* p3 = x + 3 * (size_t)c;
        double e1x = p2[0] - p1[0], e1y = p2[1] - p1[1], e1z = p2[2] - p1[2];
        double e2x = p3[0] - p1[0], e2y = p3[1] - p1[1], e2z = p3[2] - p1[2];
        double cx = 0.5 * (e1y * e2z - e1z * e2y), cy = 0.5 * (e1z * e2x - e1x * e2z), cz = 0.5 * (e1x * e2y - e1y * e2x);
        double ar = sqrt(cx * cx + cy * cy + cz * cz);
        const double third = 1. / 3.;
        acc[0] += ar;
        acc[1] += third * (p1[0] + p2[0] + p3[0]) * ar;
        acc[2] += third * (p1[1] + p2[1] + p3[1]) * ar;
        acc[3] += third * (p1[2] + p2[2] + p3[2]) * ar;
    }
    warp_sum4(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 4; ++k) red[4 * wid + k] = acc[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int w = 0; w < kNaThreads / 32; ++w)
            for (int k = 0; k < 4; ++k) s[k] += red[4 * w + k];
        for (int k = 0; k < 4; ++k) part[4 * blockIdx.x + k] = s[k];
    }
}

// one warp sums the partials in a fixed order: lane l takes blocks l, l + 32, ...
__global__ void k_na_final(const double* __restrict__ part, int nb, double* __restrict__ out4) {
    double s[4] = {0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += 32)
        for (int k = 0; k < 4; ++k) s[k] += part[4 * b + k];
    warp_sum4(s);
    if (threadIdx.x == 0) {
        out4[0] = s[0];
        out4[1] = s[1] / s[0];
        out4[2] = s[2] / s[0];
        out4[3] = s[3] / s[0];
    }
}

}  // namespace

extern "C" int wcfe_area_tot_noalloc(const double* x_dev, int32_t n_vert, const int32_t* tri_dev, int32_t n_tri,
                                     double* area4_dev, void* stream) {
    if (!x_dev || !tri_dev || !area4_dev || n_vert <= 0 || n_tri <= 0) return WCFE_ERR_ARG;
    const int nb = (n_tri + kNaElems - 1) / kNaElems;
    if (nb > kNaMaxBlocks) return WCFE_ERR_LIMIT;
    // an error left pending by earlier work is not ours to clear, and would be taken
    // for this call's launch status below
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return wcfe::set_error((std::string("wcfe_area_tot_noalloc: CUDA error pending before the call: ") +
                                cudaGetErrorString(pending)).c_str(),
                               WCFE_ERR_CUDA);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return WCFE_ERR_NODEVICE;
    double* part = nullptr;
    {
        // set-up, once per device and with that device current: the host-side name of the
        // array is not a device address, so look the address up and keep it
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_addr[dev]) {
            void* p = nullptr;
            cudaError_t rc = cudaGetSymbolAddress(&p, g_na_part);
            if (rc != cudaSuccess || !p) {
                cudaGetLastError();   // the failed lookup's own error
                return wcfe::set_error("wcfe_area_tot_noalloc: cudaGetSymbolAddress failed", WCFE_ERR_CUDA);
            }
            g_na_addr[dev] = static_cast<double*>(p);
        }
        part = g_na_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_na_partials<<<nb, kNaThreads, 0, st>>>(x_dev, n_vert, tri_dev, n_tri, part);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_na_final<<<1, 32, 0, st>>>(part, nb, area4_dev);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return wcfe::set_error((std::string("wcfe_area_tot_noalloc launch: ") + cudaGetErrorString(e)).c_str(),
                               WCFE_ERR_CUDA);
    return WCFE_OK;
}
