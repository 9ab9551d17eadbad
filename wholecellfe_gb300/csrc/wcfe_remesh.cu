// wcfe_remesh.cu — device side of El Topo co-residency: the cell state follows the host's
// remeshing without a host round trip.
//
// El Topo carries each vertex's state through its operations: an edge split appends a
// vertex whose every field is 0.5 (s[a] + s[b]) (eltopo3d/edgesplitter.cpp:564-577, both
// ends possibly earlier splits), collapses and flips leave the states of the surviving
// vertices as they are, and defrag_mesh keeps the survivors in order
// (eltopo3d/surftrack.cpp:487-593).  Here: pack the old state into binary64 records
// (either state layout), apply the splits level by level (a level's splits read only
// old vertices and earlier levels), and gather the survivors into the new state block.
// Positions are not interpolated: the host's remeshed positions are authoritative.
#include <cuda_runtime.h>

#include <algorithm>

#include "wcfe_device.cuh"

namespace wcfe {

// binary64 record of one vertex: V [0,3), A [3,6), ea [6,12), cA 12, cC 13, fau [14,17), rho 17
constexpr int kRemeshRec = 18;

namespace {

__device__ __forceinline__ double ffd(float hi, float lo) { return (double)hi + (double)lo; }
__device__ __forceinline__ void ff_split(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}
// exact split of a binary64 position coordinate into h + m + l
__device__ __forceinline__ void tf_split(double x, float& h, float& m, float& l) {
    h = __double2float_rn(x);
    const double r = x - (double)h;
    m = __double2float_rn(r);
    l = __double2float_rn(r - (double)m);
}

__global__ void k_remesh_pack(CellDev c, int mixed, const void* rho, double* __restrict__ ext,
                              unsigned long long* __restrict__ hdr) {
    const int n = c.nv, par = c.ctl[0];
    const size_t N = (size_t)n;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        double* r = ext + (size_t)kRemeshRec * v;
        if (!mixed) {
            const double4 V = c.vel[v], A = c.acc[v], u = c.fau[v];
            r[0] = V.x; r[1] = V.y; r[2] = V.z;
            r[3] = A.x; r[4] = A.y; r[5] = A.z;
            const double* e = c.ea[par] + 6 * (size_t)v;
#pragma unroll
            for (int q = 0; q < 6; ++q) r[6 + q] = e[q];
            r[12] = c.cA[v];
            r[13] = c.cC[v];
            r[14] = u.x; r[15] = u.y; r[16] = u.z;
            r[17] = rho ? static_cast<const double*>(rho)[v] : 0.0;
        } else {
            const float4* vh = reinterpret_cast<const float4*>(c.vel);
            const float4* uh = reinterpret_cast<const float4*>(c.fau);
            const float4* ah = reinterpret_cast<const float4*>(c.acc);
            const float4* eh = reinterpret_cast<const float4*>(c.ea[par]);
            const float* ca = reinterpret_cast<const float*>(c.cA);
            const float* cc = reinterpret_cast<const float*>(c.cC);
            const float4 V0 = vh[v], V1 = vh[N + v], U0 = uh[v], U1 = uh[N + v], A = ah[v];
            const float4 e0 = eh[v], e1 = eh[N + v], e2 = eh[2 * N + v];
            r[0] = ffd(V0.x, V1.x); r[1] = ffd(V0.y, V1.y); r[2] = ffd(V0.z, V1.z);
            r[3] = A.x; r[4] = A.y; r[5] = A.z;
            r[6] = ffd(e0.x, e1.x); r[7] = ffd(e0.y, e1.y); r[8] = ffd(e0.z, e1.z); r[9] = ffd(e0.w, e1.w);
            r[10] = ffd(e2.x, e2.z); r[11] = ffd(e2.y, e2.w);
            r[12] = ffd(ca[v], ca[N + v]);
            r[13] = ffd(cc[v], cc[N + v]);
            r[14] = ffd(U0.x, U1.x); r[15] = ffd(U0.y, U1.y); r[16] = ffd(U0.z, U1.z);
            r[17] = rho ? (double)static_cast<const float*>(rho)[v] : 0.0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        hdr[0] = (unsigned long long)__double_as_longlong(c.clk[0]);
        hdr[1] = c.ap[0];
        hdr[2] = c.status[0];
    }
}

// the splits of one level: vertex n_old + k takes 0.5 (s[a] + s[b]) field by field
__global__ void k_remesh_split(double* __restrict__ ext, int n_old, const int* __restrict__ ks, int cnt,
                               const int2* __restrict__ ab) {
    const long long total = (long long)cnt * kRemeshRec;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int k = ks[i / kRemeshRec], f = (int)(i % kRemeshRec);
        const int2 s = ab[k];
        ext[(size_t)kRemeshRec * (n_old + k) + f] =
            0.5 * (ext[(size_t)kRemeshRec * s.x + f] + ext[(size_t)kRemeshRec * s.y + f]);
    }
}

// the survivors into the new (zeroed, parity 0) state block
__global__ void k_remesh_unpack(CellDev c, int mixed, const double* __restrict__ ext, const int* __restrict__ keep,
                                const double* __restrict__ x, void* rho, const unsigned long long* __restrict__ hdr) {
    const int n = c.nv;
    const size_t N = (size_t)n;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double* r = ext + (size_t)kRemeshRec * keep[j];
        const double* p = x + 3 * (size_t)j;
        if (!mixed) {
            c.pos[0][j] = make_double4(p[0], p[1], p[2], 0.0);
            c.vel[j] = make_double4(r[0], r[1], r[2], 0.0);
            c.acc[j] = make_double4(r[3], r[4], r[5], 0.0);
            double* e = c.ea[0] + 6 * (size_t)j;
#pragma unroll
            for (int q = 0; q < 6; ++q) e[q] = r[6 + q];
            c.cA[j] = r[12];
            c.cC[j] = r[13];
            c.fau[j] = make_double4(r[14], r[15], r[16], 0.0);
            if (rho) static_cast<double*>(rho)[j] = r[17];
        } else {
            float4* ph = reinterpret_cast<float4*>(c.pos[0]);
            float4* vh = reinterpret_cast<float4*>(c.vel);
            float4* uh = reinterpret_cast<float4*>(c.fau);
            float4* ah = reinterpret_cast<float4*>(c.acc);
            float4 h, l;
            // positions: triple-float x and y (the third floats in the w slots), float-float z
            tf_split(p[0], h.x, l.x, h.w);
            tf_split(p[1], h.y, l.y, l.w);
            ff_split(p[2], h.z, l.z);
            ph[j] = h; ph[N + j] = l;
            ff_split(r[0], h.x, l.x); ff_split(r[1], h.y, l.y); ff_split(r[2], h.z, l.z);
            vh[j] = h; vh[N + j] = l;
            ff_split(r[14], h.x, l.x); ff_split(r[15], h.y, l.y); ff_split(r[16], h.z, l.z);
            uh[j] = h; uh[N + j] = l;
            ah[j] = make_float4(__double2float_rn(r[3]), __double2float_rn(r[4]), __double2float_rn(r[5]), 0.0f);
            float4 e0, e1, e2;
            ff_split(r[6], e0.x, e1.x); ff_split(r[7], e0.y, e1.y); ff_split(r[8], e0.z, e1.z); ff_split(r[9], e0.w, e1.w);
            ff_split(r[10], e2.x, e2.z); ff_split(r[11], e2.y, e2.w);
            for (int b = 0; b < 2; ++b) {   // both strain buffers (the mixed step carries xz, yz unchanged)
                float4* eh = reinterpret_cast<float4*>(c.ea[b]);
                eh[j] = e0; eh[N + j] = e1; eh[2 * N + j] = e2;
            }
            float* ca = reinterpret_cast<float*>(c.cA);
            float* cc = reinterpret_cast<float*>(c.cC);
            ff_split(r[12], ca[j], ca[N + j]);
            ff_split(r[13], cc[j], cc[N + j]);
            if (rho) static_cast<float*>(rho)[j] = __double2float_rn(r[17]);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        c.ctl[0] = 0;
        c.clk[0] = __longlong_as_double((long long)hdr[0]);
        c.ap[0] = hdr[1];
        c.status[0] = (uint32_t)hdr[2];
    }
}

int grid_of(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }

}  // namespace

void launch_remesh_pack(const CellDev& c, int mixed, const void* rho, double* ext, unsigned long long* hdr,
                        cudaStream_t st) {
    k_remesh_pack<<<grid_of(c.nv), 256, 0, st>>>(c, mixed, rho, ext, hdr);
}
void launch_remesh_split(double* ext, int n_old, const int* ks, int cnt, const int2* ab, cudaStream_t st) {
    if (cnt > 0) k_remesh_split<<<grid_of((long long)cnt * kRemeshRec), 256, 0, st>>>(ext, n_old, ks, cnt, ab);
}
void launch_remesh_unpack(const CellDev& c, int mixed, const double* ext, const int* keep, const double* x, void* rho,
                          const unsigned long long* hdr, cudaStream_t st) {
    k_remesh_unpack<<<grid_of(c.nv), 256, 0, st>>>(c, mixed, ext, keep, x, rho, hdr);
}

}  // namespace wcfe
