// wcfe_common.cuh — device helpers shared by the FP64 and mixed-precision kernels.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "wcfe_device.cuh"

namespace wcfe {

// ---------------------------------------------------------------------------
// unfused arithmetic for reproduced decisions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xnorm3(double x, double y, double z) {
    return __dsqrt_rn(xa(xa(xm(x, x), xm(y, y)), xm(z, z)));
}

__device__ __forceinline__ double4 ld4(const double4* p) {
    double4 r;
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y;
    return r;
}
__device__ __forceinline__ double4 ld4v(const double4* p) {  // plain (coherent) load for data written this launch
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = q[0], b = q[1];
    return make_double4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void st4(double4* p, double x, double y, double z) {
    double2* q = reinterpret_cast<double2*>(p);
    q[0] = make_double2(x, y);
    q[1] = make_double2(z, 0.0);
}

// predicted velocity and position, bit-identical wherever they are recomputed
__device__ __forceinline__ void predict_vertex(const double4& x, const double4& V, const double4& A, double dt,
                                               double hdt, double vh[3], double xn[3]) {
    vh[0] = xa(V.x, xm(hdt, A.x));
    vh[1] = xa(V.y, xm(hdt, A.y));
    vh[2] = 0.0;
    xn[0] = xa(x.x, xm(dt, vh[0]));
    xn[1] = xa(x.y, xm(dt, vh[1]));
    xn[2] = xa(x.z, xm(dt, vh[2]));
}

// The radial protrusion driver (wcfe_params.protrude_v, the oracle's wo_drive_protrusion;
// the reference's velocity drivers prescribe the half-step velocity of driven nodes the
// same way, driverVelocities_Uniaxial UL:125-168): a boundary vertex moves radially from
// (protrude_cx, protrude_cy) at protrude_v, V_hlf = v (X - c) / |X - c| in the plane.
__device__ __forceinline__ void drive_protrusion(const wcfe_params& p, bool boundary, const double4& x, double dt,
                                                 double vh[3], double xn[3]) {
    if (p.protrude_v == 0.0 || !boundary) return;
    const double dx = xs(x.x, p.protrude_cx), dy = xs(x.y, p.protrude_cy);
    const double r = __dsqrt_rn(xa(xm(dx, dx), xm(dy, dy)));
    if (r == 0.0) return;
    vh[0] = xm(p.protrude_v, __ddiv_rn(dx, r));
    vh[1] = xm(p.protrude_v, __ddiv_rn(dy, r));
    vh[2] = 0.0;
    xn[0] = xa(x.x, xm(dt, vh[0]));
    xn[1] = xa(x.y, xm(dt, vh[1]));
    xn[2] = xa(x.z, xm(dt, vh[2]));
}
// predict_vertex with the cell's driver applied to vertex v
__device__ __forceinline__ void predict_vertex_c(const CellDev& c, int v, const double4& x, const double4& V,
                                                 const double4& A, double dt, double hdt, double vh[3], double xn[3]) {
    predict_vertex(x, V, A, dt, hdt, vh, xn);
    drive_protrusion(c.prm, c.bnd_rank[v] >= 0, x, dt, vh, xn);
}

// MD force-extension fit, UL:1203-1214
static __constant__ double c_md_px[6] = {0., 2.51250583e-03, 4.40265201e-03, 5.91408228e-03, 11.76817302e-03, 17.001e-03};
static __constant__ double c_md_py[6] = {-7.15514497, 71.80501308, 356.62420075, 356.96656556, 126.21811585, 528.40481124};
static __constant__ double c_md_k[6] = {31426.8556, 99485.86235, 67080.67086, -7908.39043, 21978.66923, 76858.39733};

// Spring force vector of bond u and the Bell force magnitude (UL:1245-1264, :2112-2137; k1 :1259, :2077)
__device__ __forceinline__ void spring_force(const wcfe_params& p, double ux, double uy, double uz, double fs[3],
                                             double* bell) {
    double D = xnorm3(ux, uy, uz);
    if (p.force_law == WCFE_LAW_LINEAR && p.rest_len == 0.0) {
        fs[0] = p.k_lin * ux; fs[1] = p.k_lin * uy; fs[2] = p.k_lin * uz;
        *bell = p.linear_norm2d ? p.k_lin * __dsqrt_rn(xa(xm(ux, ux), xm(uy, uy))) : p.k_lin * D;
        return;
    }
    double dx = 0, dy = 0, dz = 0;
    if (D != 0) {
        const double iD = 1.0 / D;
        dx = ux * iD; dy = uy * iD; dz = uz * iD;
    }
    double mag = 0.0;
    if (p.force_law == WCFE_LAW_MD_TABLE) {
        int j = -1;
        if (D >= c_md_px[5]) j = 5;
        else {
#pragma unroll
            for (int q = 0; q < 5; ++q)
                if (D < c_md_px[q + 1] && D >= c_md_px[q]) j = q;
        }
        if (j >= 0) mag = c_md_py[j] + c_md_k[j] * xs(D, c_md_px[j]);
    } else if (p.force_law == WCFE_LAW_LINEAR) {
        mag = D > p.rest_len ? p.k_lin * (D - p.rest_len) : 0.0;   // slack below the rest length
    } else {
        double e = D - p.rest_len;
        mag = e > 0.0 ? p.poly_k0 * (e + e * e * e / (3.0 * p.poly_x0 * p.poly_x0)) : 0.0;
    }
    fs[0] = mag * dx; fs[1] = mag * dy; fs[2] = mag * dz;
    if (p.force_law == WCFE_LAW_LINEAR && p.linear_norm2d) {
        double D2 = __dsqrt_rn(xa(xm(ux, ux), xm(uy, uy)));
        *bell = D2 > p.rest_len ? p.k_lin * (D2 - p.rest_len) : 0.0;
    } else {
        *bell = sqrt(fs[0] * fs[0] + fs[1] * fs[1] + fs[2] * fs[2]);
    }
}

// Containment test of point (px, py, pz) in triangle (p1, p2, p3) with barycentric weights
// (UL:2061-2100 and UL:1317-1465 use the same construction), unfused
__device__ __forceinline__ bool tri_contains(const double4& p1, const double4& p2, const double4& p3, double px, double py,
                                             double pz, double w[3]) {
    double e1x = xs(p2.x, p1.x), e1y = xs(p2.y, p1.y), e1z = xs(p2.z, p1.z);
    double e2x = xs(p3.x, p1.x), e2y = xs(p3.y, p1.y), e2z = xs(p3.z, p1.z);
    double nx = xs(xm(e1y, e2z), xm(e1z, e2y)), ny = xs(xm(e1z, e2x), xm(e1x, e2z)), nz = xs(xm(e1x, e2y), xm(e1y, e2x));
    double At = xm(0.5, xnorm3(nx, ny, nz));
    double epx = xs(px, p1.x), epy = xs(py, p1.y), epz = xs(pz, p1.z);
    double ax = xs(xm(e1y, epz), xm(e1z, epy)), ay = xs(xm(e1z, epx), xm(e1x, epz)), az = xs(xm(e1x, epy), xm(e1y, epx));
    double A3 = -1;
    if (az >= 0) A3 = xm(0.5, xnorm3(ax, ay, az));
    double bx = xs(xm(epy, e2z), xm(epz, e2y)), by = xs(xm(epz, e2x), xm(epx, e2z)), bz = xs(xm(epx, e2y), xm(epy, e2x));
    double A2 = -1;
    if (bz >= 0) A2 = xm(0.5, xnorm3(bx, by, bz));
    double A1 = xs(xs(At, A2), A3);
    if (A1 >= 0 && A2 >= 0 && A3 >= 0) {
        w[0] = A1 / At; w[1] = A2 / At; w[2] = A3 / At;
        return true;
    }
    return false;
}

// Point location in the substrate (UL:2061-2100): the last containing triangle wins.
// Positions P: the substrate's own X, or those of a coupled substrate cell.
__device__ __forceinline__ int locate_in(const SubDev& s, const double4* __restrict__ P, double px, double py, double pz,
                                         double w[3]) {
    int gx = (int)floor((px - s.ox) * s.inv_h), gy = (int)floor((py - s.oy) * s.inv_h);
    if (!(gx >= 0 && gx < s.gx && gy >= 0 && gy < s.gy)) return -1;
    int g = gy * s.gx + gx;
    int found = -1;
    for (int k = s.cell_ptr[g]; k < s.cell_ptr[g + 1]; ++k) {
        int e = s.cell_tri[k];
        int4 t = s.tri[e];
        double wk[3];
        if (tri_contains(ld4(P + t.x), ld4(P + t.y), ld4(P + t.z), px, py, pz, wk)) {
            found = e;
            w[0] = wk[0]; w[1] = wk[1]; w[2] = wk[2];
        }
    }
    return found;
}
__device__ __forceinline__ int locate(const SubDev& s, double px, double py, double pz, double w[3]) {
    return locate_in(s, s.X, px, py, pz, w);
}

// boundary neighbours and outward normal (UL:1489-1543)
__device__ __forceinline__ bool boundary_frame(const CellDev& c, const double4* __restrict__ xp, int rank,
                                               const double xi[3], double x1[3], double x2[3]) {
    int j1 = -1, j2 = -1;
    for (int k = c.bnd_cptr[rank]; k < c.bnd_cptr[rank + 1]; ++k) {
        int2 cd = c.bnd_cand[k];
        double4 pb = ld4v(xp + cd.x), pi = ld4v(xp + cd.y);
        double d1x = xs(xi[0], pb.x), d1y = xs(xi[1], pb.y);
        double d2x = xs(pi.x, xi[0]), d2y = xs(pi.y, xi[1]);
        double ncz = xs(xm(d1x, d2y), xm(d1y, d2x));
        if (ncz > 0) j1 = cd.x;
        else j2 = cd.x;
    }
    if (j1 < 0 || j2 < 0) return false;
    double4 a = ld4v(xp + j1), bq = ld4v(xp + j2);
    x1[0] = a.x; x1[1] = a.y; x1[2] = a.z;
    x2[0] = bq.x; x2[1] = bq.y; x2[2] = bq.z;
    return true;
}


// The last vertex-phase block of a cell (an atomic ticket in ctl[2]) reduces the
// cell's per-block area partials in a fixed order into area4 = {A, cx, cy, cz}.
__device__ __forceinline__ void finish_area(const CellDev& c) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 2), 1u);
        s_last = ((int)t == c.nk1 - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x < 32) {
        double s4[4] = {0, 0, 0, 0};
        for (int k = threadIdx.x; k < c.nk1; k += 32)
#pragma unroll
            for (int q = 0; q < 4; ++q) s4[q] += __ldcg(c.k1_part + 4 * k + q);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s4[q] += __shfl_xor_sync(0xffffffffu, s4[q], o);
        if (threadIdx.x == 0) {
            c.area4[0] = s4[0];
            c.area4[1] = s4[1] / s4[0];
            c.area4[2] = s4[2] / s4[0];
            c.area4[3] = s4[3] / s4[0];
            c.ctl[2] = 0;
        }
    }
}

// Blocks per SM of `kernel` at a launch shape (at least 1), cached per device, kernel,
// block size and dynamic shared memory (wcfe_kernels.cu): the occupancy query is a driver
// call of a few microseconds, and the host issues the same shapes every step.
int occupancy_cached(const void* kernel, int threads, size_t smem);

}  // namespace wcfe
