// wcfe_mixed.cu — the mixed-precision form (WCFE_PREC_MIXED) of the step.
//
// The cell is a planar membrane (z = 0) with counter-clockwise triangles, as
// the reference's cell path is: read_ecomsol forces z = 0 (cellBP/iomesh.cpp:519)
// and driverVelocities_Explicit zeroes the normal velocity (UL:119).  Then
// N = n = e3 and every tensor of evalElementRe (UL:710-928) is an in-plane 2x2
// block plus a decoupled zz entry; this form computes the 2x2 blocks.
//
// Element assembly runs in FP32 in an increment form that is algebraically the
// reference's.  With F = I + H, E the integration-point strain and P the
// in-plane identity, the stress is
//     S_pas = mu [c0 P + beta / theta_g - theta_g (1 + eta) gamma]
//     beta  = be_t - I   = 2 E (I - 2E)^-1
//     gamma = C^-1 - I   = -c C^-1,  c = H + H^T + H^T H
//     eta   = lambda_N^2 - 1 = (theta_g^2 (1 + de) - (1 + dth)^2) / (1 + dth)^2
//     c0    = -(theta_g^2 - 1 + theta_g^2 eta) / theta_g
// with de = det(I - 2E) - 1 and dth = det F - 1 from the invariants.  Every
// FP32 quantity is thus a small number at full relative precision, not a
// difference of two O(1) numbers.  The isotropic active stress kappa t_act I
// contributes w b_i per element corner; on a closed one-ring these sum to
// exactly zero, so it stays out of the FP32 element and is added in FP64 for
// boundary vertices: (1/2) kappa t_act thick e3 x sum (X_k - X_j).  The strain
// update uses K = F^-1 - I = -H F^-1:
//     ea_s - E = theta_g^2 D + (theta_g^2 - 1)(E - I/2),
//     D = K^T E + E K + K^T E K - (K + K^T + K^T K)/2.
//
// The vertex phase packs each vertex's element inputs into an FP32 record:
// the position as float-float (hi, lo), the step displacement u = x - X and
// the strain.  The element loop therefore does no FP64 arithmetic.  The state
// and every accumulation (x, V, the strain, c_C, the bond vector) stay FP64; the
// per-step force and acceleration are FP32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "wcfe_common.cuh"
#include "wcfe_cvt.h"

namespace wcfe {

struct MixedArgs {
    const CellDev* cells;
    const WorkItem* work;
    int nwork, emax;
    double dt, dt_real, hdt, cdt, ap_thresh, t_override;
    int vh_from_buf, half;   // cdt = dt_real - dt/2; half = dt_real > dt/2
};

// sign tests of doubles on the integer pipe (the FP64 pipe is the scarce one)
__device__ __forceinline__ bool dzero(double x) { return (dbits(x) << 1) == 0; }
__device__ __forceinline__ bool dneg(double x) {   // x < 0
    const uint64_t b = dbits(x);
    return (int64_t)b < 0 && (b << 1) != 0 && (b << 1) <= (0x7FF0000000000000ull << 1);
}
__device__ __forceinline__ bool dpos(double x) {   // x > 0
    const uint64_t b = dbits(x);
    return (int64_t)b > 0 && b <= 0x7FF0000000000000ull;
}

constexpr int kRec = 3;      // float4 per vertex record
constexpr int kSlot32 = 20;  // floats per element slot in shared memory

// MD force-extension fit (UL:1203-1214) in FP32
static __constant__ float c_md_px32[6] = {0.f, 2.51250583e-03f, 4.40265201e-03f, 5.91408228e-03f, 11.76817302e-03f, 17.001e-03f};
static __constant__ float c_md_py32[6] = {-7.15514497f, 71.80501308f, 356.62420075f, 356.96656556f, 126.21811585f, 528.40481124f};
static __constant__ float c_md_k32[6] = {31426.8556f, 99485.86235f, 67080.67086f, -7908.39043f, 21978.66923f, 76858.39733f};

// Spring force of bond u in FP32 (UL:1245-1264; k1 UL:1259-1261; the polynomial extension)
// and the Bell force magnitude of updateFA (UL:2137; k1 UL:2077).
__device__ __forceinline__ void spring_force32(const ParamF& p, float ux, float uy, float uz, float fs[3],
                                               float* bell) {
    const float D = sqrtf(ux * ux + uy * uy + uz * uz);
    const float k = p.k_lin, L0 = p.rest_len;
    if (p.law == PF_LINEAR0) {
        fs[0] = k * ux; fs[1] = k * uy; fs[2] = k * uz;
        *bell = p.norm2d ? k * sqrtf(ux * ux + uy * uy) : k * D;
        return;
    }
    const float iD = D != 0.0f ? 1.0f / D : 0.0f;
    float mag = 0.0f;
    if (p.law == PF_MD) {
        int j = -1;
        if (D >= c_md_px32[5]) j = 5;
        else {
#pragma unroll
            for (int q = 0; q < 5; ++q)
                if (D < c_md_px32[q + 1] && D >= c_md_px32[q]) j = q;
        }
        if (j >= 0) mag = c_md_py32[j] + c_md_k32[j] * (D - c_md_px32[j]);
    } else if (p.law == PF_LINEAR) {
        mag = k * (D - L0);
    } else {
        const float e = D - L0;
        mag = p.poly_k0 * (e + e * e * e * p.poly_c3);
    }
    fs[0] = mag * ux * iD; fs[1] = mag * uy * iD; fs[2] = mag * uz * iD;
    if (p.law == PF_LINEAR && p.norm2d) *bell = fabsf(k * (sqrtf(ux * ux + uy * uy) - L0));
    else *bell = fabsf(mag) * (D != 0.0f ? 1.0f : 0.0f);
}

struct ElemParams {   // per-cell constants of the element, hoisted out of the element loop
    float mu, thick, grow, s_iso, t_an, cx, cy;
};

// planar element in the increment form; outputs per corner: Re (x, y), Re_ea (xx, yy, xy, zz)
struct Elem2 {
    float re[3][2];
    float rea[3][4];
    float mm, acur;
};

__device__ __forceinline__ void element2d(const float4 r[3][kRec], const ElemParams& q, Elem2& o) {
    // r0 = (Xhi.x, Xhi.y, Xlo.x, Xlo.y), r1 = (u.x, u.y, exx, eyy), r2 = (exy, ezz, -, -)
    const float G1x = (r[1][0].x - r[0][0].x) + (r[1][0].z - r[0][0].z);
    const float G1y = (r[1][0].y - r[0][0].y) + (r[1][0].w - r[0][0].w);
    const float G2x = (r[2][0].x - r[0][0].x) + (r[2][0].z - r[0][0].z);
    const float G2y = (r[2][0].y - r[0][0].y) + (r[2][0].w - r[0][0].w);
    const float d1x = r[1][1].x - r[0][1].x, d1y = r[1][1].y - r[0][1].y;
    const float d2x = r[2][1].x - r[0][1].x, d2y = r[2][1].y - r[0][1].y;
    const float Gc = G1x * G2y - G1y * G2x;  // > 0: counter-clockwise
    const float iG = 1.0f / Gc;
    // shape gradients in the reference configuration: b1 = (G2 x e3)/Gc, b2 = (e3 x G1)/Gc
    const float b1x = G2y * iG, b1y = -G2x * iG;
    const float b2x = -G1y * iG, b2y = G1x * iG;
    const float b0x = -b1x - b2x, b0y = -b1y - b2y;
    // H = d1 (x) b1 + d2 (x) b2
    const float H00 = d1x * b1x + d2x * b2x, H01 = d1x * b1y + d2x * b2y;
    const float H10 = d1y * b1x + d2y * b2x, H11 = d1y * b1y + d2y * b2y;
    const float gc = (G1x + d1x) * (G2y + d2y) - (G1y + d1y) * (G2x + d2x);
    // strain at the integration point
    const float third = 1.0f / 3.0f;
    const float exx = third * (r[0][1].z + r[1][1].z + r[2][1].z);
    const float eyy = third * (r[0][1].w + r[1][1].w + r[2][1].w);
    const float exy = third * (r[0][2].x + r[1][2].x + r[2][2].x);
    const float ezz = third * (r[0][2].y + r[1][2].y + r[2][2].y);
    // beta = 2 E (I - 2E)^-1 ; de = det(I - 2E) - 1 (with the zz factor 1 - 2 ezz)
    const float m00 = 1.0f - 2.0f * exx, m11 = 1.0f - 2.0f * eyy, m01 = -2.0f * exy;
    const float dm1 = -2.0f * (exx + eyy) + 4.0f * (exx * eyy - exy * exy);  // det(I - 2E_2) - 1
    const float idM = 1.0f / (1.0f + dm1);
    const float i00 = m11 * idM, i01 = -m01 * idM, i11 = m00 * idM;  // (I - 2E)^-1, symmetric
    const float be00 = 2.0f * (exx * i00 + exy * i01), be01 = 2.0f * (exx * i01 + exy * i11);
    const float be11 = 2.0f * (exy * i01 + eyy * i11);
    const float de = dm1 - 2.0f * ezz * (1.0f + dm1);
    // gamma = -c (I + c)^-1, c = H + H^T + H^T H
    const float c00 = 2.0f * H00 + (H00 * H00 + H10 * H10);
    const float c11 = 2.0f * H11 + (H01 * H01 + H11 * H11);
    const float c01 = H01 + H10 + (H00 * H01 + H10 * H11);
    const float dC = (1.0f + c00) * (1.0f + c11) - c01 * c01;
    const float iC = 1.0f / dC;
    const float ci00 = (1.0f + c11) * iC, ci01 = -c01 * iC, ci11 = (1.0f + c00) * iC;
    const float ga00 = -(c00 * ci00 + c01 * ci01), ga01 = -(c00 * ci01 + c01 * ci11);
    const float ga11 = -(c01 * ci01 + c11 * ci11);
    // dth = det F - 1 = tr H + det H
    const float dth = (H00 + H11) + (H00 * H11 - H01 * H10);
    const float g = q.grow, thg = 1.0f + g, gg2 = 2.0f * g + g * g;
    const float one_dth = 1.0f + dth;
    const float eta = (gg2 + thg * thg * de - 2.0f * dth - dth * dth) / (one_dth * one_dth);
    const float c0 = -(gg2 + thg * thg * eta) / thg;
    const float ith = 1.0f / thg, tge = thg * (1.0f + eta);
    float S00 = q.mu * (c0 + be00 * ith - tge * ga00);
    float S01 = q.mu * (be01 * ith - tge * ga01);
    float S11 = q.mu * (c0 + be11 * ith - tge * ga11);
    if (q.t_an != 0.0f) {  // anisotropic active stress t_act (1 - 2 kappa) a0 a0^T
        float ax = third * ((r[0][0].x + r[1][0].x + r[2][0].x) + (r[0][0].z + r[1][0].z + r[2][0].z) +
                            (r[0][1].x + r[1][1].x + r[2][1].x)) - q.cx;
        float ay = third * ((r[0][0].y + r[1][0].y + r[2][0].y) + (r[0][0].w + r[1][0].w + r[2][0].w) +
                            (r[0][1].y + r[1][1].y + r[2][1].y)) - q.cy;
        const float ia = rsqrtf(ax * ax + ay * ay);
        ax *= ia; ay *= ia;
        S00 += q.t_an * ax * ax; S01 += q.t_an * ax * ay; S11 += q.t_an * ay * ay;
    }
    // T = s_iso H + (I + H) S
    const float T00 = q.s_iso * H00 + S00 + (H00 * S00 + H01 * S01);
    const float T01 = q.s_iso * H01 + S01 + (H00 * S01 + H01 * S11);
    const float T10 = q.s_iso * H10 + S01 + (H10 * S00 + H11 * S01);
    const float T11 = q.s_iso * H11 + S11 + (H10 * S01 + H11 * S11);
    const float wA = 0.5f * Gc * q.thick;
    o.re[0][0] = wA * (T00 * b0x + T01 * b0y); o.re[0][1] = wA * (T10 * b0x + T11 * b0y);
    o.re[1][0] = wA * (T00 * b1x + T01 * b1y); o.re[1][1] = wA * (T10 * b1x + T11 * b1y);
    o.re[2][0] = wA * (T00 * b2x + T01 * b2y); o.re[2][1] = wA * (T10 * b2x + T11 * b2y);
    // strain: K = -H (I + H)^-1
    const float iF = 1.0f / one_dth;  // det(I + H) = 1 + dth
    const float f00 = (1.0f + H11) * iF, f01 = -H01 * iF, f10 = -H10 * iF, f11 = (1.0f + H00) * iF;
    const float K00 = -(H00 * f00 + H01 * f10), K01 = -(H00 * f01 + H01 * f11);
    const float K10 = -(H10 * f00 + H11 * f10), K11 = -(H10 * f01 + H11 * f11);
    // E K and K^T E K
    const float EK00 = exx * K00 + exy * K10, EK01 = exx * K01 + exy * K11;
    const float EK10 = exy * K00 + eyy * K10, EK11 = exy * K01 + eyy * K11;
    const float KEK00 = K00 * EK00 + K10 * EK10, KEK01 = K00 * EK01 + K10 * EK11;
    const float KEK11 = K01 * EK01 + K11 * EK11;
    const float KK00 = K00 * K00 + K10 * K10, KK01 = K00 * K01 + K10 * K11, KK11 = K01 * K01 + K11 * K11;
    // D = K^T E + E K + K^T E K - (K + K^T + K^T K)/2; (K^T E)_ij = (E K)_ji
    const float D00 = 2.0f * EK00 + KEK00 - 0.5f * (2.0f * K00 + KK00);
    const float D11 = 2.0f * EK11 + KEK11 - 0.5f * (2.0f * K11 + KK11);
    const float D01 = (EK10 + EK01) + KEK01 - 0.5f * (K01 + K10 + KK01);
    const float tg2 = thg * thg, gg = tg2 - 1.0f;
    const float dvxx = tg2 * D00 + gg * (exx - 0.5f), dvyy = tg2 * D11 + gg * (eyy - 0.5f);
    const float dvxy = tg2 * D01 + gg * exy, dvzz = gg * (ezz - 0.5f);
    const float w3 = third * wA;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o.rea[i][0] = w3 * ((exx - r[i][1].z) + dvxx);
        o.rea[i][1] = w3 * ((eyy - r[i][1].w) + dvyy);
        o.rea[i][2] = w3 * ((exy - r[i][2].x) + dvxy);
        o.rea[i][3] = w3 * ((ezz - r[i][2].y) + dvzz);
    }
    o.mm = w3;
    o.acur = 0.5f * fabsf(gc);
}

constexpr int kBndSlots = 128;   // boundary vertices a patch CTA queues for its second loop

// Boundary terms of vertex v (rank `rank`) in FP64, added to (F0, F1): the isotropic
// active stress of the open one-ring, AP push (calculateForce_AP UL:1477-1569),
// bending (calculateBendingForce2D UL:1571-1689) and area constraint
// (calculateAreaConstraintForce UL:1691-1784), on the neighbour frame of UL:1500-1531.
__device__ __forceinline__ void boundary_force(const CellDev& c, const MixedArgs& a, const int4& pt,
                                               const double4* __restrict__ X, const double4* __restrict__ xp, int v,
                                               int rank, unsigned long long ap_call, float& F0, float& F1) {
    const wcfe_params& p = c.prm;
    const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
    const double s_iso = p.kappa * (t < p.tact_t1 ? t * p.tact_rate : p.tact_max);
    const double area_tot = c.area4[0];
    const double4 xv4 = ld4v(xp + v);
    const double xi[3] = {xv4.x, xv4.y, xv4.z};
    // isotropic active stress on the open one-ring: (1/2) s_iso thick e3 x sum (X_k - X_j)
    double sx = 0, sy = 0;
    for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
        const int code = c.vc_code[k];
        const int cn = code & 3;
        const int e = c.patch_elems[pt.z + (code >> 2)];
        const int4 t4 = c.tri[e];
        const int ids[3] = {t4.x, t4.y, t4.z};
        const double4 Xj = ld4v(X + ids[(cn + 1) % 3]), Xk = ld4v(X + ids[(cn + 2) % 3]);
        sx += Xk.x - Xj.x;
        sy += Xk.y - Xj.y;
    }
    const double w = 0.5 * s_iso * p.thick;
    double Fb0 = w * sy, Fb1 = -w * sx;  // minus the residual term w e3 x s
    double x1[3], x2[3];
    if (boundary_frame(c, xp, rank, xi, x1, x2)) {
        const double d1x = xi[0] - x1[0], d1y = xi[1] - x1[1], d2x = x2[0] - xi[0], d2y = x2[1] - xi[1];
        const double d1z = xi[2] - x1[2], d2z = x2[2] - xi[2];
        const double nn1 = sqrt(d1y * d1y + d1x * d1x), nn2 = sqrt(d2y * d2y + d2x * d2x);
        const double l1 = sqrt(d1x * d1x + d1y * d1y + d1z * d1z), l2 = sqrt(d2x * d2x + d2y * d2y + d2z * d2z);
        const double L = l1 + l2;
        const double nx = l1 / L * (d1y / nn1) + l2 / L * (d2y / nn2);
        const double ny = l1 / L * (-d1x / nn1) + l2 / L * (-d2x / nn2);
        double fb = 0.0;
        if (p.ap_enable) {
            const uint32_t r31 = ap_draw(p.seed, p.stream, ap_call, (uint32_t)rank);
            const double Pr = (double)r31 / ((double)2147483647 + 1.);
            const double lim = p.ap_density * L / 2;
            const double cnt = lim > 0 ? ceil(lim) : 0.0;
            const double apt = isnan(a.ap_thresh) ? c.ap_thresh : a.ap_thresh;
            fb += (Pr < apt) ? p.ap_force * cnt : 0.0;
        }
        const double e1x = d1x / l1, e1y = d1y / l1, e1z = d1z / l1, e2x = d2x / l2, e2y = d2y / l2, e2z = d2z / l2;
        const double cost = e1x * e2x + e1y * e2y + e1z * e2z;
        const double ez = xs(xm(e1x, e2y), xm(e1y, e2x));
        const double turna = ez > 0 ? cost - 1 : 1 - cost;
        fb += p.k_bend * (turna * 2 / L);
        fb += -p.k_area * (area_tot - p.area0) / 2 * L;
        Fb0 += fb * nx;
        Fb1 += fb * ny;
    }
    F0 += (float)Fb0;
    F1 += (float)Fb1;
}

// Explicit update of vertex v (UL:592-628): A in FP32 from the FP32 force; V and the
// strain accumulate in FP64.
__device__ __forceinline__ void finish_vertex(const CellDev& c, const MixedArgs& a, int par, int v, float F0, float F1,
                                              float Q0, float Q1, float Q2, float Q3, float MMf) {
    const ParamF& pf = c.pf;
    const double4 V4 = ld4v(c.vel + v), A4 = ld4v(c.acc + v);
    double vh0, vh1;
    if (a.vh_from_buf) {
        const double4 h = ld4v(c.vhl + v);
        vh0 = h.x; vh1 = h.y;
    } else {
        vh0 = fma(a.hdt, A4.x, V4.x);
        vh1 = fma(a.hdt, A4.y, V4.y);
    }
    const float rhom = pf.rho;
    const float iM = 1.0f / (MMf * rhom);
    const float damp_m = pf.damp * MMf * rhom;
    const float vh0f = f64_to_f32_rn(vh0), vh1f = f64_to_f32_rn(vh1);
    const float An0 = (F0 - pf.drag * vh0f - damp_m * f64_to_f32_rn(V4.x)) * iM;
    const float An1 = (F1 - pf.drag * vh1f - damp_m * f64_to_f32_rn(V4.y)) * iM;
    const float An2 = dzero(V4.z) ? 0.0f : (-damp_m * f64_to_f32_rn(V4.z)) * iM;  // no force normal to the plane
    const double An0d = f32_to_f64(An0), An1d = f32_to_f64(An1), An2d = f32_to_f64(An2);
    double Vn0, Vn1, Vn2;
    if (a.half) {
        Vn0 = fma(a.cdt, An0d, vh0);
        Vn1 = fma(a.cdt, An1d, vh1);
        Vn2 = a.cdt * An2d;
    } else {
        Vn0 = fma(a.dt_real, An0d, V4.x);
        Vn1 = fma(a.dt_real, An1d, V4.y);
        Vn2 = fma(a.dt_real, An2d, V4.z);
    }
    const double2* eo = reinterpret_cast<const double2*>(c.ea[par] + 6 * (size_t)v);
    double2* en = reinterpret_cast<double2*>(c.ea[par ^ 1] + 6 * (size_t)v);
    const float iMM = 1.0f / MMf;
    const double2 e0 = eo[0], e1 = eo[1], e2 = eo[2];  // (xx, yy), (zz, xy), (xz, yz)
    en[0] = make_double2(e0.x + f32_to_f64(Q0 * iMM), e0.y + f32_to_f64(Q1 * iMM));
    en[1] = make_double2(e1.x + f32_to_f64(Q3 * iMM), e1.y + f32_to_f64(Q2 * iMM));
    en[2] = e2;
    st4(c.acc + v, An0d, An1d, An2d);
    st4(c.vel + v, Vn0, Vn1, Vn2);
    // NaN/Inf in the state shows up in the FP32 quantities derived from it
    const float chk = An0 + An1 + Q0 + Q1 + Q2 + vh0f + vh1f;
    if (!isfinite(chk)) atomicOr(c.status, 1u);
}

__global__ void __launch_bounds__(128) k_patch_phase_mixed(MixedArgs a) {
    extern __shared__ float smf[];
    const int emax = a.emax;
    // structure of arrays: field k of slot j at smf[k * emax + j]
    __shared__ ElemParams s_q;
    __shared__ int s_nbnd;
    __shared__ float s_bnd[8 * kBndSlots];
    for (int w = blockIdx.x; w < a.nwork; w += gridDim.x) {
        const WorkItem it = a.work[w];
        const CellDev& c = a.cells[it.cell];
        const int4 pt = c.patch[it.idx];
        const int par = c.ctl[0];
        const double4* __restrict__ X = c.pos[par];
        const double4* __restrict__ xp = c.pos[par ^ 1];
        const float4* __restrict__ rec = c.rec;
        const unsigned long long ap_call = c.ap[0];
        if (threadIdx.x == 0) {   // the element constants of this cell and step, once per CTA
            s_nbnd = 0;
            const wcfe_params& p = c.prm;
            const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
            const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
            s_q.mu = (float)p.mu;
            s_q.thick = (float)p.thick;
            s_q.grow = (float)(p.thetag_dot * a.dt_real);
            s_q.s_iso = (float)(p.kappa * t_act);
            s_q.t_an = (float)((1.0 - 2.0 * p.kappa) * t_act);
            s_q.cx = (float)c.area4[1];
            s_q.cy = (float)c.area4[2];
        }
        __syncthreads();
        const ElemParams q = s_q;
        // ---- elements of the patch -> shared memory ----
        for (int j = threadIdx.x; j < pt.w; j += blockDim.x) {
            const int e = c.patch_elems[pt.z + j];
            const int4 t4 = __ldg(c.tri + e);
            const int id[3] = {t4.x, t4.y, t4.z};
            float4 r[3][kRec];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int m = 0; m < kRec; ++m) r[k][m] = rec[kRec * (size_t)id[k] + m];
            Elem2 o;
            element2d(r, q, o);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                smf[(2 * k + 0) * emax + j] = o.re[k][0];
                smf[(2 * k + 1) * emax + j] = o.re[k][1];
#pragma unroll
                for (int m = 0; m < 4; ++m) smf[(6 + 4 * k + m) * emax + j] = o.rea[k][m];
            }
            smf[18 * emax + j] = o.mm;
            smf[19 * emax + j] = o.acur;
        }
        __syncthreads();
        // ---- owned vertices: forces and the acceleration in FP32, accumulations in FP64 ----
        // Interior vertices finish here.  Boundary vertices queue their FP32 sums in shared
        // memory and finish in a second loop over consecutive threads, so that the FP64
        // boundary terms run on full warps instead of one or two lanes of many warps.
        const ParamF& pf = c.pf;
        const float rho_max = pf.rho_i_max;
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            float R0 = 0, R1 = 0, Q0 = 0, Q1 = 0, Q2 = 0, Q3 = 0, MMf = 0, Asf = 0;
            for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                const int code = c.vc_code[k];
                const int sl = code >> 2, cn = code & 3;
                R0 += smf[(2 * cn) * emax + sl];
                R1 += smf[(2 * cn + 1) * emax + sl];
                Q0 += smf[(6 + 4 * cn) * emax + sl];
                Q1 += smf[(7 + 4 * cn) * emax + sl];
                Q2 += smf[(8 + 4 * cn) * emax + sl];
                Q3 += smf[(9 + 4 * cn) * emax + sl];
                MMf += smf[18 * emax + sl];
                Asf += smf[19 * emax + sl];
            }
            const float Asum = Asf * (1.0f / 3.0f);
            // integrin force (UL:1241-1269) in FP32
            const double4 f4 = ld4v(c.fau + v);
            float fs[3], bell;
            spring_force32(pf, f64_to_f32_rn(f4.x), f64_to_f32_rn(f4.y), f64_to_f32_rn(f4.z), fs, &bell);
            const float rho = c.rho_w ? f64_to_f32_rn(c.rho_w[v]) : rho_max;
            const float kfa = -f64_to_f32_rn(c.cC[v]) * Asum * rho;
            float F0 = kfa * fs[0] - R0, F1 = kfa * fs[1] - R1;
            const int rank = c.bnd_rank[v];
            if (rank >= 0) {
                const int slot = atomicAdd(&s_nbnd, 1);
                if (slot < kBndSlots) {
                    float* b = s_bnd + 8 * slot;
                    b[0] = __int_as_float(i); b[1] = F0; b[2] = F1; b[3] = Q0;
                    b[4] = Q1; b[5] = Q2; b[6] = Q3; b[7] = MMf;
                    continue;
                }
                boundary_force(c, a, pt, X, xp, v, rank, ap_call, F0, F1);   // queue full: finish in place
            }
            finish_vertex(c, a, par, v, F0, F1, Q0, Q1, Q2, Q3, MMf);
        }
        __syncthreads();
        const int nq = min(s_nbnd, kBndSlots);
        for (int j = threadIdx.x; j < nq; j += blockDim.x) {
            const float* b = s_bnd + 8 * j;
            const int v = pt.x + __float_as_int(b[0]);
            float F0 = b[1], F1 = b[2];
            boundary_force(c, a, pt, X, xp, v, c.bnd_rank[v], ap_call, F0, F1);
            finish_vertex(c, a, par, v, F0, F1, b[3], b[4], b[5], b[6], b[7]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned int done = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 1), 1u);
            if ((int)done == c.np - 1) {
                c.ctl[1] = 0;
                c.ctl[0] = par ^ 1;
                c.clk[0] = c.clk[0] + a.dt_real;
                c.ap[0] = ap_call + 1ull;
            }
        }
    }
}

// ===========================================================================
// mixed-form vertex phase: predict (FP64), bond kinetics with FP32 rates and
// FP64 accumulation, the FP32 element records, and the cell area and
// area-weighted centroid from the boundary loop (shoelace over the directed
// boundary edges).  For a planar mesh without inverted elements that equals
// calculateAreaTot's sum of element areas.
// ===========================================================================
enum { VM_PREDICT = 1, VM_UPDATE_FA = 2, VM_EXPORT = 8, VM_IMPORT = 16, VM_NOAREA = 32 };

__device__ __forceinline__ void predict_mixed(const double4& X, const double4& V, const double4& A, double dt,
                                              double hdt, double vh[2], double xn[3]) {
    vh[0] = fma(hdt, A.x, V.x);
    vh[1] = fma(hdt, A.y, V.y);
    xn[0] = fma(dt, vh[0], X.x);
    xn[1] = fma(dt, vh[1], X.y);
    xn[2] = X.z;  // V_hlf.z = 0 (UL:119)
}

// The cell area and centroid of the mixed form, from the predicted positions of
// the boundary loop (shoelace over the directed boundary edges).  The last block
// of the cell to finish (ticket ctl[2]) reads the positions the other blocks
// wrote (through L2) and sums the terms in a fixed order: boundary ranks strided
// over the threads, then lanes, then warps.  Only that block runs the FP64
// shoelace, with all of its lanes busy.
__device__ __forceinline__ void finish_area_boundary(const CellDev& c, const double4* xo) {
    __shared__ int s_last;
    __shared__ double s_w[kK1Threads / 32][3];
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 2), 1u);
        s_last = ((int)t == c.nk1 - 1);
    }
    __syncthreads();
    if (!s_last) return;   // block-uniform
    __threadfence();
    double s0 = 0, s1 = 0, s2 = 0;
    for (int r = threadIdx.x; r < c.nb; r += blockDim.x) {
        const double2 xi = __ldcg(reinterpret_cast<const double2*>(xo + c.bnd_vert[r]));
        for (int k = c.bnd_optr[r]; k < c.bnd_optr[r + 1]; ++k) {
            const double2 xj = __ldcg(reinterpret_cast<const double2*>(xo + c.bnd_out[k]));
            const double cr = xi.x * xj.y - xj.x * xi.y;
            s0 += 0.5 * cr;
            s1 += (1.0 / 6.0) * (xi.x + xj.x) * cr;
            s2 += (1.0 / 6.0) * (xi.y + xj.y) * cr;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    const int wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_w[wid][0] = s0; s_w[wid][1] = s1; s_w[wid][2] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double A = 0, Ax = 0, Ay = 0;
        for (int w = 0; w < nw; ++w) {
            A += s_w[w][0]; Ax += s_w[w][1]; Ay += s_w[w][2];
        }
        c.area4[0] = A;
        c.area4[1] = Ax / A;
        c.area4[2] = Ay / A;
        c.area4[3] = 0.0;
        c.ctl[2] = 0;
    }
}

// One block per work item (a block of c.vb consecutive vertices of one cell).
__global__ void __launch_bounds__(kK1Threads, 3) k_vertex_phase_mixed(const CellDev* __restrict__ cells,
                                                                    const WorkItem* __restrict__ work,
                                                                    double dt, double hdt, float dtf, int flags,
                                                                    const double* __restrict__ stage_in,
                                                                    double* __restrict__ stage_out) {
    const WorkItem it = work[blockIdx.x];
    const CellDev& c = cells[it.cell];
    const int v = it.idx * c.vb + threadIdx.x;
    if (v < c.nv) {
        const int par = c.ctl[0];
        const double4* __restrict__ X = c.pos[par];
        double4* __restrict__ xo = c.pos[par ^ 1];
        const double4 Xv = ld4(X + v);
        double xn[3];
        if (flags & VM_IMPORT) {
            const double* qq = stage_in + 3 * (size_t)(c.hoff + v);
            xn[0] = qq[0]; xn[1] = qq[1]; xn[2] = qq[2];
            st4(xo + v, xn[0], xn[1], xn[2]);
        } else if (flags & VM_PREDICT) {
            double vh[2];
            predict_mixed(Xv, ld4(c.vel + v), ld4(c.acc + v), dt, hdt, vh, xn);
            st4(xo + v, xn[0], xn[1], xn[2]);
            if (flags & VM_EXPORT) {
                st4(c.vhl + v, vh[0], vh[1], 0.0);
                double* qq = stage_out + 3 * (size_t)(c.hoff + v);
                qq[0] = xn[0]; qq[1] = xn[1]; qq[2] = xn[2];
            }
        } else {
            const double4 t = ld4v(xo + v);
            xn[0] = t.x; xn[1] = t.y; xn[2] = t.z;
        }
        const double cu0 = xn[0] - Xv.x, cu1 = xn[1] - Xv.y;  // exact differences
        if (flags & VM_UPDATE_FA) {
            const ParamF& pf = c.pf;
            const double4 f = ld4(c.fau + v);
            const double cold = c.cC[v], cAv = c.cA[v];
            double u0 = f.x + cu0, u1 = f.y + cu1, u2 = f.z;
            if (c.has_sub && c.sub.moving) {
                double wgt[3];
                const int e = locate(c.sub, xs(Xv.x, f.x), xs(Xv.y, f.y), xs(Xv.z, f.z), wgt);
                if (e >= 0) {
                    const int4 t = c.sub.tri[e];
                    const double4 a0 = ld4(c.sub.x + t.x), a1 = ld4(c.sub.x + t.y), a2 = ld4(c.sub.x + t.z);
                    const double4 b0 = ld4(c.sub.X + t.x), b1 = ld4(c.sub.X + t.y), b2 = ld4(c.sub.X + t.z);
                    u0 -= wgt[0] * (a0.x - b0.x) + wgt[1] * (a1.x - b1.x) + wgt[2] * (a2.x - b2.x);
                    u1 -= wgt[0] * (a0.y - b0.y) + wgt[1] * (a1.y - b1.y) + wgt[2] * (a2.y - b2.y);
                    u2 -= wgt[0] * (a0.z - b0.z) + wgt[1] * (a1.z - b1.z) + wgt[2] * (a2.z - b2.z);
                }
            }
            float fs[3], force;
            spring_force32(pf, f64_to_f32_rn(u0), f64_to_f32_rn(u1), f64_to_f32_rn(u2), fs, &force);
            const float koff = pf.ka * __expf(force * pf.iFa) + pf.kb * __expf(-force * pf.iFb);
            const float coldf = f64_to_f32_rn(cold), kon = pf.k_on;
            double cn = cold + f32_to_f64(dtf * (kon * (1.0f - coldf) - koff * coldf));
            if (dneg(cn)) cn = 0;
            if (dneg(cAv)) c.cA[v] = 0;
            double n0, n1, n2;
            const bool keep_pos = dpos(cold) && (1.0f - dtf * koff) > 0.0f;
            if (keep_pos && dpos(cn)) {
                // keep / c_new = 1 + ds with ds = -dt k_on (1 - c_old) / c_new exactly
                const double ds = f32_to_f64(-dtf * kon * (1.0f - coldf) / f64_to_f32_rn(cn));
                n0 = fma(u0, ds, u0); n1 = fma(u1, ds, u1); n2 = fma(u2, ds, u2);
            } else {
                n0 = 0.0 * u0; n1 = 0.0 * u1; n2 = 0.0 * u2;
            }
            c.cC[v] = cn;
            st4(c.fau + v, n0, n1, n2);
        }
        if (!(flags & VM_EXPORT)) {
            const double2* e2 = reinterpret_cast<const double2*>(c.ea[par] + 6 * (size_t)v);
            const double2 q0 = __ldg(e2), q1 = __ldg(e2 + 1);  // (xx, yy), (zz, xy)
            const float hx = f64_to_f32_rn(Xv.x), hy = f64_to_f32_rn(Xv.y);
            const float lx = f64_to_f32_rn(Xv.x - f32_to_f64(hx)), ly = f64_to_f32_rn(Xv.y - f32_to_f64(hy));
            float4* r = c.rec + kRec * (size_t)v;
            r[0] = make_float4(hx, hy, lx, ly);
            r[1] = make_float4(f64_to_f32_rn(cu0), f64_to_f32_rn(cu1), f64_to_f32_rn(q0.x), f64_to_f32_rn(q0.y));
            r[2] = make_float4(f64_to_f32_rn(q1.y), f64_to_f32_rn(q1.x), 0.0f, 0.0f);
        }
        // boundary positions are read by the block that finishes the area
        if (!(flags & VM_NOAREA) && c.bnd_rank[v] >= 0) __threadfence();
    }
    if (!(flags & VM_NOAREA)) finish_area_boundary(c, c.pos[c.ctl[0] ^ 1]);
}

void launch_vertex_mixed(const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
                         int threads, cudaStream_t st, const double* stage_in, double* stage_out) {
    if (nwork <= 0) return;
    (void)grid;   // one block per work item
    k_vertex_phase_mixed<<<nwork, threads, 0, st>>>(cells, work, dt, dt / 2.0, (float)dt, flags, stage_in, stage_out);
}

size_t mixed_smem_bytes(int emax) { return sizeof(float) * (size_t)emax * kSlot32; }

cudaError_t configure_mixed(size_t max_smem) {
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, (const void*)k_patch_phase_mixed);
    if (e != cudaSuccess) return e;
    size_t dyn = max_smem > at.sharedSizeBytes ? max_smem - at.sharedSizeBytes : 0;
    return cudaFuncSetAttribute((const void*)k_patch_phase_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

int mixed_occupancy(int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, (const void*)k_patch_phase_mixed, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

void launch_patch_mixed(const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt, double dt_real,
                        double ap_thresh, double t_override, int vh_from_buf, int threads, int grid, cudaStream_t st) {
    if (nwork <= 0) return;
    MixedArgs a;
    a.cells = cells;
    a.work = work;
    a.nwork = nwork;
    a.emax = emax;
    a.dt = dt;
    a.dt_real = dt_real;
    a.hdt = dt / 2.0;
    a.cdt = dt_real - dt / 2.0;
    a.half = dt_real > dt / 2.0;
    a.ap_thresh = ap_thresh;
    a.t_override = t_override;
    a.vh_from_buf = vh_from_buf;
    k_patch_phase_mixed<<<grid, threads, mixed_smem_bytes(emax), st>>>(a);
}

}  // namespace wcfe
