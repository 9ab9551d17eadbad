// wcfe_mixed.cu — the mixed-precision patch phase (WCFE_PREC_MIXED).
//
// Element assembly runs in FP32 in an increment form of evalElementRe
// (UL:710-928); the state, the per-vertex accumulation of boundary terms and
// the explicit update stay in FP64.  With F = I + H, E the nodal-average
// strain and P = I - N N, the reference's stress is rewritten exactly as
//     S_pas = mu [c0 P + beta / theta_g - theta_g (1 + eta) gamma]
//     beta  = be_t - I   = 2 E (I - 2E)^-1
//     gamma = C^-1 - I   = -c C^-1,  c = H + H^T + H^T H
//     eta   = lambda_N^2 - 1 = (theta_g^2 (1 + de) - (1 + dth)^2) / (1 + dth)^2
//     c0    = -(theta_g^2 - 1 + theta_g^2 eta) / theta_g
// (de = det(I - 2E) - 1 and dth = det F - 1 from the invariants), so every
// FP32 quantity is a small number carried at full relative precision instead
// of a difference of two O(1) numbers.  The isotropic part kappa t_act I of the
// active stress contributes w b_i per element corner; on a closed one-ring
// these sum to exactly zero, so it is left out of the FP32 element and added in
// FP64 for boundary vertices as (1/2) kappa t_act thick N x (X_end - X_start)
// summed over the one-ring.  The strain update uses K = F^-1 - I = -H F^-1:
//     ea_s = E + K^T E + E K + K^T E K - (K + K^T + K^T K)/2     (theta_g = 1)
//
// The element inputs come from a per-vertex FP32 record written by the vertex
// phase: positions as float-float (hi, lo), the step displacement u = x - X,
// and the strain, so the element loop performs no FP64 arithmetic at all.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "wcfe_common.cuh"

namespace wcfe {

struct PatchArgs;  // defined in wcfe_kernels.cu; the mixed kernel takes its own argument block

struct MixedArgs {
    const CellDev* cells;
    const WorkItem* work;
    int nwork, emax;
    double dt, dt_real, hdt, ap_thresh, t_override;
    int vh_from_buf;
};


// 3x3 helpers in FP32 (row-major)
__device__ __forceinline__ void adj3f(const float m[9], float o[9], float* det) {
    float c00 = m[4] * m[8] - m[5] * m[7];
    float c10 = m[5] * m[6] - m[3] * m[8];
    float c20 = m[3] * m[7] - m[4] * m[6];
    *det = c00 * m[0] + c10 * m[1] + c20 * m[2];
    o[0] = c00; o[3] = c10; o[6] = c20;
    o[1] = m[2] * m[7] - m[1] * m[8];
    o[4] = m[0] * m[8] - m[2] * m[6];
    o[7] = m[1] * m[6] - m[0] * m[7];
    o[2] = m[1] * m[5] - m[2] * m[4];
    o[5] = m[2] * m[3] - m[0] * m[5];
    o[8] = m[0] * m[4] - m[1] * m[3];
}
__device__ __forceinline__ void mm3f(const float a[9], const float b[9], float o[9]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) o[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
}
// det(I + M) - 1 from the invariants of M
__device__ __forceinline__ float detp1m1(const float m[9]) {
    float tr = m[0] + m[4] + m[8];
    float i2 = (m[0] * m[4] - m[1] * m[3]) + (m[0] * m[8] - m[2] * m[6]) + (m[4] * m[8] - m[5] * m[7]);
    float d = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
    return tr + i2 + d;
}

// per-vertex record: float4 r0 = (Xhi.x, Xhi.y, Xhi.z, u.x), r1 = (Xlo.x, Xlo.y, Xlo.z, u.y),
//                    r2 = (u.z, ea0, ea1, ea2), r3 = (ea3, ea4, ea5, 0)
struct ElemOut32 {
    float re[3][3];
    float rea[3][6];
    float mm, acur;
};

__device__ __forceinline__ void element_mixed(const float4 r[3][4], const wcfe_params& p, float mu, float s_iso,
                                              float t_an, float grow, const float cen[3], ElemOut32& o) {
    float Xh[3][3], Xl[3][3], u[3][3], ea[3][6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        Xh[k][0] = r[k][0].x; Xh[k][1] = r[k][0].y; Xh[k][2] = r[k][0].z;
        Xl[k][0] = r[k][1].x; Xl[k][1] = r[k][1].y; Xl[k][2] = r[k][1].z;
        u[k][0] = r[k][0].w; u[k][1] = r[k][1].w; u[k][2] = r[k][2].x;
        ea[k][0] = r[k][2].y; ea[k][1] = r[k][2].z; ea[k][2] = r[k][2].w;
        ea[k][3] = r[k][3].x; ea[k][4] = r[k][3].y; ea[k][5] = r[k][3].z;
    }
    float G1[3], G2[3], d1[3], d2[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        G1[k] = (Xh[1][k] - Xh[0][k]) + (Xl[1][k] - Xl[0][k]);
        G2[k] = (Xh[2][k] - Xh[0][k]) + (Xl[2][k] - Xl[0][k]);
        d1[k] = u[1][k] - u[0][k];
        d2[k] = u[2][k] - u[0][k];
    }
    float Gc[3] = {G1[1] * G2[2] - G1[2] * G2[1], G1[2] * G2[0] - G1[0] * G2[2], G1[0] * G2[1] - G1[1] * G2[0]};
    float nG = sqrtf(Gc[0] * Gc[0] + Gc[1] * Gc[1] + Gc[2] * Gc[2]);
    float inG = 1.0f / nG;
    float N[3] = {Gc[0] * inG, Gc[1] * inG, Gc[2] * inG};
    // dual basis: G1inv = (G2 x N)/|GxG|, G2inv = (N x G1)/|GxG|
    float b1[3] = {(G2[1] * N[2] - G2[2] * N[1]) * inG, (G2[2] * N[0] - G2[0] * N[2]) * inG, (G2[0] * N[1] - G2[1] * N[0]) * inG};
    float b2[3] = {(N[1] * G1[2] - N[2] * G1[1]) * inG, (N[2] * G1[0] - N[0] * G1[2]) * inG, (N[0] * G1[1] - N[1] * G1[0]) * inG};
    float g1[3] = {G1[0] + d1[0], G1[1] + d1[1], G1[2] + d1[2]};
    float g2[3] = {G2[0] + d2[0], G2[1] + d2[1], G2[2] + d2[2]};
    float gc[3] = {g1[1] * g2[2] - g1[2] * g2[1], g1[2] * g2[0] - g1[0] * g2[2], g1[0] * g2[1] - g1[1] * g2[0]};
    float ng = sqrtf(gc[0] * gc[0] + gc[1] * gc[1] + gc[2] * gc[2]);
    // n - N = dgc/ng - Gc (ng - nG)/(ng nG) with ng - nG = dgc.(gc + Gc)/(ng + nG): no cancellation
    float dgc[3] = {gc[0] - Gc[0], gc[1] - Gc[1], gc[2] - Gc[2]};
    float ing = 1.0f / ng;
    float dng = (dgc[0] * (gc[0] + Gc[0]) + dgc[1] * (gc[1] + Gc[1]) + dgc[2] * (gc[2] + Gc[2])) / (ng + nG);
    float dn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dn[k] = dgc[k] * ing - Gc[k] * (dng * ing * inG);
    float H[9];
#pragma unroll
    for (int rr = 0; rr < 3; ++rr)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) H[rr * 3 + cc] = d1[rr] * b1[cc] + d2[rr] * b2[cc] + dn[rr] * N[cc];
    // strain at the integration point
    const float third = 1.0f / 3.0f;
    float ev[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) ev[q] = third * (ea[0][q] + ea[1][q] + ea[2][q]);
    float E[9] = {ev[0], ev[3], ev[4], ev[3], ev[1], ev[5], ev[4], ev[5], ev[2]};
    float M2[9], aM[9], dM;
#pragma unroll
    for (int k = 0; k < 9; ++k) M2[k] = -2.0f * E[k];
    M2[0] += 1.0f; M2[4] += 1.0f; M2[8] += 1.0f;
    adj3f(M2, aM, &dM);
    float idM = 1.0f / dM;
    float Minv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Minv[k] = aM[k] * idM;
    float beta[9];
    mm3f(E, Minv, beta);
#pragma unroll
    for (int k = 0; k < 9; ++k) beta[k] *= 2.0f;
    float m2E[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m2E[k] = -2.0f * E[k];
    float de = detp1m1(m2E);
    // C = I + c, c = H + H^T + H^T H
    float cmat[9], Cm[9], aC[9], dC;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            cmat[i * 3 + j] = H[i * 3 + j] + H[j * 3 + i] + (H[i] * H[j] + H[3 + i] * H[3 + j] + H[6 + i] * H[6 + j]);
#pragma unroll
    for (int k = 0; k < 9; ++k) Cm[k] = cmat[k];
    Cm[0] += 1.0f; Cm[4] += 1.0f; Cm[8] += 1.0f;
    adj3f(Cm, aC, &dC);
    float idC = 1.0f / dC;
    float Cinv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Cinv[k] = aC[k] * idC;
    float gam[9];
    mm3f(cmat, Cinv, gam);
#pragma unroll
    for (int k = 0; k < 9; ++k) gam[k] = -gam[k];
    float dth = detp1m1(H);
    const float g = grow;            // theta_g - 1 = thetag_dot dt_real (UL:847)
    const float thg = 1.0f + g;
    float one_dth = 1.0f + dth;
    float eta = ((2.0f * g + g * g) + thg * thg * de - 2.0f * dth - dth * dth) / (one_dth * one_dth);
    float c0 = -((2.0f * g + g * g) + thg * thg * eta) / thg;
    float S[9];
#pragma unroll
    for (int rr = 0; rr < 3; ++rr)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            float P = (rr == cc ? 1.0f : 0.0f) - N[rr] * N[cc];
            S[rr * 3 + cc] = mu * (c0 * P + beta[rr * 3 + cc] / thg - thg * (1.0f + eta) * gam[rr * 3 + cc]);
        }
    // anisotropic active part t_act (1 - 2 kappa) a0 a0^T (zero for kappa = 1/2)
    if (t_an != 0.0f) {
        float a0[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            a0[k] = third * ((Xh[0][k] + Xh[1][k] + Xh[2][k]) + (Xl[0][k] + Xl[1][k] + Xl[2][k]) +
                             (u[0][k] + u[1][k] + u[2][k])) - cen[k];
        float ia = rsqrtf(a0[0] * a0[0] + a0[1] * a0[1] + a0[2] * a0[2]);
#pragma unroll
        for (int rr = 0; rr < 3; ++rr)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) S[rr * 3 + cc] += t_an * (a0[rr] * ia) * (a0[cc] * ia);
    }
    // T = s_iso H + (I + H) S   (the isotropic part s_iso I is handled per vertex in FP64)
    float HS[9];
    mm3f(H, S, HS);
    float T[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) T[k] = s_iso * H[k] + S[k] + HS[k];
    const float wA = 0.5f * nG * (float)p.thick;
    float b0[3] = {-b1[0] - b2[0], -b1[1] - b2[1], -b1[2] - b2[2]};
    const float* bb[3] = {b0, b1, b2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) o.re[i][rr] = wA * (T[rr * 3] * bb[i][0] + T[rr * 3 + 1] * bb[i][1] + T[rr * 3 + 2] * bb[i][2]);
    // strain: K = F^-1 - I = -H F^-1
    float Fm[9], aF[9], dF;
#pragma unroll
    for (int k = 0; k < 9; ++k) Fm[k] = H[k];
    Fm[0] += 1.0f; Fm[4] += 1.0f; Fm[8] += 1.0f;
    adj3f(Fm, aF, &dF);
    float idF = 1.0f / dF;
    float Finv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Finv[k] = aF[k] * idF;
    float K[9];
    mm3f(H, Finv, K);
#pragma unroll
    for (int k = 0; k < 9; ++k) K[k] = -K[k];
    float EK[9], KtE[9], KtEK[9], KtK[9];
    mm3f(E, K, EK);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            KtE[i * 3 + j] = K[i] * E[j] + K[3 + i] * E[3 + j] + K[6 + i] * E[6 + j];
            KtK[i * 3 + j] = K[i] * K[j] + K[3 + i] * K[3 + j] + K[6 + i] * K[6 + j];
        }
    mm3f(KtE, K, KtEK);
    float D[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            D[i * 3 + j] = KtE[i * 3 + j] + EK[i * 3 + j] + KtEK[i * 3 + j] - 0.5f * (K[i * 3 + j] + K[j * 3 + i] + KtK[i * 3 + j]);
    // theta_g != 1: ea_s = (1 - thg^2)/2 I + thg^2 (E + D), written as E + [(1 - thg^2)/2 I + (thg^2 - 1) E + thg^2 D]
    const float tg2 = thg * thg, gg = tg2 - 1.0f;
    float dv[6] = {tg2 * D[0] + gg * (ev[0] - 0.5f), tg2 * D[4] + gg * (ev[1] - 0.5f), tg2 * D[8] + gg * (ev[2] - 0.5f),
                   tg2 * D[1] + gg * ev[3], tg2 * D[2] + gg * ev[4], tg2 * D[5] + gg * ev[5]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 6; ++q) o.rea[i][q] = third * wA * ((ev[q] - ea[i][q]) + dv[q]);
    o.mm = third * wA;
    o.acur = 0.5f * ng;
}

constexpr int kSlot32 = 29;

__global__ void __launch_bounds__(128) k_patch_phase_mixed(MixedArgs a) {
    extern __shared__ float smf[];
    const int emax = a.emax;
    float* s_re = smf;
    float* s_rea = s_re + 9 * emax;
    float* s_mm = s_rea + 18 * emax;
    float* s_ac = s_mm + emax;
    __shared__ double s_red[4];
    for (int w = blockIdx.x; w < a.nwork; w += gridDim.x) {
        const WorkItem it = a.work[w];
        const CellDev& c = a.cells[it.cell];
        const wcfe_params& p = c.prm;
        const int4 pt = c.patch[it.idx];
        const int par = c.ctl[0];
        const double4* __restrict__ X = c.pos[par];
        const double4* __restrict__ xp = c.pos[par ^ 1];
        const float4* __restrict__ rec = c.rec;
        if (threadIdx.x < 32) {
            double s4[4] = {0, 0, 0, 0};
            for (int k = threadIdx.x; k < c.nk1; k += 32)
#pragma unroll
                for (int q = 0; q < 4; ++q) s4[q] += c.k1_part[4 * k + q];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s4[q] += __shfl_xor_sync(0xffffffffu, s4[q], o);
            if (threadIdx.x == 0) {
                s_red[0] = s4[0];
                s_red[1] = s4[1] / s4[0]; s_red[2] = s4[2] / s4[0]; s_red[3] = s4[3] / s4[0];
            }
        }
        __syncthreads();
        const double area_tot = s_red[0];
        const float cen[3] = {(float)s_red[1], (float)s_red[2], (float)s_red[3]};
        const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
        const unsigned long long ap_call = c.ap[0];
        const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
        const double s_iso = p.kappa * t_act;
        const float t_an = (float)((1.0 - 2.0 * p.kappa) * t_act);
        for (int j = threadIdx.x; j < pt.w; j += blockDim.x) {
            const int e = c.patch_elems[pt.z + j];
            const int4 t4 = __ldg(c.tri + e);
            const int id[3] = {t4.x, t4.y, t4.z};
            float4 r[3][4];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int q = 0; q < 4; ++q) r[k][q] = rec[4 * (size_t)id[k] + q];
            ElemOut32 o;
            element_mixed(r, p, (float)p.mu, (float)s_iso, t_an, (float)(p.thetag_dot * a.dt_real), cen, o);
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int rr = 0; rr < 3; ++rr) s_re[j * 9 + k * 3 + rr] = o.re[k][rr];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int q = 0; q < 6; ++q) s_rea[j * 18 + k * 6 + q] = o.rea[k][q];
            s_mm[j] = o.mm;
            s_ac[j] = o.acur;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            float R[3] = {0, 0, 0}, Rq[6] = {0, 0, 0, 0, 0, 0}, MMf = 0, Asf = 0;
            for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                const int code = c.vc_code[k];
                const int sl = code >> 2, cn = code & 3;
#pragma unroll
                for (int r = 0; r < 3; ++r) R[r] += s_re[sl * 9 + cn * 3 + r];
#pragma unroll
                for (int q = 0; q < 6; ++q) Rq[q] += s_rea[sl * 18 + cn * 6 + q];
                MMf += s_mm[sl];
                Asf += s_ac[sl];
            }
            const double MM = (double)MMf;
            const double Asum = (double)Asf / 3.0;
            const double4 xv4 = ld4v(xp + v);
            const double xi[3] = {xv4.x, xv4.y, xv4.z};
            double Rd[3] = {(double)R[0], (double)R[1], (double)R[2]};
            const double4 f4 = ld4v(c.fau + v);
            double fs[3], bell;
            spring_force(p, f4.x, f4.y, f4.z, fs, &bell);
            const double rho = c.rho_w ? c.rho_w[v] : p.rho_i_max;
            const double cCv = c.cC[v];
            double Ffa[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) Ffa[r] = -cCv * fs[r] * Asum * rho;
            double Fap[3] = {0, 0, 0}, Fb[3] = {0, 0, 0}, Far[3] = {0, 0, 0};
            const int rank = c.bnd_rank[v];
            if (rank >= 0) {
                // isotropic active stress on the open one-ring: (1/2) s_iso thick sum N x (X_k - X_j)
                double sx = 0, sy = 0, sz = 0;
                for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                    const int code = c.vc_code[k];
                    const int cn = code & 3;
                    const int e = c.patch_elems[pt.z + (code >> 2)];
                    const int4 t4 = c.tri[e];
                    const int ids[3] = {t4.x, t4.y, t4.z};
                    const double4 Xi = ld4v(X + ids[cn]);
                    const double4 Xj = ld4v(X + ids[(cn + 1) % 3]), Xk = ld4v(X + ids[(cn + 2) % 3]);
                    // orientation of the element (its normal N = +-e3 for a planar membrane)
                    const double oz = (Xj.x - Xi.x) * (Xk.y - Xi.y) - (Xj.y - Xi.y) * (Xk.x - Xi.x);
                    const double sg = oz >= 0 ? 1.0 : -1.0;
                    sx += sg * (Xk.x - Xj.x); sy += sg * (Xk.y - Xj.y); sz += sg * (Xk.z - Xj.z);
                }
                // planar membrane: N = e3, so N x (sx, sy) = (-sy, sx)
                const double w = 0.5 * s_iso * p.thick;
                Rd[0] += w * (-sy);
                Rd[1] += w * sx;
                (void)sz;
                double x1[3], x2[3];
                if (boundary_frame(c, xp, rank, xi, x1, x2)) {
                    double d1[3] = {xi[0] - x1[0], xi[1] - x1[1], xi[2] - x1[2]};
                    double d2[3] = {x2[0] - xi[0], x2[1] - xi[1], x2[2] - xi[2]};
                    double n1[3] = {d1[1], -d1[0], 0.0}, n2[3] = {d2[1], -d2[0], 0.0};
                    double nn1 = sqrt(n1[0] * n1[0] + n1[1] * n1[1]), nn2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1]);
                    double l1 = sqrt(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]);
                    double l2 = sqrt(d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2]);
                    double L = l1 + l2;
                    double nrm[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r) nrm[r] = l1 / L * (n1[r] / nn1) + l2 / L * (n2[r] / nn2);
                    if (p.ap_enable) {
                        uint32_t r31 = ap_draw(p.seed, p.stream, ap_call, (uint32_t)rank);
                        double Pr = (double)r31 / ((double)2147483647 + 1.);
                        double lim = p.ap_density * L / 2;
                        double cnt = lim > 0 ? ceil(lim) : 0.0;
                        const double apt = isnan(a.ap_thresh) ? c.ap_thresh : a.ap_thresh;
                        double fsc = (Pr < apt) ? p.ap_force * cnt : 0.0;
#pragma unroll
                        for (int r = 0; r < 3; ++r) Fap[r] = fsc * nrm[r];
                    }
                    double ed1[3] = {d1[0] / l1, d1[1] / l1, d1[2] / l1}, ed2[3] = {d2[0] / l2, d2[1] / l2, d2[2] / l2};
                    double cost = ed1[0] * ed2[0] + ed1[1] * ed2[1] + ed1[2] * ed2[2];
                    double ez = xs(xm(ed1[0], ed2[1]), xm(ed1[1], ed2[0]));
                    double turna = ez > 0 ? cost - 1 : 1 - cost;
                    double kap = turna * 2 / L;
#pragma unroll
                    for (int r = 0; r < 3; ++r) Fb[r] = p.k_bend * kap * nrm[r];
                    double sc = -p.k_area * (area_tot - p.area0) / 2 * L;
#pragma unroll
                    for (int r = 0; r < 3; ++r) Far[r] = sc * nrm[r];
                }
            }
            const double4 V4 = ld4v(c.vel + v), A4 = ld4v(c.acc + v);
            double vh[3];
            if (a.vh_from_buf) {
                double4 h = ld4v(c.vhl + v);
                vh[0] = h.x; vh[1] = h.y; vh[2] = h.z;
            } else {
                const double4 Xv = ld4v(X + v);
                vh[0] = xa(V4.x, xm(a.hdt, A4.x));
                vh[1] = xa(V4.y, xm(a.hdt, A4.y));
                vh[2] = 0.0;
                (void)Xv;
            }
            const double Vo[3] = {V4.x, V4.y, V4.z};
            double An[3], Vn[3];
            const double md = p.damp * MM * p.rho, mr = MM * p.rho;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                double f = -p.drag * vh[r] + Fb[r] + Fap[r] + Ffa[r] + Far[r] - Rd[r];
                An[r] = (f - md * Vo[r]) / mr;
            }
            const bool half = a.dt_real > a.dt / 2.0;
#pragma unroll
            for (int r = 0; r < 3; ++r) Vn[r] = half ? vh[r] + (a.dt_real - a.dt / 2.0) * An[r] : Vo[r] + a.dt_real * An[r];
            const double* eao = c.ea[par] + 6 * (size_t)v;
            double* en = c.ea[par ^ 1] + 6 * (size_t)v;
            const float iM = 1.0f / MMf;
            double chk = 0;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                double nv = eao[q] + (double)(Rq[q] * iM);
                en[q] = nv;
                chk += nv;
            }
            st4(c.acc + v, An[0], An[1], An[2]);
            st4(c.vel + v, Vn[0], Vn[1], Vn[2]);
            chk += An[0] + An[1] + An[2] + Vn[0] + Vn[1] + Vn[2] + xi[0] + xi[1];
            if (!isfinite(chk)) atomicOr(c.status, 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            unsigned int done = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 1), 1u);
            if ((int)done == c.np - 1) {
                c.ctl[1] = 0;
                c.ctl[0] = par ^ 1;
                c.clk[0] = c.clk[0] + a.dt_real;
                c.ap[0] = ap_call + 1ull;
            }
        }
    }
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
    a.ap_thresh = ap_thresh;
    a.t_override = t_override;
    a.vh_from_buf = vh_from_buf;
    k_patch_phase_mixed<<<grid, threads, mixed_smem_bytes(emax), st>>>(a);
}

}  // namespace wcfe
