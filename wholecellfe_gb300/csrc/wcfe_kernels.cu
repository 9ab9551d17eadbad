// wcfe_kernels.cu — sm_103a kernels of the explicit mechanics step.
//
// One step of every live cell is two launches over flat work lists that mix
// all cells (uneven sizes welcome):
//
//   k_vertex_phase  (block = 256 vertices + 512 elements of one cell)
//       A1 predict  (driverVelocities_Explicit UL:103-124, main.cpp:227-231)
//       A5 bond kinetics (updateFA UL:2026-2174) with grid point location
//       A2 per-block partial sums of area and area-weighted centroid (calculateAreaTot UL:1662-1688)
//   k_patch_phase   (block = one patch: a contiguous vertex range + every element touching it)
//       A3 element residuals (evalElementRe UL:710-928) staged in shared memory,
//          gathered per vertex in the mesh's one-ring order: deterministic, no atomics
//       A4 integrin force (calculateForce_FA UL:1198-1303)
//       A6-A8 boundary forces (UL:1477-1784)
//       A9 explicit update (updateForces_Explicit UL:567-628)
//
// Decisions the reference makes on floating-point signs (boundary-curve
// orientation UL:1518, turning-angle sign UL:1611, point-in-triangle UL:2086-2091,
// MD-table breakpoints UL:2127-2134) use unfused round-to-nearest operations,
// so they are made exactly as the oracle makes them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "wcfe_common.cuh"

namespace wcfe {

// ---------------------------------------------------------------------------
// deterministic block reduction of 4 doubles (fixed tree, no atomics)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_sum4(double v[4], double* red /* >= 4*32 */) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < 4; ++k) red[wid * 4 + k] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double s = lane < nw ? red[lane * 4 + k] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            v[k] = s;
        }
    }
}

// ===========================================================================
// vertex phase
// ===========================================================================
enum { VP_PREDICT = 1, VP_UPDATE_FA = 2, VP_RECORD = 4, VP_EXPORT = 8, VP_IMPORT = 16, VP_NOAREA = 32 };

__global__ void __launch_bounds__(kK1Threads) k_vertex_phase(const CellDev* __restrict__ cells,
                                                           const WorkItem* __restrict__ work, int nwork, double dt,
                                                           double hdt, int flags, const double* __restrict__ stage_in,
                                                           double* __restrict__ stage_out) {
    __shared__ double red[4 * 32];
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const CellDev& c = cells[it.cell];
        if (cell_done(c)) continue;   // block-uniform: a serving cell that ran its steps
        const int b = it.idx;
        const int nv = c.nv, nt = c.nt;
        const int par = c.ctl[0];
        double4* __restrict__ X = c.pos[par];
        double4* __restrict__ xo = c.pos[par ^ 1];
        // ---- vertices ----
        const int VB = c.vb;
        const int v = b * VB + threadIdx.x;
        if (v < nv && (int)threadIdx.x < VB) {
            const double4 Xv = ld4(X + v);
            double xn[3];
            if (flags & VP_IMPORT) {
                // positions integrated on the host (El Topo), packed [sum n][3] in cell order
                const double* q = stage_in + 3 * (size_t)(c.hoff + v);
                xn[0] = q[0]; xn[1] = q[1]; xn[2] = q[2];
                st4(xo + v, xn[0], xn[1], xn[2]);
            } else if (flags & VP_PREDICT) {
                double vh[3];
                predict_vertex_c(c, v, Xv, ld4(c.vel + v), ld4(c.acc + v), dt, hdt, vh, xn);
                st4(xo + v, xn[0], xn[1], xn[2]);
                if (flags & VP_EXPORT) {
                    st4(c.vhl + v, vh[0], vh[1], vh[2]);
                    double* q = stage_out + 3 * (size_t)(c.hoff + v);
                    q[0] = xn[0]; q[1] = xn[1]; q[2] = xn[2];
                }
            } else {
                double4 t = ld4v(xo + v);
                xn[0] = t.x; xn[1] = t.y; xn[2] = t.z;
            }
            if ((flags & VP_UPDATE_FA) && c.material != 2) {
                const wcfe_params& p = c.prm;
                double4 f = ld4v(c.fau + v);
                double cu0 = xs(xn[0], Xv.x), cu1 = xs(xn[1], Xv.y), cu2 = xs(xn[2], Xv.z);
                double su0 = 0, su1 = 0, su2 = 0;
                if (c.has_sub && c.sub.scell) {
                    // deformable substrate of the same engine: locate in its step-start positions; its
                    // displacement over the step is its own predict (the same arithmetic as its vertex phase)
                    const CellDev& sc = *c.sub.scell;
                    const double4* __restrict__ Xs = sc.pos[sc.ctl[0]];
                    double wgt[3];
                    int e = locate_in(c.sub, Xs, xs(Xv.x, f.x), xs(Xv.y, f.y), xs(Xv.z, f.z), wgt);
                    if (e >= 0) {
                        int4 t = c.sub.tri[e];
                        const int id[3] = {t.x, t.y, t.z};
                        double d[3][3];
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const double4 Xk = ld4(Xs + id[k]);
                            double vh[3], xk[3];
                            predict_vertex(Xk, ld4(sc.vel + id[k]), ld4(sc.acc + id[k]), dt, hdt, vh, xk);
                            d[k][0] = xk[0] - Xk.x; d[k][1] = xk[1] - Xk.y; d[k][2] = xk[2] - Xk.z;
                        }
                        su0 = wgt[0] * d[0][0] + wgt[1] * d[1][0] + wgt[2] * d[2][0];
                        su1 = wgt[0] * d[0][1] + wgt[1] * d[1][1] + wgt[2] * d[2][1];
                        su2 = wgt[0] * d[0][2] + wgt[1] * d[1][2] + wgt[2] * d[2][2];
                    }
                } else if (c.has_sub && c.sub.moving) {
                    double wgt[3];
                    int e = locate(c.sub, xs(Xv.x, f.x), xs(Xv.y, f.y), xs(Xv.z, f.z), wgt);
                    if (e >= 0) {
                        int4 t = c.sub.tri[e];
                        double4 a0 = ld4(c.sub.x + t.x), a1 = ld4(c.sub.x + t.y), a2 = ld4(c.sub.x + t.z);
                        double4 b0 = ld4(c.sub.X + t.x), b1 = ld4(c.sub.X + t.y), b2 = ld4(c.sub.X + t.z);
                        su0 = wgt[0] * (a0.x - b0.x) + wgt[1] * (a1.x - b1.x) + wgt[2] * (a2.x - b2.x);
                        su1 = wgt[0] * (a0.y - b0.y) + wgt[1] * (a1.y - b1.y) + wgt[2] * (a2.y - b2.y);
                        su2 = wgt[0] * (a0.z - b0.z) + wgt[1] * (a1.z - b1.z) + wgt[2] * (a2.z - b2.z);
                    }
                }
                double u0 = xs(xa(f.x, cu0), su0), u1 = xs(xa(f.y, cu1), su1), u2 = xs(xa(f.z, cu2), su2);
                double fs[3], force;
                spring_force(p, u0, u1, u2, fs, &force);
                double koff = p.ka * exp(force / p.Fa) + p.kb * exp(-force / p.Fb);
                double cold = c.cC[v];
                double cn = cold + dt * p.k_on * (1 - cold) - dt * koff * cold;
                if (cn < 0) cn = 0;
                double ca = c.cA[v];
                if (ca < 0) c.cA[v] = 0;
                double keep = cold - dt * koff * cold;
                if (keep > 0 && cn > 0) {
                    u0 = u0 * keep / cn; u1 = u1 * keep / cn; u2 = u2 * keep / cn;
                } else {
                    u0 = 0.0 * u0; u1 = 0.0 * u1; u2 = 0.0 * u2;
                }
                c.cC[v] = cn;
                st4(c.fau + v, u0, u1, u2);
            }
        }
        if (flags & VP_NOAREA) continue;
        // ---- area and area-weighted centroid of this block's elements ----
        double acc[4] = {0, 0, 0, 0};
        const int e_end = min(nt, (b + 1) * 2 * VB);
        for (int e = b * 2 * VB + threadIdx.x; e < e_end; e += blockDim.x) {
            int4 t = __ldg(c.tri + e);
            double p[3][3];
            const int id[3] = {t.x, t.y, t.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (flags & VP_IMPORT) {
                    const double* q = stage_in + 3 * (size_t)(c.hoff + id[k]);
                    p[k][0] = q[0]; p[k][1] = q[1]; p[k][2] = q[2];
                } else if (flags & VP_PREDICT) {
                    double vh[3];
                    predict_vertex_c(c, id[k], ld4(X + id[k]), ld4(c.vel + id[k]), ld4(c.acc + id[k]), dt, hdt, vh,
                                     p[k]);
                } else {
                    double4 q = ld4v(xo + id[k]);
                    p[k][0] = q.x; p[k][1] = q.y; p[k][2] = q.z;
                }
            }
            double e1x = p[1][0] - p[0][0], e1y = p[1][1] - p[0][1], e1z = p[1][2] - p[0][2];
            double e2x = p[2][0] - p[0][0], e2y = p[2][1] - p[0][1], e2z = p[2][2] - p[0][2];
            double a;
            if (e1z == 0.0 && e2z == 0.0) {
                a = fabs(0.5 * (e1x * e2y - e1y * e2x));  // planar element: the norm of (0, 0, cz) is |cz| exactly
            } else {
                double cx = 0.5 * (e1y * e2z - e1z * e2y), cy = 0.5 * (e1z * e2x - e1x * e2z), cz = 0.5 * (e1x * e2y - e1y * e2x);
                a = sqrt(cx * cx + cy * cy + cz * cz);
            }
            const double third = 1. / 3.;
            acc[0] += a;
            acc[1] += third * (p[0][0] + p[1][0] + p[2][0]) * a;
            acc[2] += third * (p[0][1] + p[1][1] + p[2][1]) * a;
            acc[3] += third * (p[0][2] + p[1][2] + p[2][2]) * a;
        }
        block_sum4(acc, red);
        if (threadIdx.x == 0)
            for (int k = 0; k < 4; ++k) c.k1_part[4 * b + k] = acc[k];
        finish_area(c);
        __syncthreads();
    }
}

// ===========================================================================
// element residual, FP64 (evalElementRe UL:710-928), formulated as
// Re_i = |G1 x G2|/2 * thick * F S b_i with b the reference-configuration
// shape gradients, which equals the reference's S_voigt . varE_voigt.
// ===========================================================================
struct ElemOut64 {
    double re[3][3];
    double rea[3][6];
    double mm;     // lumped mass per corner (UL:914)
    double acur;   // current area |g1 x g2|/2 (the Asum term of UL:1226-1239)
};

__device__ __forceinline__ void inv3(const double m[9], double o[9]) {
    double c00 = m[4] * m[8] - m[5] * m[7];
    double c10 = m[5] * m[6] - m[3] * m[8];
    double c20 = m[3] * m[7] - m[4] * m[6];
    double det = c00 * m[0] + c10 * m[1] + c20 * m[2];  // along row 0 of m with cofactors of column 0 of m^T
    double id = 1.0 / det;
    o[0] = c00 * id; o[3] = c10 * id; o[6] = c20 * id;
    o[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    o[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    o[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}
__device__ __forceinline__ double det3(const double m[9]) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

template <bool DIFF>
__device__ __forceinline__ void element_fp64(const double X[3][3], const double x[3][3], const double ea[3][6],
                                             const double* cA3, const double* cC3, const wcfe_params& p, double mu,
                                             double t_act, int isotropic_act, const double cen[3], double dt_real,
                                             ElemOut64& o, double* reA, double* reC) {
    double G1[3], G2[3], N[3], g1[3], g2[3], n[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        G1[k] = X[1][k] - X[0][k]; G2[k] = X[2][k] - X[0][k];
        g1[k] = x[1][k] - x[0][k]; g2[k] = x[2][k] - x[0][k];
    }
    double Gc[3] = {G1[1] * G2[2] - G1[2] * G2[1], G1[2] * G2[0] - G1[0] * G2[2], G1[0] * G2[1] - G1[1] * G2[0]};
    double gc[3] = {g1[1] * g2[2] - g1[2] * g2[1], g1[2] * g2[0] - g1[0] * g2[2], g1[0] * g2[1] - g1[1] * g2[0]};
    double nG = sqrt(Gc[0] * Gc[0] + Gc[1] * Gc[1] + Gc[2] * Gc[2]);
    double ng = sqrt(gc[0] * gc[0] + gc[1] * gc[1] + gc[2] * gc[2]);
    const double inG = 1.0 / nG, ing = 1.0 / ng;
#pragma unroll
    for (int k = 0; k < 3; ++k) { N[k] = Gc[k] * inG; n[k] = gc[k] * ing; }

    const double third = 1.0 / 3.0;
    double ev[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) ev[q] = third * ea[0][q] + third * ea[1][q] + third * ea[2][q];
    double aux[9] = {1.0 - 2.0 * ev[0], -2.0 * ev[3], -2.0 * ev[4], -2.0 * ev[3], 1.0 - 2.0 * ev[1],
                     -2.0 * ev[5], -2.0 * ev[4], -2.0 * ev[5], 1.0 - 2.0 * ev[2]};
    double bet[9];
    inv3(aux, bet);
    double G[9] = {G1[0], G2[0], N[0], G1[1], G2[1], N[1], G1[2], G2[2], N[2]};
    double Gi[9];
    inv3(G, Gi);
    double F[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) F[r * 3 + c] = g1[r] * Gi[c] + g2[r] * Gi[3 + c] + n[r] * N[c];
    double C[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) C[i * 3 + j] = F[i] * F[j] + F[3 + i] * F[3 + j] + F[6 + i] * F[6 + j];
    double Ci[9];
    inv3(C, Ci);
    double theta_e_t = sqrt(det3(bet));
    double theta_g = 1.0 + p.thetag_dot * dt_real;
    double theta = det3(F);
    double theta_e = theta * theta_e_t / theta_g;
    double lamN = 1.0 / theta_e;
    double pr = -mu * (lamN * lamN);
    double S[9];
    double s1 = mu / theta_g, s2 = theta_g * pr;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double nn = N[r] * N[c];
            S[r * 3 + c] = s1 * (bet[r * 3 + c] - nn) + s2 * (Ci[r * 3 + c] - nn);
        }
    if (isotropic_act) {
        S[0] += t_act; S[4] += t_act; S[8] += t_act;
    } else {
        double a0[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) a0[k] = third * (x[0][k] + x[1][k] + x[2][k]) - cen[k];
        double na = sqrt(a0[0] * a0[0] + a0[1] * a0[1] + a0[2] * a0[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) a0[k] = a0[k] / na;
        double kap = p.kappa, an = 1.0 - 2.0 * kap;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) S[r * 3 + c] += t_act * ((r == c ? kap : 0.0) + an * a0[r] * a0[c]);
    }
    // strain update (UL:884-887): ea_s = (I - (F be_t F^T / theta_g^2)^-1) / 2
    double Fb[9], be[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Fb[i * 3 + j] = F[i * 3] * bet[j] + F[i * 3 + 1] * bet[3 + j] + F[i * 3 + 2] * bet[6 + j];
    double sg = 1.0 / (theta_g * theta_g);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) be[i * 3 + j] = sg * (Fb[i * 3] * F[j * 3] + Fb[i * 3 + 1] * F[j * 3 + 1] + Fb[i * 3 + 2] * F[j * 3 + 2]);
    double bei[9];
    inv3(be, bei);
    double eas[6] = {0.5 * (1.0 - bei[0]), 0.5 * (1.0 - bei[4]), 0.5 * (1.0 - bei[8]), -0.5 * bei[1], -0.5 * bei[2], -0.5 * bei[5]};
    // residual: Re_i = w F S b_i
    double FS[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) FS[i * 3 + j] = F[i * 3] * S[j] + F[i * 3 + 1] * S[3 + j] + F[i * 3 + 2] * S[6 + j];
    const double wA = nG / 2.0 * p.thick;
    double b[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { b[1][k] = Gi[k]; b[2][k] = Gi[3 + k]; b[0][k] = -Gi[k] - Gi[3 + k]; }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int r = 0; r < 3; ++r) o.re[i][r] = (FS[r * 3] * b[i][0] + FS[r * 3 + 1] * b[i][1] + FS[r * 3 + 2] * b[i][2]) * wA;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 6; ++q) o.rea[i][q] = third * (eas[q] - ea[i][q]) * wA;
    o.mm = third * wA;
    o.acur = 0.5 * ng;
    if (DIFF) {
        double g[9] = {g1[0], g2[0], n[0], g1[1], g2[1], n[1], g1[2], g2[2], n[2]};
        double gi[9];
        inv3(g, gi);
        double gA[3], gC[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            gA[k] = cA3[0] * gi[k] + cA3[1] * gi[3 + k] + cA3[2] * (-gi[k] - gi[3 + k]);
            gC[k] = cC3[0] * gi[k] + cC3[1] * gi[3 + k] + cC3[2] * (-gi[k] - gi[3 + k]);
        }
        double cAm = third * (cA3[0] + cA3[1] + cA3[2]), cCm = third * (cC3[0] + cC3[1] + cC3[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double gN[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) gN[k] = i == 0 ? (-gi[k] - gi[3 + k]) : (i == 1 ? gi[k] : gi[3 + k]);
            reA[i] = (cAm * third - dt_real * p.D_A * (gA[0] * gN[0] + gA[1] * gN[1] + gA[2] * gN[2])) * wA;
            reC[i] = (cCm * third - dt_real * p.D_C * (gC[0] * gN[0] + gC[1] * gN[1] + gC[2] * gN[2])) * wA;
        }
    }
}

// ===========================================================================
// patch phase
// ===========================================================================
enum { PP_STEP = 0, PP_RESIDUAL = 1, PP_FORCES = 2 };

struct PatchArgs {
    const CellDev* cells;
    const WorkItem* work;
    int nwork, emax;
    double dt, dt_real, hdt, ap_thresh, t_override;
    int vh_from_buf;
    const double* centroid_override;  // residual diagnostics: the caller's centroid (device, 3 doubles)
    double* out0;                     // diagnostics outputs (host layout)
    double* out1;
    double* out2;
    double* out3;
    double* out4;
    int packed;                       // 1: outputs indexed by the cell's offset in the packed arrays (hoff + v)
};

constexpr int kSlot64 = 29;  // re 9, rea 18, mm, acur

template <int MODE>
__global__ void __launch_bounds__(128) k_patch_phase_fp64(PatchArgs a) {
    extern __shared__ double sm[];
    const int emax = a.emax;
    double* s_re = sm;                     // [emax][9]
    double* s_rea = s_re + 9 * emax;       // [emax][18]
    double* s_mm = s_rea + 18 * emax;      // [emax]
    double* s_ac = s_mm + emax;            // [emax]
    double* s_dA = s_ac + emax;            // [emax][3] diffusion (residual diagnostics only)
    double* s_dC = s_dA + (MODE == PP_RESIDUAL ? 3 * emax : 0);
    for (int w = blockIdx.x; w < a.nwork; w += gridDim.x) {
        const WorkItem it = a.work[w];
        const CellDev& c = a.cells[it.cell];
        if (MODE == PP_STEP && cell_done(c)) continue;   // block-uniform
        const wcfe_params& p = c.prm;
        const int4 pt = c.patch[it.idx];
        const int par = c.ctl[0];
        const double4* __restrict__ X = c.pos[par];
        const double4* __restrict__ xp = c.pos[par ^ 1];
        const double* __restrict__ eao = c.ea[par];
        const double area_tot = c.area4[0];
        double cen[3] = {c.area4[1], c.area4[2], c.area4[3]};
        if (MODE == PP_RESIDUAL && a.centroid_override) {
            cen[0] = a.centroid_override[0]; cen[1] = a.centroid_override[1]; cen[2] = a.centroid_override[2];
        }
        const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
        const unsigned long long ap_call = c.ap[0];
        const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
        // ---- elements of the patch -> shared memory ----
        if (MODE != PP_FORCES || true) {
            for (int j = threadIdx.x; j < pt.w; j += blockDim.x) {
                const int e = c.patch_elems[pt.z + j];
                const int4 t4 = __ldg(c.tri + e);
                const int id[3] = {t4.x, t4.y, t4.z};
                double Xe[3][3], xe[3][3], ee[3][6], cA3[3], cC3[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    double4 q = ld4(X + id[k]);
                    Xe[k][0] = q.x; Xe[k][1] = q.y; Xe[k][2] = q.z;
                    double4 r = ld4v(xp + id[k]);
                    xe[k][0] = r.x; xe[k][1] = r.y; xe[k][2] = r.z;
                    const double2* e2 = reinterpret_cast<const double2*>(eao + 6 * (size_t)id[k]);
                    double2 u0 = __ldg(e2), u1 = __ldg(e2 + 1), u2 = __ldg(e2 + 2);
                    ee[k][0] = u0.x; ee[k][1] = u0.y; ee[k][2] = u1.x; ee[k][3] = u1.y; ee[k][4] = u2.x; ee[k][5] = u2.y;
                    if (MODE == PP_RESIDUAL) { cA3[k] = c.cA[id[k]]; cC3[k] = c.cC[id[k]]; }
                }
                ElemOut64 o;
                double rA[3], rC[3];
                const double mu_el = c.mu_e ? c.mu_e[e] : p.mu;
                // substrate (mat 2, UL:989-1176): no active stress
                element_fp64<MODE == PP_RESIDUAL>(Xe, xe, ee, cA3, cC3, p, mu_el, c.material == 2 ? 0.0 : t_act,
                                                  c.material == 2 ? 1 : 0, cen, a.dt_real, o, rA, rC);
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int r = 0; r < 3; ++r) s_re[j * 9 + k * 3 + r] = o.re[k][r];
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int q = 0; q < 6; ++q) s_rea[j * 18 + k * 6 + q] = o.rea[k][q];
                s_mm[j] = o.mm;
                s_ac[j] = o.acur;
                if (MODE == PP_RESIDUAL) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) { s_dA[j * 3 + k] = rA[k]; s_dC[j * 3 + k] = rC[k]; }
                }
            }
        }
        __syncthreads();
        // ---- owned vertices ----
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            double R[3] = {0, 0, 0}, Rq[6] = {0, 0, 0, 0, 0, 0}, MM = 0, Asum = 0, dA = 0, dC = 0;
            for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                const int code = c.vc_code[k];
                const int sl = code >> 2, cn = code & 3;
#pragma unroll
                for (int r = 0; r < 3; ++r) R[r] += s_re[sl * 9 + cn * 3 + r];
#pragma unroll
                for (int q = 0; q < 6; ++q) Rq[q] += s_rea[sl * 18 + cn * 6 + q];
                MM += s_mm[sl];
                Asum += s_ac[sl] / 3;
                if (MODE == PP_RESIDUAL) { dA += s_dA[sl * 3 + cn]; dC += s_dC[sl * 3 + cn]; }
            }
            const size_t ov = a.packed ? (size_t)c.hoff + v : (size_t)v;   // output row
            if (MODE == PP_RESIDUAL) {
                if (a.out0) for (int r = 0; r < 3; ++r) a.out0[3 * ov + r] = R[r];
                if (a.out1) for (int q = 0; q < 6; ++q) a.out1[6 * ov + q] = Rq[q];
                if (a.out2) a.out2[ov] = MM;
                if (a.out3) a.out3[ov] = dA;
                if (a.out4) a.out4[ov] = dC;
                continue;
            }
            const double4 xv4 = ld4v(xp + v);
            double xi[3] = {xv4.x, xv4.y, xv4.z};
            // integrin force (UL:1241-1269)
            const double4 f4 = ld4v(c.fau + v);
            double fs[3], bell;
            spring_force(p, f4.x, f4.y, f4.z, fs, &bell);
            const double rho = c.rho_w ? c.rho_w[v] : p.rho_i_max;
            const double cCv = c.cC[v];
            const bool subs = c.material == 2;
            double Ffa[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) Ffa[r] = subs ? 0.0 : -cCv * fs[r] * Asum * rho;
            if (MODE == PP_STEP && !subs && c.has_sub && c.sub.scell) {
                // reaction of this vertex's bonds on a deformable substrate (calculateForce_FA_subs
                // UL:1305-1475): at the anchor x - fa_u, onto every containing triangle of the
                // substrate's predicted positions, by barycentric weight; fixed-point sums (2^-40) so
                // the total does not depend on the order of the atomic adds
                const CellDev& sc = *c.sub.scell;
                const double4* __restrict__ xs_s = sc.pos[sc.ctl[0] ^ 1];
                const double Px = xs(xi[0], f4.x), Py = xs(xi[1], f4.y), Pz = xs(xi[2], f4.z);
                const SubDev& g = c.sub;
                const int gx = (int)floor((Px - g.ox) * g.inv_h), gy = (int)floor((Py - g.oy) * g.inv_h);
                if (gx >= 0 && gx < g.gx && gy >= 0 && gy < g.gy) {
                    const int gc = gy * g.gx + gx;
                    for (int k = g.cell_ptr[gc]; k < g.cell_ptr[gc + 1]; ++k) {
                        const int4 t = g.tri[g.cell_tri[k]];
                        double w[3];
                        if (!tri_contains(ld4v(xs_s + t.x), ld4v(xs_s + t.y), ld4v(xs_s + t.z), Px, Py, Pz, w)) continue;
                        const int id[3] = {t.x, t.y, t.z};
#pragma unroll
                        for (int q = 0; q < 3; ++q)
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
                                const double val = cCv * fs[r] * w[q] * Asum * rho;
                                if (!(fabs(val) < 4.0e6)) atomicOr(c.status, 32u);
                                atomicAdd(g.fext + 4 * (size_t)id[q] + r,
                                          (unsigned long long)__double2ll_rn(val * 1099511627776.0));
                            }
                    }
                }
            }
            double Fap[3] = {0, 0, 0}, Fb[3] = {0, 0, 0}, Far[3] = {0, 0, 0};
            const int rank = subs ? -1 : c.bnd_rank[v];
            if (rank >= 0) {
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
                    // bending (UL:1600-1657); orientation decided with unfused arithmetic
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
            if (MODE == PP_FORCES) {
                for (int r = 0; r < 3; ++r) {
                    if (a.out0) a.out0[3 * ov + r] = Ffa[r];
                    if (a.out1) a.out1[3 * ov + r] = Fap[r];
                    if (a.out2) a.out2[3 * ov + r] = Fb[r];
                    if (a.out3) a.out3[3 * ov + r] = Far[r];
                }
                continue;
            }
            // explicit update (UL:592-628)
            const double4 V4 = ld4v(c.vel + v), A4 = ld4v(c.acc + v);
            double vh[3];
            if (a.vh_from_buf) {
                double4 h = ld4v(c.vhl + v);
                vh[0] = h.x; vh[1] = h.y; vh[2] = h.z;
            } else {
                double xn_unused[3];
                predict_vertex_c(c, v, X[v], V4, A4, a.dt, a.hdt, vh, xn_unused);
            }
            const double Vo[3] = {V4.x, V4.y, V4.z};
            double An[3], Vn[3];
            const double md = p.damp * MM * p.rho, imr = 1.0 / (MM * p.rho), iMM = 1.0 / MM;
            if (subs) {
                // substrate update (updateForces_Explicit, substrate overload UL:429-504):
                // f = F_FA_subs - Res, no drag; the reactions are consumed and cleared
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    unsigned long long* q = c.fext_in + 4 * (size_t)v + r;
                    const double fr = (double)(long long)*q * (1.0 / 1099511627776.0);
                    *q = 0ull;
                    An[r] = ((fr - R[r]) - md * Vo[r]) * imr;
                }
            } else {
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    double f = -p.drag * vh[r] + Fb[r] + Fap[r] + Ffa[r] + Far[r] - R[r];
                    An[r] = (f - md * Vo[r]) * imr;
                }
            }
            const bool half = a.dt_real > a.dt / 2.0;
#pragma unroll
            for (int r = 0; r < 3; ++r) Vn[r] = half ? vh[r] + (a.dt_real - a.dt / 2.0) * An[r] : Vo[r] + a.dt_real * An[r];
            const double2* eo = reinterpret_cast<const double2*>(eao + 6 * (size_t)v);
            double2* en = reinterpret_cast<double2*>(c.ea[par ^ 1] + 6 * (size_t)v);
            double2 e0 = eo[0], e1 = eo[1], e2 = eo[2];
            double2 n0 = make_double2(e0.x + Rq[0] * iMM, e0.y + Rq[1] * iMM);
            double2 n1 = make_double2(e1.x + Rq[2] * iMM, e1.y + Rq[3] * iMM);
            double2 n2 = make_double2(e2.x + Rq[4] * iMM, e2.y + Rq[5] * iMM);
            en[0] = n0; en[1] = n1; en[2] = n2;
            st4(c.acc + v, An[0], An[1], An[2]);
            st4(c.vel + v, Vn[0], Vn[1], Vn[2]);
            double chk = An[0] + An[1] + An[2] + Vn[0] + Vn[1] + Vn[2] + n0.x + n0.y + n1.x + n1.y + n2.x + n2.y + xi[0] + xi[1];
            if (!isfinite(chk)) atomicOr(c.status, 1u);
        }
        __syncthreads();
        if (MODE == PP_STEP && threadIdx.x == 0) {
            // the last CTA of this cell to finish the step advances its control words
            __threadfence();
            unsigned int done = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 1), 1u);
            if ((int)done == c.np - 1) {
                c.ctl[1] = 0;
                c.ctl[0] = par ^ 1;
                c.clk[0] = c.clk[0] + a.dt_real;
                c.ap[0] = ap_call + 1ull;
                count_step(c);
            }
        }
    }
}

// drop-in predict of one cell: V_hlf to vhl, x_pred to pos[par^1] and to the host-layout staging buffer
__global__ void k_predict(const CellDev* __restrict__ cells, int cell, double dt, double hdt, double* xout,
                          double* vhout) {
    const CellDev& c = cells[cell];
    const int par = c.ctl[0];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < c.nv; v += gridDim.x * blockDim.x) {
        double vh[3], xn[3];
        predict_vertex_c(c, v, ld4(c.pos[par] + v), ld4(c.vel + v), ld4(c.acc + v), dt, hdt, vh, xn);
        st4(c.vhl + v, vh[0], vh[1], vh[2]);
        st4(c.pos[par ^ 1] + v, xn[0], xn[1], xn[2]);
        if (xout) { xout[3 * (size_t)v] = xn[0]; xout[3 * (size_t)v + 1] = xn[1]; xout[3 * (size_t)v + 2] = xn[2]; }
        if (vhout) { vhout[3 * (size_t)v] = vh[0]; vhout[3 * (size_t)v + 1] = vh[1]; vhout[3 * (size_t)v + 2] = vh[2]; }
    }
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------

void launch_vertex_phase(const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
                         int threads, cudaStream_t st, const double* stage_in, double* stage_out) {
    if (nwork <= 0) return;
    k_vertex_phase<<<grid, threads, 0, st>>>(cells, work, nwork, dt, dt / 2.0, flags, stage_in, stage_out);
}

// mixed-precision patch phase (wcfe_mixed.cu)
size_t mixed_smem_bytes(int emax);
cudaError_t configure_mixed(size_t max_smem);
int mixed_occupancy(int threads, size_t smem);
void launch_patch_mixed(const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt, double dt_real,
                        double ap_thresh, double t_override, int vh_from_buf, int threads, int grid, cudaStream_t st);

// The step of a WCFE_PREC_MIXED engine runs the mixed kernel; the diagnostic
// modes (reference-function mirrors) always run in FP64.
size_t patch_smem_bytes(int prec, int mode, int emax) {
    if (prec == WCFE_PREC_MIXED && mode == PP_STEP) return mixed_smem_bytes(emax);
    return sizeof(double) * (size_t)emax * (kSlot64 + (mode == PP_RESIDUAL ? 6 : 0));
}

static const void* patch_kernel(int mode) {
    if (mode == PP_STEP) return (const void*)k_patch_phase_fp64<PP_STEP>;
    if (mode == PP_RESIDUAL) return (const void*)k_patch_phase_fp64<PP_RESIDUAL>;
    return (const void*)k_patch_phase_fp64<PP_FORCES>;
}

int occupancy_cached(const void* kernel, int threads, size_t smem) {
    struct Entry {
        int dev;
        const void* kernel;
        int threads;
        size_t smem;
        int blocks;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        for (const Entry& x : cache)
            if (x.dev == dev && x.kernel == kernel && x.threads == threads && x.smem == smem) return x.blocks;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    n = n > 0 ? n : 1;
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back({dev, kernel, threads, smem, n});
    return n;
}

int patch_occupancy(int prec, int threads, size_t smem) {
    if (prec == WCFE_PREC_MIXED) return mixed_occupancy(threads, smem);
    return occupancy_cached(patch_kernel(PP_STEP), threads, smem);
}

bool mixed_available() { return true; }

int vertex_occupancy(int threads) { return occupancy_cached((const void*)k_vertex_phase, threads, 0); }

void launch_patch(int prec, int mode, const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt,
                  double dt_real, double ap_thresh, double t_override, int vh_from_buf, const double* centroid_dev,
                  double* o0, double* o1, double* o2, double* o3, double* o4, int threads, int grid, cudaStream_t st,
                  int packed) {
    if (nwork <= 0) return;
    if (prec == WCFE_PREC_MIXED && mode == PP_STEP) {
        launch_patch_mixed(cells, work, nwork, emax, dt, dt_real, ap_thresh, t_override, vh_from_buf, threads, grid, st);
        return;
    }
    PatchArgs a;
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
    a.centroid_override = centroid_dev;
    a.out0 = o0; a.out1 = o1; a.out2 = o2; a.out3 = o3; a.out4 = o4;
    a.packed = packed;
    size_t smem = patch_smem_bytes(WCFE_PREC_FP64, mode, emax);
    if (mode == PP_STEP) k_patch_phase_fp64<PP_STEP><<<grid, threads, smem, st>>>(a);
    else if (mode == PP_RESIDUAL) k_patch_phase_fp64<PP_RESIDUAL><<<grid, threads, smem, st>>>(a);
    else k_patch_phase_fp64<PP_FORCES><<<grid, threads, smem, st>>>(a);
}

void launch_predict(const CellDev* cells, int cell, double dt, double* xout, double* vhout, int nv, cudaStream_t st) {
    int grid = (nv + 255) / 256;
    if (grid < 1) grid = 1;
    k_predict<<<grid, 256, 0, st>>>(cells, cell, dt, dt / 2.0, xout, vhout);
}

// Opt every patch kernel into the largest dynamic shared memory the device
// allows next to its static shared memory.
static cudaError_t optin(const void* fn, size_t max_smem) {
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, fn);
    if (e != cudaSuccess) return e;
    size_t dyn = max_smem > at.sharedSizeBytes ? max_smem - at.sharedSizeBytes : 0;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

cudaError_t configure_kernels(size_t max_smem) {
    for (int mode = PP_STEP; mode <= PP_FORCES; ++mode) {
        cudaError_t e = optin(patch_kernel(mode), max_smem);
        if (e != cudaSuccess) return e;
    }
    return configure_mixed(max_smem);
}

}  // namespace wcfe
