/*
 * wcfe_oracle.c — CPU restatement (plain C, FP64) of wholeCellFE's per-step
 * mechanics, the oracle for the GPU path.
 *
 * TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and the CPU
 * baseline / reference arm of bench.py load this library as the checker.
 * The product library never links, loads or calls it.
 *
 * Each function restates one reference function of
 * dredremontes/wholeCellFE, variant wholeCellFE_kMD unless stated, file
 * cellBP/UL_growth_explicit.cpp ("UL" below) and cellBP/main.cpp.  Its
 * arithmetic follows the reference's order of operations, so that it agrees
 * with the reference compiled from source (oracle/_ref, built by
 * oracle/build_ref.sh) to rounding.  The agreement is checked by
 * tests/test_oracle_ref.py here and pinned by the golden fixtures in
 * tests/golden/ that the reference itself produced.
 *
 * Where the reference reads an uninitialised value, this restatement defines
 * it:
 *  - subs_u when the anchor lies in no substrate triangle (UL:2053) is 0;
 *  - force_s when D is NaN (UL:1258-1264) is 0.
 * Its only random draw, libc rand() in calculateForce_AP (UL:1546), is
 * replaced by the counter-based stream defined in include/wcfe.h.
 *
 * Layout: host arrays in the reference's memory order (double[n][3] for
 * Vec3d vectors, double[n][6] for the Voigt strains).  Compile with
 * -ffp-contract=off so x86 and Arm give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/wcfe.h"

#define WO_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* mesh description                                                    */
/* ------------------------------------------------------------------ */
typedef struct wo_mesh {
    int32_t nv, nt;
    const int32_t* tri;     /* [nt][3] */
    const int32_t* vt_ptr;  /* [nv+1] vertex -> triangle map, mesh order */
    const int32_t* vt_idx;
    const uint8_t* bnd;     /* [nv] NonDestructiveTriMesh::m_is_boundary_vertex */
    const double* mu_e;     /* [nt] optional per-element shear modulus of a cell (NULL: p->mu); an
                               extension without reference counterpart (the reference has one mu per
                               material, UL:721-728) */
} wo_mesh;

/* ------------------------------------------------------------------ */
/* small 3-vector / 3x3 helpers (row-major m[r*3+c])                   */
/* ------------------------------------------------------------------ */
static void v_sub(const double* a, const double* b, double* o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
static void v_cross(const double* a, const double* b, double* o) {
    /* Eigen MatrixBase::cross component order */
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double v_norm(const double* a) { return sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]); }
static double v_dot(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* determinant by cofactor expansion along row 0 */
static double m_det(const double* m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}
/* inverse by the adjugate: cofactors of column 0 give det, then every entry is cofactor * (1/det) */
static void m_inv(const double* m, double* o) {
#define M(r, c) m[(r) * 3 + (c)]
#define COF(i, j) (M(((i) + 1) % 3, ((j) + 1) % 3) * M(((i) + 2) % 3, ((j) + 2) % 3) - M(((i) + 1) % 3, ((j) + 2) % 3) * M(((i) + 2) % 3, ((j) + 1) % 3))
    double c00 = COF(0, 0), c10 = COF(1, 0), c20 = COF(2, 0);
    double det = (c00 * M(0, 0) + c10 * M(1, 0)) + c20 * M(2, 0);
    double id = 1.0 / det;
    o[0] = c00 * id; o[1] = c10 * id; o[2] = c20 * id;
    o[3] = COF(0, 1) * id; o[4] = COF(1, 1) * id; o[5] = COF(2, 1) * id;
    o[6] = COF(0, 2) * id; o[7] = COF(1, 2) * id; o[8] = COF(2, 2) * id;
#undef COF
#undef M
}
/* o = a * b */
static void m_mul(const double* a, const double* b, double* o) {
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = (a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j]) + a[i * 3 + 2] * b[2 * 3 + j];
    memcpy(o, t, sizeof t);
}
/* o = a^T * b */
static void m_tmul(const double* a, const double* b, double* o) {
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = (a[0 * 3 + i] * b[0 * 3 + j] + a[1 * 3 + i] * b[1 * 3 + j]) + a[2 * 3 + i] * b[2 * 3 + j];
    memcpy(o, t, sizeof t);
}
/* o = a * b^T */
static void m_mult(const double* a, const double* b, double* o) {
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = (a[i * 3 + 0] * b[j * 3 + 0] + a[i * 3 + 1] * b[j * 3 + 1]) + a[i * 3 + 2] * b[j * 3 + 2];
    memcpy(o, t, sizeof t);
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the AP draw   */
/* ------------------------------------------------------------------ */
WO_API void wo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
WO_API uint32_t wo_ap_draw(uint32_t seed, uint32_t stream, uint64_t call, uint32_t k) {
    uint32_t ctr[4] = {k, (uint32_t)call, (uint32_t)(call >> 32), 0u};
    uint32_t key[2] = {seed, stream};
    uint32_t out[4];
    wo_philox4x32_10(ctr, key, out);
    return out[0] >> 1;
}

/* ------------------------------------------------------------------ */
/* reference constants                                                 */
/* ------------------------------------------------------------------ */
WO_API void wo_params_default(wcfe_params* p, int32_t variant) {
    memset(p, 0, sizeof *p);
    p->mu = 1000.0; p->thick = 1.0; p->thetag_dot = 0.0; p->kappa = 0.5;
    p->tact_rate = 200.0; p->tact_t1 = 2.0; p->tact_max = 400.0;
    p->D_A = 1.0; p->D_C = 1e-10;
    if (variant == WCFE_VARIANT_KMD) { p->force_law = WCFE_LAW_MD_TABLE; p->k_lin = 31000.0; p->linear_norm2d = 0; }
    else if (variant == WCFE_VARIANT_K1) { p->force_law = WCFE_LAW_LINEAR; p->k_lin = 1000.0; p->linear_norm2d = 1; }
    else { p->force_law = WCFE_LAW_LINEAR; p->k_lin = 31000.0; p->linear_norm2d = 1; }
    p->rest_len = 0.0; p->poly_k0 = 31000.0; p->poly_x0 = 0.005;
    p->rho_i_max = 100.0;
    p->k_on = 1.0; p->ka = 0.004; p->kb = 10.0; p->Fa = 15.0; p->Fb = 15.0;
    p->k_bend = 20.0; p->k_area = 1.0; p->area0 = 10 * 10 * 3.1416;
    p->ap_rate = 10.0; p->ap_force = 5.0; p->ap_density = 100.0; p->ap_enable = 1;
    p->seed = 1u; p->stream = 0u;
    p->drag = 0.001; p->damp = 0.001; p->rho = 1.0;
}

/* MD force-extension fit, UL:1203-1214 (extension um, force pN, stiffness pN/um) */
static const double MD_PX[6] = {0., 2.51250583e-03, 4.40265201e-03, 5.91408228e-03, 11.76817302e-03, 17.001e-03};
static const double MD_PY[6] = {-7.15514497, 71.80501308, 356.62420075, 356.96656556, 126.21811585, 528.40481124};
static const double MD_K[6] = {31426.8556, 99485.86235, 67080.67086, -7908.39043, 21978.66923, 76858.39733};

/* active stress ramp, UL:743-757 */
static double t_act_of(const wcfe_params* p, double time) {
    return time < p->tact_t1 ? time * p->tact_rate : p->tact_max;
}

/*
 * Integrin spring force vector for bond vector u (UL:1245-1264 for the MD
 * table; k1 UL:1259-1261 for the linear law).  Also returns the Bell force
 * magnitude used by updateFA (UL:2112-2137; k1 UL:2077).
 */
static void spring_force(const wcfe_params* p, const double* u, double* fs, double* bell_force) {
    double D = sqrt((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
    if (p->force_law == WCFE_LAW_LINEAR && p->rest_len == 0.0) {
        /* k1 / k31: F = k u (UL k1:1259-1261) and force_FA = k |u_xy| (k1:2077) */
        fs[0] = p->k_lin * u[0]; fs[1] = p->k_lin * u[1]; fs[2] = p->k_lin * u[2];
        if (p->linear_norm2d) *bell_force = p->k_lin * sqrt(u[0] * u[0] + u[1] * u[1]);
        else *bell_force = p->k_lin * D;
        return;
    }
    double uD[3] = {0, 0, 0};
    if (D != 0) { uD[0] = u[0] / D; uD[1] = u[1] / D; uD[2] = u[2] / D; }
    double mag = 0.0;
    if (p->force_law == WCFE_LAW_MD_TABLE) {
        for (int j = 0; j < 5; ++j) {
            if (D < MD_PX[j + 1] && D >= MD_PX[j]) mag = MD_PY[j] + MD_K[j] * (D - MD_PX[j]);
            else if (D >= MD_PX[5]) mag = MD_PY[5] + MD_K[5] * (D - MD_PX[5]);
        }
    } else if (p->force_law == WCFE_LAW_LINEAR) {
        /* a bond with a rest length is slack below it (tension only) */
        mag = D > p->rest_len ? p->k_lin * (D - p->rest_len) : 0.0;
    } else {
        double e = D - p->rest_len;
        mag = e > 0.0 ? p->poly_k0 * (e + e * e * e / (3.0 * p->poly_x0 * p->poly_x0)) : 0.0;
    }
    fs[0] = mag * uD[0]; fs[1] = mag * uD[1]; fs[2] = mag * uD[2];
    if (p->force_law == WCFE_LAW_LINEAR && p->linear_norm2d) {
        double D2 = sqrt(u[0] * u[0] + u[1] * u[1]);
        *bell_force = D2 > p->rest_len ? p->k_lin * (D2 - p->rest_len) : 0.0;
    } else {
        *bell_force = sqrt((fs[0] * fs[0] + fs[1] * fs[1]) + fs[2] * fs[2]);
    }
}

/* ------------------------------------------------------------------ */
/* A1  driverVelocities_Explicit UL:103-124 + new_positions main:227-231 */
/* ------------------------------------------------------------------ */
WO_API void wo_predict(int32_t nv, const double* x, const double* V, const double* A, double dt, double* Vh, double* xpred) {
    for (int i = 0; i < nv; ++i) {
        for (int c = 0; c < 3; ++c) Vh[i * 3 + c] = V[i * 3 + c] + (dt / 2.0) * A[i * 3 + c];
        Vh[i * 3 + 2] = 0.0;
        for (int c = 0; c < 3; ++c) xpred[i * 3 + c] = x[i * 3 + c] + dt * Vh[i * 3 + c];
    }
}

/* ------------------------------------------------------------------ */
/* A2  calculateAreaTot UL:1662-1688                                   */
/* ------------------------------------------------------------------ */
WO_API void wo_area_tot(const wo_mesh* m, const double* x, double out4[4]) {
    double area = 0, cen[3] = {0, 0, 0};
    for (int e = 0; e < m->nt; ++e) {
        const double* p1 = x + 3 * m->tri[3 * e + 0];
        const double* p2 = x + 3 * m->tri[3 * e + 1];
        const double* p3 = x + 3 * m->tri[3 * e + 2];
        double e1[3], e2[3], cr[3];
        v_sub(p2, p1, e1); v_sub(p3, p1, e2); v_cross(e1, e2, cr);
        double av[3] = {0.5 * cr[0], 0.5 * cr[1], 0.5 * cr[2]};
        double ce[3];
        for (int c = 0; c < 3; ++c) ce[c] = 1. / 3. * ((p1[c] + p2[c]) + p3[c]);
        double a = v_norm(av);
        for (int c = 0; c < 3; ++c) cen[c] += ce[c] * a;
        area += a;
    }
    out4[0] = area;
    for (int c = 0; c < 3; ++c) out4[1 + c] = cen[c] / area;
}

/* ------------------------------------------------------------------ */
/* A3  evalElementRe UL:710-928 (mat 1) and UL:989-1176 (mat 2)        */
/* ------------------------------------------------------------------ */
typedef struct wo_elem_out {
    double Re[9], Re_ea[18], MMe[3], ReA[3], ReC[3];
} wo_elem_out;

static void wo_element(const double* X1, const double* X2, const double* X3,
                       const double* x1, const double* x2, const double* x3,
                       const double* ea1, const double* ea2, const double* ea3,
                       const double* cA3, const double* cC3, double dt_real, int mat, double mu,
                       const wcfe_params* p, double t_act, const double* centroid, wo_elem_out* o) {
    const double thick = p->thick;
    double G1[3], G2[3], GxG[3], N[3];
    v_sub(X2, X1, G1); v_sub(X3, X1, G2); v_cross(G1, G2, GxG);
    double nG = v_norm(GxG);
    for (int c = 0; c < 3; ++c) N[c] = GxG[c] / nG;

    const double third = 1.0 / 3.0;
    double ev[6];
    for (int q = 0; q < 6; ++q) ev[q] = (third * ea1[q] + third * ea2[q]) + third * ea3[q];
    double Et[9] = {ev[0], ev[3], ev[4], ev[3], ev[1], ev[5], ev[4], ev[5], ev[2]};
    double aux[9], bet[9], NN[9], bets[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) aux[r * 3 + c] = (r == c ? 1.0 : 0.0) - 2.0 * Et[r * 3 + c];
    m_inv(aux, bet);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) { NN[r * 3 + c] = N[r] * N[c]; bets[r * 3 + c] = bet[r * 3 + c] - NN[r * 3 + c]; }

    double g1[3], g2[3], gxg[3], n[3];
    v_sub(x2, x1, g1); v_sub(x3, x1, g2); v_cross(g1, g2, gxg);
    double ng = v_norm(gxg);
    for (int c = 0; c < 3; ++c) n[c] = gxg[c] / ng;

    double G[9] = {G1[0], G2[0], N[0], G1[1], G2[1], N[1], G1[2], G2[2], N[2]};
    double g[9] = {g1[0], g2[0], n[0], g1[1], g2[1], n[1], g1[2], g2[2], n[2]};
    double Gi[9];
    m_inv(G, Gi);
    const double* G1i = Gi;      /* row 0 */
    const double* G2i = Gi + 3;  /* row 1 */
    double F[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) F[r * 3 + c] = (g1[r] * G1i[c] + g2[r] * G2i[c]) + n[r] * N[c];
    double C[9], Ci[9], Cis[9];
    m_tmul(F, F, C);
    m_inv(C, Ci);
    for (int k = 0; k < 9; ++k) Cis[k] = Ci[k] - NN[k];

    /* diffusion gradients (UL:835-843) */
    double gi[9];
    m_inv(g, gi);
    const double* g1i = gi;
    const double* g2i = gi + 3;
    double gradA[3], gradC[3];
    for (int c = 0; c < 3; ++c) {
        gradA[c] = (cA3[0] * g1i[c] + cA3[1] * g2i[c]) + cA3[2] * (-g1i[c] - g2i[c]);
        gradC[c] = (cC3[0] * g1i[c] + cC3[1] * g2i[c]) + cC3[2] * (-g1i[c] - g2i[c]);
    }
    double cAm = (1. / 3.) * ((cA3[0] + cA3[1]) + cA3[2]);
    double cCm = (1. / 3.) * ((cC3[0] + cC3[1]) + cC3[2]);

    double theta_e_t = sqrt(m_det(bet));
    double theta_g = 1.0 + p->thetag_dot * dt_real;
    double theta = m_det(F);
    double theta_e = theta * theta_e_t / theta_g;
    double lamN = 1.0 / theta_e;
    double pr = -mu * (lamN * lamN);

    double S[9];
    for (int k = 0; k < 9; ++k) S[k] = (mu / theta_g) * bets[k] + theta_g * pr * Cis[k];
    if (mat == 1) {
        double ce[3], a0[3];
        for (int c = 0; c < 3; ++c) ce[c] = 1. / 3. * ((x1[c] + x2[c]) + x3[c]);
        v_sub(ce, centroid, a0);
        double na = v_norm(a0);
        for (int c = 0; c < 3; ++c) a0[c] = a0[c] / na;
        double kap = p->kappa;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double sact = t_act * (kap * (r == c ? 1.0 : 0.0) + (1 - 2 * kap) * a0[r] * a0[c]);
                S[r * 3 + c] = sact + S[r * 3 + c];
            }
    } else {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S[r * 3 + c] = t_act * (r == c ? 1.0 : 0.0) + S[r * 3 + c];
    }

    /* strain update (UL:884-887) */
    double Fb[9], be[9], bei[9], eas[9];
    m_mul(F, bet, Fb);
    m_mult(Fb, F, be);
    double sg = 1.0 / (theta_g * theta_g);
    for (int k = 0; k < 9; ++k) be[k] = sg * be[k];
    m_inv(be, bei);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) eas[r * 3 + c] = 0.5 * ((r == c ? 1.0 : 0.0) - bei[r * 3 + c]);
    double easv[6] = {eas[0], eas[4], eas[8], eas[1], eas[2], eas[5]};
    double Sv[6] = {S[0], S[4], S[8], S[1], S[2], S[5]};

    const double* eanode[3] = {ea1, ea2, ea3};
    for (int i = 0; i < 3; ++i) {
        for (int pdir = 0; pdir < 3; ++pdir) {
            /* varg1 = -e_p [i==0] + e_p [i==1]; varg2 = -e_p [i==0] + e_p [i==2] (UL:893-897) */
            double s1 = (i == 0 ? -1.0 : 0.0) + (i == 1 ? 1.0 : 0.0);
            double s2 = (i == 0 ? -1.0 : 0.0) + (i == 2 ? 1.0 : 0.0);
            double vF[9];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) vF[r * 3 + c] = (r == pdir) ? (s1 * G1i[c] + s2 * G2i[c]) : (0.0 * G1i[c] + 0.0 * G2i[c]);
            double t1[9], t2[9], vE[9];
            m_tmul(vF, F, t1);
            m_tmul(F, vF, t2);
            for (int k = 0; k < 9; ++k) vE[k] = 0.5 * (t1[k] + t2[k]);
            double vEv[6] = {vE[0], vE[4], vE[8], 2 * vE[1], 2 * vE[2], 2 * vE[5]};
            double dot = 0;
            for (int q = 0; q < 6; ++q) dot += Sv[q] * vEv[q];
            o->Re[i * 3 + pdir] = dot * nG / 2.0 * thick;
        }
        for (int q = 0; q < 6; ++q) o->Re_ea[i * 6 + q] = (1. / 3.) * (easv[q] - eanode[i][q]) * nG / 2.0 * thick;
        o->MMe[i] = (1. / 3.) * nG / 2.0 * thick;
        double gN[3];
        for (int c = 0; c < 3; ++c) {
            double v0 = (i == 0), v1 = (i == 1), v2 = (i == 2);
            gN[c] = (v0 * g1i[c] + v1 * g2i[c]) + v2 * (-g1i[c] - g2i[c]);
        }
        o->ReA[i] = (cAm * (1. / 3.) - dt_real * p->D_A * v_dot(gradA, gN)) * nG / 2.0 * thick;
        o->ReC[i] = (cCm * (1. / 3.) - dt_real * p->D_C * v_dot(gradC, gN)) * nG / 2.0 * thick;
    }
}

/* calculateRes, cell overload UL:632-707 (mat 1) and substrate overload UL:931-986 (mat 2) */
WO_API void wo_calc_res(const wo_mesh* m, const double* X, const double* x, const double* ea,
                        const double* cA, const double* cC, double dt_real, int mat,
                        const wcfe_params* p, const double* centroid, double time,
                        double* Res, double* Res_ea, double* MM, double* ResA, double* ResC) {
    int nv = m->nv;
    memset(Res, 0, sizeof(double) * 3 * nv);
    memset(Res_ea, 0, sizeof(double) * 6 * nv);
    memset(MM, 0, sizeof(double) * nv);
    if (ResA) memset(ResA, 0, sizeof(double) * nv);
    if (ResC) memset(ResC, 0, sizeof(double) * nv);
    double mu = p->mu;
    double t_act = (mat == 1) ? t_act_of(p, time) : 0.0;
    static const double zero3[3] = {0, 0, 0};
    for (int e = 0; e < m->nt; ++e) {
        int a = m->tri[3 * e], b = m->tri[3 * e + 1], c = m->tri[3 * e + 2];
        double cAe[3] = {0, 0, 0}, cCe[3] = {0, 0, 0};
        if (cA) { cAe[0] = cA[a]; cAe[1] = cA[b]; cAe[2] = cA[c]; }
        if (cC) { cCe[0] = cC[a]; cCe[1] = cC[b]; cCe[2] = cC[c]; }
        wo_elem_out o;
        const double mu_el = (mat == 1 && m->mu_e) ? m->mu_e[e] : mu;
        wo_element(X + 3 * a, X + 3 * b, X + 3 * c, x + 3 * a, x + 3 * b, x + 3 * c, ea + 6 * a, ea + 6 * b, ea + 6 * c,
                   cAe, cCe, dt_real, mat, mu_el, p, t_act, centroid ? centroid : zero3, &o);
        int idx[3] = {a, b, c};
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) Res[idx[i] * 3 + k] += o.Re[i * 3 + k];
            for (int k = 0; k < 6; ++k) Res_ea[idx[i] * 6 + k] += o.Re_ea[i * 6 + k];
            MM[idx[i]] += o.MMe[i];
            if (ResA) ResA[idx[i]] += o.ReA[i];
            if (ResC) ResC[idx[i]] += o.ReC[i];
        }
    }
}

/* ------------------------------------------------------------------ */
/* A4  calculateForce_FA UL:1198-1303 (linear: k1 UL:1196-1261)         */
/* ------------------------------------------------------------------ */
static double onering_area3(const wo_mesh* m, const double* x, int v) {
    double Asum = 0.0;
    for (int k = m->vt_ptr[v]; k < m->vt_ptr[v + 1]; ++k) {
        int t = m->vt_idx[k];
        const double* p0 = x + 3 * m->tri[3 * t];
        const double* p1 = x + 3 * m->tri[3 * t + 1];
        const double* p2 = x + 3 * m->tri[3 * t + 2];
        double E1[3], E2[3], nr[3];
        v_sub(p1, p0, E1); v_sub(p2, p0, E2); v_cross(E1, E2, nr);
        double a = 0.5 * v_norm(nr);
        Asum += a / 3;
    }
    return Asum;
}

WO_API void wo_force_fa(const wo_mesh* m, const double* x, const double* cC, const double* fau,
                        const wcfe_params* p, const double* rho_w, double* F) {
    for (int v = 0; v < m->nv; ++v) {
        double Asum = onering_area3(m, x, v);
        double fs[3], bf;
        spring_force(p, fau + 3 * v, fs, &bf);
        double rho = rho_w ? rho_w[v] : p->rho_i_max;
        for (int c = 0; c < 3; ++c) F[3 * v + c] = -cC[v] * fs[c] * Asum * rho;
    }
}

/* ------------------------------------------------------------------ */
/* boundary-curve neighbours j1 (start) / j2 (end), UL:1489-1531        */
/* ------------------------------------------------------------------ */
/* Returns j1, j2 vertex ids (-1 when not found) and the neighbour count ct. */
static void bnd_neighbours(const wo_mesh* m, const double* x, int v, int* j1, int* j2, int* ct) {
    *j1 = -1; *j2 = -1; *ct = 0;
    const double* pv = x + 3 * v;
    for (int k = m->vt_ptr[v]; k < m->vt_ptr[v + 1]; ++k) {
        const int32_t* t = m->tri + 3 * m->vt_idx[k];
        for (int a = 0; a < 3; ++a) {
            int nj = t[a];
            if (m->bnd[nj] && nj != v) {
                *ct += 1;
                int nint = -1;
                for (int b = 0; b < 3; ++b)
                    if (t[b] != nj && t[b] != v) { nint = t[b]; break; }
                const double* pb = x + 3 * nj;
                const double* pi = x + 3 * nint;
                double d1[3], d2[3], nc[3];
                v_sub(pv, pb, d1); v_sub(pi, pv, d2); v_cross(d1, d2, nc);
                if (nc[2] > 0) *j1 = nj;
                else *j2 = nj;
            }
        }
    }
}

/* outward normal weighting shared by A6-A8 (UL:1535-1543, :1626-1647) */
static void bnd_normal(const double* xi, const double* x1, const double* x2, double* nrm, double* l1o, double* l2o) {
    double d1[3], d2[3];
    v_sub(xi, x1, d1); v_sub(x2, xi, d2);
    /* normal = -e3 x d: (d_y, -d_x, 0) with the reference's cross order */
    double e3[3] = {0, 0, 1}, c1[3], c2[3];
    v_cross(e3, d1, c1); v_cross(e3, d2, c2);
    double n1[3] = {-c1[0], -c1[1], -c1[2]}, n2[3] = {-c2[0], -c2[1], -c2[2]};
    double nn1 = v_norm(n1), nn2 = v_norm(n2);
    for (int c = 0; c < 3; ++c) { n1[c] = n1[c] / nn1; n2[c] = n2[c] / nn2; }
    double l1 = v_norm(d1), l2 = v_norm(d2);
    double L = l1 + l2;
    for (int c = 0; c < 3; ++c) nrm[c] = l1 / L * n1[c] + l2 / L * n2[c];
    *l1o = l1; *l2o = l2;
}

/* A6  calculateForce_AP UL:1477-1568, rand() replaced by the counter-based stream */
WO_API void wo_force_ap(const wo_mesh* m, const double* x, double dt_real, const wcfe_params* p, uint64_t call, double* F) {
    memset(F, 0, sizeof(double) * 3 * m->nv);
    uint32_t k = 0;
    double thr = p->ap_rate * dt_real * exp(-p->ap_rate * dt_real);
    for (int v = 0; v < m->nv; ++v) {
        if (!m->bnd[v]) continue;
        int j1, j2, ct;
        bnd_neighbours(m, x, v, &j1, &j2, &ct);
        uint32_t r = wo_ap_draw(p->seed, p->stream, call, k++);
        if (j1 < 0 || j2 < 0) continue; /* reference reads uninitialised vectors here (UL:1528-1531) */
        double nrm[3], l1, l2;
        bnd_normal(x + 3 * v, x + 3 * j1, x + 3 * j2, nrm, &l1, &l2);
        double L = l1 + l2;
        double Pr = (double)r / ((double)2147483647 + 1.);
        double fsc = 0;
        for (int ii = 0; ii < p->ap_density * L / 2; ii++)
            if (Pr < thr) fsc += p->ap_force;
        for (int c = 0; c < 3; ++c) F[3 * v + c] = fsc * nrm[c];
    }
}

/* A7  calculateBendingForce2D UL:1571-1660 */
WO_API void wo_force_bending(const wo_mesh* m, const double* x, const wcfe_params* p, double* F) {
    memset(F, 0, sizeof(double) * 3 * m->nv);
    for (int v = 0; v < m->nv; ++v) {
        if (!m->bnd[v]) continue;
        int j1, j2, ct;
        bnd_neighbours(m, x, v, &j1, &j2, &ct);
        if (j1 < 0 || j2 < 0) continue;
        const double* xi = x + 3 * v;
        double ed1[3], ed2[3];
        v_sub(xi, x + 3 * j1, ed1); v_sub(x + 3 * j2, xi, ed2);
        double n1 = v_norm(ed1), n2 = v_norm(ed2);
        for (int c = 0; c < 3; ++c) { ed1[c] = ed1[c] / n1; ed2[c] = ed2[c] / n2; }
        double costurn = v_dot(ed1, ed2);
        double e3s[3];
        v_cross(ed1, ed2, e3s);
        double turna = (e3s[2] > 0) ? costurn - 1 : 1 - costurn;
        double nrm[3], l1, l2;
        bnd_normal(xi, x + 3 * j1, x + 3 * j2, nrm, &l1, &l2);
        double L = l1 + l2;
        double kap = turna * 2 / L;
        for (int c = 0; c < 3; ++c) F[3 * v + c] = p->k_bend * kap * nrm[c];
    }
}

/* A8  calculateAreaConstraintForce UL:1691-1784 (its acos curvature is computed but unused there) */
WO_API void wo_force_area(const wo_mesh* m, const double* x, double tot_area, const wcfe_params* p, double* F) {
    memset(F, 0, sizeof(double) * 3 * m->nv);
    for (int v = 0; v < m->nv; ++v) {
        if (!m->bnd[v]) continue;
        int j1, j2, ct;
        bnd_neighbours(m, x, v, &j1, &j2, &ct);
        if (j1 < 0 || j2 < 0) continue;
        double nrm[3], l1, l2;
        bnd_normal(x + 3 * v, x + 3 * j1, x + 3 * j2, nrm, &l1, &l2);
        double L = l1 + l2;
        for (int c = 0; c < 3; ++c) F[3 * v + c] = -p->k_area * (tot_area - p->area0) / 2 * L * nrm[c];
    }
}

/* boundary neighbour table for the topology tests: j1, j2, count per vertex (-1 for interior) */
WO_API void wo_bnd_table(const wo_mesh* m, const double* x, int32_t* j1o, int32_t* j2o, int32_t* cto) {
    for (int v = 0; v < m->nv; ++v) {
        if (!m->bnd[v]) { j1o[v] = j2o[v] = -1; cto[v] = 0; continue; }
        int j1, j2, ct;
        bnd_neighbours(m, x, v, &j1, &j2, &ct);
        j1o[v] = j1; j2o[v] = j2; cto[v] = ct;
    }
}

/* ------------------------------------------------------------------ */
/* A5  updateFA (full) UL:2026-2174; linear k1 UL:2005-2090             */
/* ------------------------------------------------------------------ */
/* point location by the reference's area-sign test, last containing triangle wins (UL:2061-2100) */
WO_API int32_t wo_locate(const wo_mesh* ms, const double* Xs, const double* P, double bary[3]) {
    int32_t found = -1;
    for (int e = 0; e < ms->nt; ++e) {
        const double* p1 = Xs + 3 * ms->tri[3 * e];
        const double* p2 = Xs + 3 * ms->tri[3 * e + 1];
        const double* p3 = Xs + 3 * ms->tri[3 * e + 2];
        double e1[3], e2[3], nr[3], ep[3], a3n[3], a2n[3];
        v_sub(p2, p1, e1); v_sub(p3, p1, e2); v_cross(e1, e2, nr);
        double At = 0.5 * v_norm(nr);
        v_sub(P, p1, ep);
        v_cross(e1, ep, a3n);
        double A3 = -1;
        if (a3n[2] >= 0) A3 = 0.5 * v_norm(a3n);
        double A2 = -1;
        v_cross(ep, e2, a2n);
        if (a2n[2] >= 0) A2 = 0.5 * v_norm(a2n);
        double A1 = At - A2 - A3;
        if (A1 >= 0 && A2 >= 0 && A3 >= 0) {
            found = e;
            bary[0] = A1 / At; bary[1] = A2 / At; bary[2] = A3 / At;
        }
    }
    return found;
}

WO_API void wo_update_fa(int32_t nv, double* cA, double* cC, double* fau, double dt_real,
                         const double* X, const double* x, const wo_mesh* ms, const double* Xs, const double* xs,
                         const wcfe_params* p, int32_t* loc_out) {
    for (int v = 0; v < nv; ++v) {
        double cu[3], su[3] = {0, 0, 0};
        v_sub(x + 3 * v, X + 3 * v, cu);
        int32_t loc = -1;
        if (ms && ms->nt > 0) {
            double P[3], bary[3];
            v_sub(X + 3 * v, fau + 3 * v, P);
            loc = wo_locate(ms, Xs, P, bary);
            if (loc >= 0) {
                const int32_t* t = ms->tri + 3 * loc;
                for (int c = 0; c < 3; ++c) {
                    double d0 = xs[3 * t[0] + c] - Xs[3 * t[0] + c];
                    double d1 = xs[3 * t[1] + c] - Xs[3 * t[1] + c];
                    double d2 = xs[3 * t[2] + c] - Xs[3 * t[2] + c];
                    su[c] = (bary[0] * d0 + bary[1] * d1) + bary[2] * d2;
                }
            }
        }
        if (loc_out) loc_out[v] = loc;
        for (int c = 0; c < 3; ++c) fau[3 * v + c] = fau[3 * v + c] + cu[c] - su[c];
        double fs[3], force;
        spring_force(p, fau + 3 * v, fs, &force);
        double koff = p->ka * exp(force / p->Fa) + p->kb * exp(-force / p->Fb);
        double cold = cC[v];
        cC[v] = cC[v] + dt_real * p->k_on * (1 - cC[v]) - dt_real * koff * cC[v];
        if (cC[v] < 0) cC[v] = 0;
        if (cA[v] < 0) cA[v] = 0;
        double keep = cold - dt_real * koff * cold;
        if (keep > 0 && cC[v] > 0) {
            for (int c = 0; c < 3; ++c) fau[3 * v + c] = fau[3 * v + c] * keep / cC[v];
        } else {
            for (int c = 0; c < 3; ++c) fau[3 * v + c] = 0.0 * fau[3 * v + c];
        }
    }
}

/* ------------------------------------------------------------------ */
/* A9  updateForces_Explicit, cell overload UL:508-630                  */
/* ------------------------------------------------------------------ */
typedef struct wo_force_dump {
    double* Res;  /* [nv][3] optional outputs of the intermediate forces */
    double* F_FA;
    double* F_AP;
    double* F_bend;
    double* F_area;
    double* area4;
} wo_force_dump;

WO_API void wo_update_forces(const wo_mesh* m, const double* X, const double* x, double* V, const double* Vh,
                             double* A, double* ea, const double* cA, const double* cC, const double* fau,
                             double dt, double dt_real, double t_tot, const wcfe_params* p, const double* rho_w,
                             uint64_t ap_call, wo_force_dump* dump) {
    int nv = m->nv;
    double area4[4];
    wo_area_tot(m, x, area4);
    double* Res = (double*)malloc(sizeof(double) * 3 * nv);
    double* Rea = (double*)malloc(sizeof(double) * 6 * nv);
    double* MM = (double*)malloc(sizeof(double) * nv);
    double* FFA = (double*)calloc(3 * (size_t)nv, sizeof(double));
    double* FAP = (double*)calloc(3 * (size_t)nv, sizeof(double));
    double* FB = (double*)calloc(3 * (size_t)nv, sizeof(double));
    double* FAR = (double*)calloc(3 * (size_t)nv, sizeof(double));
    wo_calc_res(m, X, x, ea, cA, cC, dt_real, 1, p, area4 + 1, t_tot, Res, Rea, MM, NULL, NULL);
    wo_force_fa(m, x, cC, fau, p, rho_w, FFA);
    if (p->ap_enable) wo_force_ap(m, x, dt_real, p, ap_call, FAP);
    wo_force_bending(m, x, p, FB);
    wo_force_area(m, x, area4[0], p, FAR);
    for (int v = 0; v < nv; ++v) {
        double Mv = MM[v];
        for (int c = 0; c < 3; ++c) {
            double fvd = -p->drag * Vh[3 * v + c];
            double f = fvd + FB[3 * v + c] + FAP[3 * v + c] + FFA[3 * v + c] + FAR[3 * v + c] - Res[3 * v + c];
            A[3 * v + c] = (f - p->damp * Mv * p->rho * V[3 * v + c]) / (Mv * p->rho);
        }
        for (int q = 0; q < 6; ++q) ea[6 * v + q] += Rea[6 * v + q] / Mv;
    }
    for (int v = 0; v < nv; ++v) {
        for (int c = 0; c < 3; ++c) {
            if (dt_real > dt / 2.0) V[3 * v + c] = Vh[3 * v + c] + (dt_real - dt / 2.0) * A[3 * v + c];
            else V[3 * v + c] = V[3 * v + c] + dt_real * A[3 * v + c];
        }
    }
    if (dump) {
        if (dump->Res) memcpy(dump->Res, Res, sizeof(double) * 3 * nv);
        if (dump->F_FA) memcpy(dump->F_FA, FFA, sizeof(double) * 3 * nv);
        if (dump->F_AP) memcpy(dump->F_AP, FAP, sizeof(double) * 3 * nv);
        if (dump->F_bend) memcpy(dump->F_bend, FB, sizeof(double) * 3 * nv);
        if (dump->F_area) memcpy(dump->F_area, FAR, sizeof(double) * 3 * nv);
        if (dump->area4) memcpy(dump->area4, area4, sizeof area4);
    }
    free(Res); free(Rea); free(MM); free(FFA); free(FAP); free(FB); free(FAR);
}

/* ------------------------------------------------------------------ */
/* A10 substrate: calculateForce_FA_subs UL:1305-1475 and the substrate */
/*     overload of updateForces_Explicit UL:429-504                     */
/* ------------------------------------------------------------------ */
WO_API void wo_force_fa_subs(const wo_mesh* ms, const double* Xs, const double* xs, const double* cC,
                             const double* xcell, const double* fau, const wo_mesh* mc, const wcfe_params* p,
                             const double* rho_w, double* F) {
    /* Xs mirrors the reference's X_t argument: its containment test on X_t is commented out
       (UL:1333-1334, 1339) and the anchors are located with the current positions x_t; the one
       use of X_t, subs_u (UL:1354), does not reach the force */
    (void)Xs;
    memset(F, 0, sizeof(double) * 3 * ms->nv);
    for (int v = 0; v < mc->nv; ++v) {
        double P[3];
        v_sub(xcell + 3 * v, fau + 3 * v, P);
        for (int e = 0; e < ms->nt; ++e) {
            const int32_t* t = ms->tri + 3 * e;
            const double* p1 = xs + 3 * t[0];
            const double* p2 = xs + 3 * t[1];
            const double* p3 = xs + 3 * t[2];
            double e1[3], e2[3], nr[3], ep[3], a3n[3], a2n[3];
            v_sub(p2, p1, e1); v_sub(p3, p1, e2); v_cross(e1, e2, nr);
            double At = 0.5 * v_norm(nr);
            v_sub(P, p1, ep);
            v_cross(e1, ep, a3n);
            double A3 = -1;
            if (a3n[2] >= 0) A3 = 0.5 * v_norm(a3n);
            double A2 = -1;
            v_cross(ep, e2, a2n);
            if (a2n[2] >= 0) A2 = 0.5 * v_norm(a2n);
            double A1 = At - A2 - A3;
            if (A1 >= 0 && A2 >= 0 && A3 >= 0) {
                double Asum = onering_area3(mc, xcell, v);
                double fs[3], bf;
                spring_force(p, fau + 3 * v, fs, &bf);
                double rho = rho_w ? rho_w[v] : p->rho_i_max;
                double w[3] = {A1 / At, A2 / At, A3 / At};
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) F[3 * t[a] + c] += cC[v] * fs[c] * w[a] * Asum * rho;
            }
        }
    }
}

WO_API void wo_update_forces_subs(const wo_mesh* ms, const double* Xs, const double* xs, double* Vs, const double* Vhs,
                                  double* As, double* eas, double dt, double dt_real, double t_tot,
                                  const double* fau, const double* cC, const double* xcell, const wo_mesh* mc,
                                  const wcfe_params* pc, const double* rho_w, double* Res_out, double* FFA_out) {
    int nv = ms->nv;
    wcfe_params ps = *pc;
    ps.mu = 1000000.0; /* substrate stiffness, UL:726 */
    double* Res = (double*)malloc(sizeof(double) * 3 * nv);
    double* Rea = (double*)malloc(sizeof(double) * 6 * nv);
    double* MM = (double*)malloc(sizeof(double) * nv);
    double* FFA = (double*)malloc(sizeof(double) * 3 * nv);
    wo_calc_res(ms, Xs, xs, eas, NULL, NULL, dt_real, 2, &ps, NULL, t_tot, Res, Rea, MM, NULL, NULL);
    wo_force_fa_subs(ms, Xs, xs, cC, xcell, fau, mc, pc, rho_w, FFA);
    for (int v = 0; v < nv; ++v) {
        double Mv = MM[v];
        for (int c = 0; c < 3; ++c) {
            double f = FFA[3 * v + c] - Res[3 * v + c];
            As[3 * v + c] = (f - pc->damp * Mv * pc->rho * Vs[3 * v + c]) / (Mv * pc->rho);
        }
        for (int q = 0; q < 6; ++q) eas[6 * v + q] += Rea[6 * v + q] / Mv;
    }
    for (int v = 0; v < nv; ++v)
        for (int c = 0; c < 3; ++c) {
            if (dt_real > dt / 2.0) Vs[3 * v + c] = Vhs[3 * v + c] + (dt_real - dt / 2.0) * As[3 * v + c];
            else Vs[3 * v + c] = Vs[3 * v + c] + dt_real * As[3 * v + c];
        }
    if (Res_out) memcpy(Res_out, Res, sizeof(double) * 3 * nv);
    if (FFA_out) memcpy(FFA_out, FFA, sizeof(double) * 3 * nv);
    free(Res); free(Rea); free(MM); free(FFA);
}

/* ------------------------------------------------------------------ */
/* one full synthetic step (cellBP/main.cpp:168-408 without El Topo):   */
/* El Topo's integrate takes the full step (actual_dt = dt) and the     */
/* substrate stays where it is (main.cpp:299).                          */
/* ------------------------------------------------------------------ */
typedef struct wo_cell {
    wo_mesh mesh;
    double *x, *V, *A, *ea, *cA, *cC, *fau;
    const double* rho_w;   /* optional per-vertex integrin density (NULL: rho_i_max) */
    wcfe_params p;
    double t;              /* simulation time at the start of the step (sim->m_curr_t) */
    uint64_t ap_call;      /* AP calls made so far */
    const wo_mesh* sub;    /* substrate mesh or NULL (plane) */
    const double* Xs;
} wo_cell;

/*
 * The radial protrusion driver (wcfe_params.protrude_v), an extension: the reference's
 * default driver (driverVelocities_Explicit UL:103-124) prescribes nothing, and its other
 * drivers (driverVelocities_Uniaxial UL:125-168) prescribe the half-step velocity of the
 * driven nodes, after which x = X + dt V_hlf as usual.  Here every boundary vertex is
 * driven radially from c = (protrude_cx, protrude_cy): V_hlf = protrude_v (X - c) / |X - c|
 * in the plane (a vertex at c keeps its default V_hlf).
 */
WO_API void wo_drive_protrusion(const wo_mesh* m, const double* X, const wcfe_params* p, double dt, double* Vh,
                                double* xn) {
    if (p->protrude_v == 0.0) return;
    for (int i = 0; i < m->nv; ++i) {
        if (!m->bnd[i]) continue;
        const double dx = X[3 * i] - p->protrude_cx, dy = X[3 * i + 1] - p->protrude_cy;
        const double r = sqrt(dx * dx + dy * dy);
        if (r == 0.0) continue;
        Vh[3 * i] = p->protrude_v * (dx / r);
        Vh[3 * i + 1] = p->protrude_v * (dy / r);
        Vh[3 * i + 2] = 0.0;
        for (int c = 0; c < 3; ++c) xn[3 * i + c] = X[3 * i + c] + dt * Vh[3 * i + c];
    }
}

WO_API void wo_cell_steps(wo_cell* c, int32_t nsteps, double dt) {
    int nv = c->mesh.nv;
    double* Vh = (double*)malloc(sizeof(double) * 3 * nv);
    double* xn = (double*)malloc(sizeof(double) * 3 * nv);
    for (int s = 0; s < nsteps; ++s) {
        wo_predict(nv, c->x, c->V, c->A, dt, Vh, xn);
        wo_drive_protrusion(&c->mesh, c->x, &c->p, dt, Vh, xn);
        wo_update_fa(nv, c->cA, c->cC, c->fau, dt, c->x, xn, c->sub, c->Xs, c->Xs, &c->p, NULL);
        wo_update_forces(&c->mesh, c->x, xn, c->V, Vh, c->A, c->ea, c->cA, c->cC, c->fau, dt, dt, c->t, &c->p,
                         c->rho_w, c->ap_call, NULL);
        c->ap_call += 1; /* one calculateForce_AP call (one srand) per step */
        memcpy(c->x, xn, sizeof(double) * 3 * nv);
        c->t += dt;
    }
    free(Vh); free(xn);
}

/* Many independent cells on nthreads host threads (the throughput baseline). */
#include <pthread.h>
typedef struct wo_pool_arg {
    wo_cell* cells;
    int32_t ncells, nsteps, stride, first;
    double dt;
} wo_pool_arg;
static void* wo_pool_main(void* a_) {
    wo_pool_arg* a = (wo_pool_arg*)a_;
    for (int i = a->first; i < a->ncells; i += a->stride) wo_cell_steps(&a->cells[i], a->nsteps, a->dt);
    return NULL;
}
WO_API void wo_cells_steps_mt(wo_cell* cells, int32_t ncells, int32_t nsteps, double dt, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    wo_pool_arg* args = (wo_pool_arg*)malloc(sizeof(wo_pool_arg) * nthreads);
    for (int t = 0; t < nthreads; ++t) {
        args[t].cells = cells; args[t].ncells = ncells; args[t].nsteps = nsteps;
        args[t].stride = nthreads; args[t].first = t; args[t].dt = dt;
        pthread_create(&th[t], NULL, wo_pool_main, &args[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th); free(args);
}

WO_API int32_t wo_sizeof_params(void) { return (int32_t)sizeof(wcfe_params); }
WO_API int32_t wo_sizeof_cell(void) { return (int32_t)sizeof(wo_cell); }
