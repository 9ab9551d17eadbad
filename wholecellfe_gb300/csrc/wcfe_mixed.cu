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
// exactly zero, so it stays out of the FP32 element and is added in float-float for
// boundary vertices: (1/2) kappa t_act thick e3 x sum (X_k - X_j).  The strain
// update uses K = F^-1 - I = -H F^-1:
//     ea_s - E = theta_g^2 D + (theta_g^2 - 1)(E - I/2),
//     D = K^T E + E K + K^T E K - (K + K^T + K^T K)/2.
//
// The vertex phase packs each vertex's element inputs into an FP32 record:
// the position as float-float (hi, lo), the step displacement u = x - X and
// the strain.  The element loop therefore does no FP64 arithmetic.  The state
// and every accumulation are extended-precision FP32 formats (wcfe_ff.cuh), not
// binary64, because GB300 retires FP64 at about 1/64 of its FP32 rate: positions
// triple-float (about 72 bits, exact for any binary64 input), velocity, strain,
// c_C and the bond vector float-float (about 48 bits).  The per-step force and
// acceleration are FP32.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "wcfe_common.cuh"
#include "wcfe_cvt.h"
#include "wcfe_ff.cuh"
#include "wcfe_tma.cuh"

namespace wcfe {

// the vertex phase's step arguments (predict, bond kinetics, element records)
struct VertexArgs {
    ff dt, hdt;
    double dtd;
    float dtf;
    int flags;
    const double* stage_in;
    double* stage_out;
};

struct MixedArgs {
    const CellDev* cells;
    const WorkItem* work;
    int nwork, emax;
    double dt_real, ap_thresh, t_override;
    ff hdt, cdt, dtr;        // dt/2, dt_real - dt/2, dt_real as float-float
    int vh_from_buf, half;   // half = dt_real > dt/2
    // the fused form (k_patch_phase_mixed<5, true>): after its owned vertices' update, each
    // patch also runs the next step's vertex phase on them with these arguments
    VertexArgs va;
};

// The mixed engine's state arrays hold float-float values (wcfe_ff.cuh) in the
// slots the FP64 engine uses for doubles, as structures of arrays over the cell's
// n vertices: pos, vel, fau and vhl as hi float4[n] then lo float4[n] (32n B);
// ea as hi float4[n] (xx, yy, zz, xy), lo float4[n], then float4[n] (xz hi,
// yz hi, xz lo, yz lo) (48n B); cA and cC as hi float[n] then lo float[n] (8n B);
// acc holds the FP32 acceleration as float4[n]; the integrin density is float[n].
__device__ __forceinline__ ff4 ldg_ff4(const double4* base, int n, int v) {
    const float4* q = reinterpret_cast<const float4*>(base);
    const float4 h = __ldg(q + v), l = __ldg(q + n + v);
    return {h.x, h.y, h.z, h.w, l.x, l.y, l.z, l.w};
}
__device__ __forceinline__ ff4 ld_ff4(const double4* base, int n, int v) {   // coherent: written in this launch
    const float4* q = reinterpret_cast<const float4*>(base);
    const float4 h = __ldcg(q + v), l = __ldcg(q + n + v);
    return {h.x, h.y, h.z, h.w, l.x, l.y, l.z, l.w};
}
__device__ __forceinline__ void st_ff4(double4* base, int n, int v, const ff4& a) {
    float4* q = reinterpret_cast<float4*>(base);
    q[v] = make_float4(a.hx, a.hy, a.hz, a.hw);
    q[n + v] = make_float4(a.lx, a.ly, a.lz, a.lw);
}
__device__ __forceinline__ ff ld_ff(const double* base, int n, int v) {
    const float* q = reinterpret_cast<const float*>(base);
    return {__ldg(q + v), __ldg(q + n + v)};
}
__device__ __forceinline__ void st_ff(double* base, int n, int v, ff a) {
    float* q = reinterpret_cast<float*>(base);
    q[v] = a.hi;
    q[n + v] = a.lo;
}
__device__ __forceinline__ float4 ld_acc(const double4* base, int v) {
    return __ldg(reinterpret_cast<const float4*>(base) + v);
}
__device__ __forceinline__ void st_acc(double4* base, int v, float4 a) { reinterpret_cast<float4*>(base)[v] = a; }
__device__ __forceinline__ float ld_rho(const double* base, int v) { return __ldg(reinterpret_cast<const float*>(base) + v); }
// a position (triple-float x, y; float-float z) as doubles (area, substrate location)
__device__ __forceinline__ void pos_d(const ff4& a, double x[3]) {
    x[0] = tf_to_d(tfx(a)); x[1] = tf_to_d(tfy(a)); x[2] = ff_to_d(ffz(a));
}
// a float-float vector as doubles
__device__ __forceinline__ void vec_d(const ff4& a, double x[3]) {
    x[0] = ff_to_d(ffx(a)); x[1] = ff_to_d(ffy(a)); x[2] = ff_to_d(ffz(a));
}

constexpr int kRec = 3;      // float4 per vertex record
constexpr int kSlot32 = 20;  // floats per element slot in shared memory

// kfa * f - R, with kfa * f exact (FMA TwoProduct) and R float-float: one final rounding
__device__ __forceinline__ float net_force(float kfa, float f, ff R) {
    const float p = kfa * f;
    const ff prod = {p, __fmaf_rn(kfa, f, -p)};
    return ff_sub(prod, R).hi;
}

// MD force-extension fit (UL:1203-1214) as float-float constants (hi, lo)
#define FFH(x) ((float)(x))
#define FFL(x) ((float)((x) - (double)(float)(x)))
#define FF6(m, a, b, c, d, e, f) {m(a), m(b), m(c), m(d), m(e), m(f)}
#define MD_PX 0., 2.51250583e-03, 4.40265201e-03, 5.91408228e-03, 11.76817302e-03, 17.001e-03
#define MD_PY -7.15514497, 71.80501308, 356.62420075, 356.96656556, 126.21811585, 528.40481124
#define MD_K 31426.8556, 99485.86235, 67080.67086, -7908.39043, 21978.66923, 76858.39733
#define FF6H(...) FF6(FFH, __VA_ARGS__)
#define FF6L(...) FF6(FFL, __VA_ARGS__)
static __constant__ float c_md_pxh[6] = FF6H(MD_PX), c_md_pxl[6] = FF6L(MD_PX);
static __constant__ float c_md_pyh[6] = FF6H(MD_PY), c_md_pyl[6] = FF6L(MD_PY);
static __constant__ float c_md_kh[6] = FF6H(MD_K), c_md_kl[6] = FF6L(MD_K);
__device__ __forceinline__ ff md_px(int j) { return {c_md_pxh[j], c_md_pxl[j]}; }
__device__ __forceinline__ ff md_py(int j) { return {c_md_pyh[j], c_md_pyl[j]}; }
__device__ __forceinline__ ff md_k(int j) { return {c_md_kh[j], c_md_kl[j]}; }

// MD force-extension fit (UL:1203-1214) in FP32
static __constant__ float c_md_px32[6] = {0.f, 2.51250583e-03f, 4.40265201e-03f, 5.91408228e-03f, 11.76817302e-03f, 17.001e-03f};
static __constant__ float c_md_py32[6] = {-7.15514497f, 71.80501308f, 356.62420075f, 356.96656556f, 126.21811585f, 528.40481124f};
static __constant__ float c_md_k32[6] = {31426.8556f, 99485.86235f, 67080.67086f, -7908.39043f, 21978.66923f, 76858.39733f};

// Spring force of bond u = (ux, uy, uz) + (lx, ly, lz) (float-float) in FP32 (UL:1245-1264;
// k1 UL:1259-1261; the polynomial extension).  The MD table is discontinuous at its
// breakpoints (a jump of 285 pN at 4.4 nm), so its branch is chosen on the float-float
// extension, as the binary64 form would choose it; the force within the branch is FP32.
__device__ __forceinline__ void spring_force32(const ParamF& p, float ux, float uy, float uz, float lx, float ly,
                                               float lz, float fs[3]) {
    const float D = sqrtf(ux * ux + uy * uy + uz * uz);
    const float k = p.k_lin, L0 = p.rest_len;
    if (p.law == PF_LINEAR0) {
        fs[0] = k * ux; fs[1] = k * uy; fs[2] = k * uz;
        return;
    }
    const float iD = D != 0.0f ? 1.0f / D : 0.0f;
    float mag = 0.0f;
    if (p.law == PF_MD) {
        const ff X = {ux, lx}, Y = {uy, ly}, Z = {uz, lz};
        const ff Dff = ff_sqrt(ff_add(ff_add(ff_mul(X, X), ff_mul(Y, Y)), ff_mul(Z, Z)));
        int j = -1;
        if (!ff_lt(Dff, md_px(5))) j = 5;
        else {
#pragma unroll
            for (int q = 0; q < 5; ++q)
                if (ff_lt(Dff, md_px(q + 1)) && !ff_lt(Dff, md_px(q))) j = q;
        }
        if (j >= 0) mag = c_md_py32[j] + c_md_k32[j] * (D - c_md_px32[j]);
    } else if (p.law == PF_LINEAR) {
        mag = D > L0 ? k * (D - L0) : 0.0f;   // slack below the rest length
    } else {
        const float e = D - L0;
        mag = e > 0.0f ? p.poly_k0 * (e + e * e * e * p.poly_c3) : 0.0f;
    }
    fs[0] = mag * ux * iD; fs[1] = mag * uy * iD; fs[2] = mag * uz * iD;
}

// Bell force magnitude of updateFA (UL:2137; k1 UL:2077) in float-float.  The off-rate
// k_a exp(F / F_a) turns a relative error e of F into (F / F_a) e, so F is carried
// to about 48 bits.
__device__ __forceinline__ ff bell_ff(const ParamF& p, ff ux, ff uy, ff uz) {
    const ff k = {p.k_lin, p.k_lin_lo}, L0 = {p.rest_len, p.rest_len_lo};
    const ff d2xy = ff_add(ff_mul(ux, ux), ff_mul(uy, uy));
    const ff d2 = ff_add(d2xy, ff_mul(uz, uz));
    if (p.law == PF_LINEAR0) return ff_mul(k, ff_sqrt(p.norm2d ? d2xy : d2));
    if (p.law == PF_LINEAR) {   // slack below the rest length
        const ff e = ff_sub(ff_sqrt(p.norm2d ? d2xy : d2), L0);
        return (e.hi > 0.0f || (e.hi == 0.0f && e.lo > 0.0f)) ? ff_mul(k, e) : ff{0.0f, 0.0f};
    }
    const ff D = ff_sqrt(d2);
    if (p.law == PF_MD) {
        int j = -1;
        if (!ff_lt(D, md_px(5))) j = 5;
        else
            for (int q = 0; q < 5; ++q)
                if (ff_lt(D, md_px(q + 1)) && !ff_lt(D, md_px(q))) j = q;
        if (j < 0 || D.hi == 0.0f) return {0.0f, 0.0f};
        return ff_abs(ff_add(md_py(j), ff_mul(md_k(j), ff_sub(D, md_px(j)))));
    }
    const ff e = ff_sub(D, L0);
    if (!(e.hi > 0.0f || (e.hi == 0.0f && e.lo > 0.0f))) return {0.0f, 0.0f};   // slack
    const ff c3 = {p.poly_c3, p.poly_c3_lo}, k0 = {p.poly_k0, p.poly_k0_lo};
    return ff_mul(k0, ff_add(e, ff_mul(ff_mul(ff_mul(e, e), e), c3)));
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

// A float-float scalar with the arithmetic operators (wcfe_ff.cuh), for element2d_ff.
struct fq {
    ff v;
    __device__ __forceinline__ fq() : v{0.0f, 0.0f} {}
    __device__ __forceinline__ fq(float x) : v{x, 0.0f} {}
    __device__ __forceinline__ fq(ff x) : v(x) {}
    __device__ __forceinline__ float f() const { return v.hi; }
};
__device__ __forceinline__ fq operator+(fq a, fq b) { return ff_add(a.v, b.v); }
__device__ __forceinline__ fq operator-(fq a, fq b) { return ff_sub(a.v, b.v); }
__device__ __forceinline__ fq operator*(fq a, fq b) { return ff_mul(a.v, b.v); }
__device__ __forceinline__ fq operator/(fq a, fq b) { return ff_div(a.v, b.v); }
__device__ __forceinline__ fq operator-(fq a) { return ff{-a.v.hi, -a.v.lo}; }

// element2d with every intermediate in float-float (about 48 bits) from the same FP32
// records, the outputs rounded to FP32 once: the mixed form's float-float element
// (wcfe_engine_set_element_precision), for runs whose accuracy the FP32 element's own
// roundings would limit.  The reference edges and the step's displacement differences are
// formed exactly from the record's words (TwoSum).
__device__ __forceinline__ void element2d_ff(const float4 r[3][kRec], const ElemParams& q, Elem2& o) {
    const fq G1x = two_sum(r[1][0].x - r[0][0].x, r[1][0].z - r[0][0].z);
    const fq G1y = two_sum(r[1][0].y - r[0][0].y, r[1][0].w - r[0][0].w);
    const fq G2x = two_sum(r[2][0].x - r[0][0].x, r[2][0].z - r[0][0].z);
    const fq G2y = two_sum(r[2][0].y - r[0][0].y, r[2][0].w - r[0][0].w);
    const fq d1x = two_sum(r[1][1].x, -r[0][1].x), d1y = two_sum(r[1][1].y, -r[0][1].y);
    const fq d2x = two_sum(r[2][1].x, -r[0][1].x), d2y = two_sum(r[2][1].y, -r[0][1].y);
    const fq Gc = G1x * G2y - G1y * G2x;
    const fq iG = fq(1.0f) / Gc;
    const fq b1x = G2y * iG, b1y = -(G2x * iG);
    const fq b2x = -(G1y * iG), b2y = G1x * iG;
    const fq b0x = -(b1x + b2x), b0y = -(b1y + b2y);
    const fq H00 = d1x * b1x + d2x * b2x, H01 = d1x * b1y + d2x * b2y;
    const fq H10 = d1y * b1x + d2y * b2x, H11 = d1y * b1y + d2y * b2y;
    const fq gc = (G1x + d1x) * (G2y + d2y) - (G1y + d1y) * (G2x + d2x);
    const fq third = fq(1.0f) / fq(3.0f);
    const fq exx = third * (fq(r[0][1].z) + r[1][1].z + r[2][1].z);
    const fq eyy = third * (fq(r[0][1].w) + r[1][1].w + r[2][1].w);
    const fq exy = third * (fq(r[0][2].x) + r[1][2].x + r[2][2].x);
    const fq ezz = third * (fq(r[0][2].y) + r[1][2].y + r[2][2].y);
    const fq one(1.0f), two(2.0f);
    const fq m00 = one - two * exx, m11 = one - two * eyy, m01 = -(two * exy);
    const fq dm1 = -(two * (exx + eyy)) + fq(4.0f) * (exx * eyy - exy * exy);
    const fq idM = one / (one + dm1);
    const fq i00 = m11 * idM, i01 = -(m01 * idM), i11 = m00 * idM;
    const fq be00 = two * (exx * i00 + exy * i01), be01 = two * (exx * i01 + exy * i11);
    const fq be11 = two * (exy * i01 + eyy * i11);
    const fq de = dm1 - two * ezz * (one + dm1);
    const fq c00 = two * H00 + (H00 * H00 + H10 * H10);
    const fq c11 = two * H11 + (H01 * H01 + H11 * H11);
    const fq c01 = H01 + H10 + (H00 * H01 + H10 * H11);
    const fq dC = (one + c00) * (one + c11) - c01 * c01;
    const fq iC = one / dC;
    const fq ci00 = (one + c11) * iC, ci01 = -(c01 * iC), ci11 = (one + c00) * iC;
    const fq ga00 = -(c00 * ci00 + c01 * ci01), ga01 = -(c00 * ci01 + c01 * ci11);
    const fq ga11 = -(c01 * ci01 + c11 * ci11);
    const fq dth = (H00 + H11) + (H00 * H11 - H01 * H10);
    const fq g = q.grow, thg = one + g, gg2 = two * g + g * g;
    const fq one_dth = one + dth;
    const fq eta = (gg2 + thg * thg * de - two * dth - dth * dth) / (one_dth * one_dth);
    const fq c0 = -(gg2 + thg * thg * eta) / thg;
    const fq ith = one / thg, tge = thg * (one + eta);
    const fq mu = q.mu;
    fq S00 = mu * (c0 + be00 * ith - tge * ga00);
    fq S01 = mu * (be01 * ith - tge * ga01);
    fq S11 = mu * (c0 + be11 * ith - tge * ga11);
    if (q.t_an != 0.0f) {  // anisotropic active stress t_act (1 - 2 kappa) a0 a0^T (direction in FP32)
        float ax = (1.0f / 3.0f) * ((r[0][0].x + r[1][0].x + r[2][0].x) + (r[0][0].z + r[1][0].z + r[2][0].z) +
                                    (r[0][1].x + r[1][1].x + r[2][1].x)) - q.cx;
        float ay = (1.0f / 3.0f) * ((r[0][0].y + r[1][0].y + r[2][0].y) + (r[0][0].w + r[1][0].w + r[2][0].w) +
                                    (r[0][1].y + r[1][1].y + r[2][1].y)) - q.cy;
        const float ia = rsqrtf(ax * ax + ay * ay);
        ax *= ia; ay *= ia;
        S00 = S00 + fq(q.t_an) * fq(ax * ax); S01 = S01 + fq(q.t_an) * fq(ax * ay);
        S11 = S11 + fq(q.t_an) * fq(ay * ay);
    }
    const fq si = q.s_iso;
    const fq T00 = si * H00 + S00 + (H00 * S00 + H01 * S01);
    const fq T01 = si * H01 + S01 + (H00 * S01 + H01 * S11);
    const fq T10 = si * H10 + S01 + (H10 * S00 + H11 * S01);
    const fq T11 = si * H11 + S11 + (H10 * S01 + H11 * S11);
    const fq wA = fq(0.5f) * Gc * q.thick;
    o.re[0][0] = (wA * (T00 * b0x + T01 * b0y)).f(); o.re[0][1] = (wA * (T10 * b0x + T11 * b0y)).f();
    o.re[1][0] = (wA * (T00 * b1x + T01 * b1y)).f(); o.re[1][1] = (wA * (T10 * b1x + T11 * b1y)).f();
    o.re[2][0] = (wA * (T00 * b2x + T01 * b2y)).f(); o.re[2][1] = (wA * (T10 * b2x + T11 * b2y)).f();
    const fq iF = one / one_dth;
    const fq f00 = (one + H11) * iF, f01 = -(H01 * iF), f10 = -(H10 * iF), f11 = (one + H00) * iF;
    const fq K00 = -(H00 * f00 + H01 * f10), K01 = -(H00 * f01 + H01 * f11);
    const fq K10 = -(H10 * f00 + H11 * f10), K11 = -(H10 * f01 + H11 * f11);
    const fq EK00 = exx * K00 + exy * K10, EK01 = exx * K01 + exy * K11;
    const fq EK10 = exy * K00 + eyy * K10, EK11 = exy * K01 + eyy * K11;
    const fq KEK00 = K00 * EK00 + K10 * EK10, KEK01 = K00 * EK01 + K10 * EK11;
    const fq KEK11 = K01 * EK01 + K11 * EK11;
    const fq KK00 = K00 * K00 + K10 * K10, KK01 = K00 * K01 + K10 * K11, KK11 = K01 * K01 + K11 * K11;
    const fq half(0.5f);
    const fq D00 = two * EK00 + KEK00 - half * (two * K00 + KK00);
    const fq D11 = two * EK11 + KEK11 - half * (two * K11 + KK11);
    const fq D01 = (EK10 + EK01) + KEK01 - half * (K01 + K10 + KK01);
    const fq tg2 = thg * thg, gg = tg2 - one;
    const fq dvxx = tg2 * D00 + gg * (exx - half), dvyy = tg2 * D11 + gg * (eyy - half);
    const fq dvxy = tg2 * D01 + gg * exy, dvzz = gg * (ezz - half);
    const fq w3 = third * wA;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o.rea[i][0] = (w3 * ((exx - r[i][1].z) + dvxx)).f();
        o.rea[i][1] = (w3 * ((eyy - r[i][1].w) + dvyy)).f();
        o.rea[i][2] = (w3 * ((exy - r[i][2].x) + dvxy)).f();
        o.rea[i][3] = (w3 * ((ezz - r[i][2].y) + dvzz)).f();
    }
    o.mm = w3.f();
    o.acur = fabsf((half * gc).f());
}

constexpr int kBndSlots = 96;    // boundary vertices a patch CTA queues for its second loop (more finish in place)

// Per-cell, per-step constants of the boundary terms (computed once per patch CTA).
struct BndConst {
    ff w;                 // (1/2) kappa t_act thick: isotropic active stress on the open one-ring
    ff area_term;         // -k_area (A - A_0) / 2 (calculateAreaConstraintForce)
    float k_bend, ap_force;
    ff half_density;      // ap_density / 2
    uint32_t ap_thr;      // r31 < ap_thr  <=>  r31 / 2^31 < ap_rate dt exp(-ap_rate dt)
    int32_t ap_enable;
    uint32_t seed, stream;
    unsigned long long ap_call;
};

__device__ __forceinline__ BndConst make_bnd_const(const CellDev& c, const MixedArgs& a, unsigned long long ap_call) {
    const wcfe_params& p = c.prm;
    const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
    const double s_iso = p.kappa * (t < p.tact_t1 ? t * p.tact_rate : p.tact_max);
    const double apt = isnan(a.ap_thresh) ? c.ap_thresh : a.ap_thresh;
    BndConst b;
    b.w = ff_from_d(0.5 * s_iso * p.thick);
    b.area_term = ff_from_d(-p.k_area * (c.area4[0] - p.area0) / 2);
    b.k_bend = (float)p.k_bend;
    b.ap_force = (float)p.ap_force;
    b.half_density = ff_from_d(p.ap_density / 2);
    const double thr = ceil(apt * 2147483648.0);
    b.ap_thr = thr <= 0.0 ? 0u : (thr >= 4294967295.0 ? 4294967295u : (uint32_t)thr);
    b.ap_enable = p.ap_enable;
    b.seed = p.seed;
    b.stream = p.stream;
    b.ap_call = ap_call;
    return b;
}

// The cell constants of one mixed-form step, formed once per cell by the vertex phase's
// finishing block (it has the cell's area and centroid) and read by every patch CTA.
struct StepConst {
    ElemParams q;
    BndConst b;
};
static_assert(sizeof(StepConst) <= 128, "step constants exceed their slot");

__device__ __forceinline__ StepConst make_step_const(const CellDev& c, double dt_real, double area, double cx,
                                                     double cy) {
    const wcfe_params& p = c.prm;
    const double t = c.clk[0];
    const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
    StepConst s;
    s.q.mu = (float)p.mu;
    s.q.thick = (float)p.thick;
    s.q.grow = (float)(p.thetag_dot * dt_real);
    s.q.s_iso = (float)(p.kappa * t_act);
    s.q.t_an = (float)((1.0 - 2.0 * p.kappa) * t_act);
    s.q.cx = (float)cx;
    s.q.cy = (float)cy;
    const double s_iso = p.kappa * t_act;
    s.b.w = ff_from_d(0.5 * s_iso * p.thick);
    s.b.area_term = ff_from_d(-p.k_area * (area - p.area0) / 2);
    s.b.k_bend = (float)p.k_bend;
    s.b.ap_force = (float)p.ap_force;
    s.b.half_density = ff_from_d(p.ap_density / 2);
    const double thr = ceil(c.ap_thresh * 2147483648.0);
    s.b.ap_thr = thr <= 0.0 ? 0u : (thr >= 4294967295.0 ? 4294967295u : (uint32_t)thr);
    s.b.ap_enable = p.ap_enable;
    s.b.seed = p.seed;
    s.b.stream = p.stream;
    s.b.ap_call = c.ap[0];
    return s;
}

// The neighbour frame of a boundary vertex (UL:1500-1531): the candidate scan of
// boundary_frame, with the orientation test on float-float differences.
__device__ __forceinline__ bool boundary_frame_ff(const CellDev& c, const double4* __restrict__ xp, int rank,
                                                  const ff4& xi, ff4& x1, ff4& x2) {
    int j1 = -1, j2 = -1;
    for (int k = c.bnd_cptr[rank]; k < c.bnd_cptr[rank + 1]; ++k) {
        const int2 cd = c.bnd_cand[k];
        const ff4 pb = ldg_ff4(xp, c.nv, cd.x), pi = ldg_ff4(xp, c.nv, cd.y);
        const ff d1x = ff_sub(ffx(xi), ffx(pb)), d1y = ff_sub(ffy(xi), ffy(pb));
        const ff d2x = ff_sub(ffx(pi), ffx(xi)), d2y = ff_sub(ffy(pi), ffy(xi));
        const ff ncz = ff_sub(ff_mul(d1x, d2y), ff_mul(d1y, d2x));
        if (ncz.hi > 0.0f) j1 = cd.x;
        else j2 = cd.x;
    }
    if (j1 < 0 || j2 < 0) return false;
    x1 = ldg_ff4(xp, c.nv, j1);
    x2 = ldg_ff4(xp, c.nv, j2);
    return true;
}

// The step-start position of vertex j as its element record holds it: triple-float x, y
// (the record's float-float (h, m) pair and the third floats in its last two slots).
__device__ __forceinline__ void rec_pos(const float4* __restrict__ rp, int j, tf& x, tf& y) {
    const float4 r0 = __ldg(rp + kRec * (size_t)j), r2 = __ldg(rp + kRec * (size_t)j + 2);
    x = {r0.x, r0.z, r2.z};
    y = {r0.y, r0.w, r2.w};
}

// Boundary terms of vertex v (rank `rank`) added to (F0, F1) in float-float, on the
// triple-float positions: the isotropic active stress of the open one-ring, AP push
// (calculateForce_AP UL:1477-1569), bending (calculateBendingForce2D UL:1571-1689) and
// area constraint (calculateAreaConstraintForce UL:1691-1784), on the neighbour frame of
// UL:1500-1531 (in the plane: the mixed form keeps z = 0).  On a boundary these forces
// nearly balance one another (a cell whose edge is at rest moves by the small remainder),
// so each is formed and summed in float-float: FP32 terms would leave their own 6e-8
// relative rounding on a net force a hundred times smaller.  The turning-angle term
// 1 - cos(theta) is |e1 - e2|^2 / 2 with e1 - e2 = (d1 l2 - d2 l1) / (l1 l2); the unit
// normal is (d1 + d2) x e3 / L, the reference's length-weighted mean of the two edge
// normals.  The AP bond count ceil(density L / 2) is taken on the float-float L.
// The step-start positions X come from the step's element records rp (the step-start
// position buffer may be overwritten by a fused next-step prediction while this runs);
// xp holds the predicted positions.
__device__ __forceinline__ void boundary_force(const CellDev& c, const BndConst& bc, const int4& pt,
                                               const float4* __restrict__ rp, const double4* __restrict__ xp, int v,
                                               int rank, ff& F0, ff& F1) {
    const ff4 xi = ldg_ff4(xp, c.nv, v);
    // isotropic active stress on the open one-ring: (1/2) s_iso thick e3 x sum (X_k - X_j)
    ff sx = {0.0f, 0.0f}, sy = {0.0f, 0.0f};
    for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
        const int code = c.vc_code[k];
        const int cn = code & 3;
        const int e = c.patch_elems[pt.z + (code >> 2)];
        const int4 t4 = c.tri[e];
        const int ids[3] = {t4.x, t4.y, t4.z};
        tf Xjx, Xjy, Xkx, Xky;
        rec_pos(rp, ids[(cn + 1) % 3], Xjx, Xjy);
        rec_pos(rp, ids[(cn + 2) % 3], Xkx, Xky);
        sx = ff_add(sx, tf_sub(Xkx, Xjx));
        sy = ff_add(sy, tf_sub(Xky, Xjy));
    }
    ff Fb0 = ff_mul(bc.w, sy), Fb1 = ff_mul(bc.w, sx);   // minus the residual term w e3 x s
    Fb1 = {-Fb1.hi, -Fb1.lo};
    ff4 x1, x2;
    if (boundary_frame_ff(c, xp, rank, xi, x1, x2)) {
        const ff D1x = tf_sub(tfx(xi), tfx(x1)), D1y = tf_sub(tfy(xi), tfy(x1));
        const ff D2x = tf_sub(tfx(x2), tfx(xi)), D2y = tf_sub(tfy(x2), tfy(xi));
        const ff L1 = ff_sqrt(ff_add(ff_mul(D1x, D1x), ff_mul(D1y, D1y)));
        const ff L2 = ff_sqrt(ff_add(ff_mul(D2x, D2x), ff_mul(D2y, D2y)));
        const ff Lf = ff_add(L1, L2);
        const ff nx = ff_div(ff_add(D1y, D2y), Lf);
        const ff nyn = ff_div(ff_add(D1x, D2x), Lf);   // -ny
        ff fb = {0.0f, 0.0f};
        if (bc.ap_enable) {
            const uint32_t r31 = ap_draw(bc.seed, bc.stream, bc.ap_call, (uint32_t)rank);
            const ff lim = ff_mul(Lf, bc.half_density);
            float cnt = 0.0f;
            if (lim.hi > 0.0f || (lim.hi == 0.0f && lim.lo > 0.0f)) {
                cnt = ceilf(lim.hi);
                if (cnt == lim.hi && lim.lo > 0.0f) cnt += 1.0f;
            }
            if (r31 < bc.ap_thr) fb = ff_mul_f({bc.ap_force, 0.0f}, cnt);
        }
        const ff l12 = ff_mul(L1, L2);
        const ff gx = ff_div(ff_sub(ff_mul(D1x, L2), ff_mul(D2x, L1)), l12);
        const ff gy = ff_div(ff_sub(ff_mul(D1y, L2), ff_mul(D2y, L1)), l12);
        ff q = ff_add(ff_mul(gx, gx), ff_mul(gy, gy));   // 2 (1 - cos(theta))
        const float ez = D1x.hi * D2y.hi - D1y.hi * D2x.hi;   // the sign of (e1 x e2).z
        if (ez > 0.0f) q = {-q.hi, -q.lo};                     // turna = -(1 - cos) for a left turn
        fb = ff_add(fb, ff_div(ff_mul_f(q, bc.k_bend), Lf));   // k_bend turna 2 / L
        fb = ff_add(fb, ff_mul(bc.area_term, Lf));
        Fb0 = ff_add(Fb0, ff_mul(fb, nx));
        Fb1 = ff_sub(Fb1, ff_mul(fb, nyn));
    }
    F0 = ff_add(F0, Fb0);
    F1 = ff_add(F1, Fb1);
}

// The radial protrusion driver (wcfe_params.protrude_v; the FP64 form's drive_protrusion):
// a boundary vertex's half-step velocity is v (X - c) / |X - c| in the plane, the speed in
// float-float and the unit direction in FP32 (a 1e-7 error of the direction moves the
// vertex by 1e-7 of one step's travel).
__device__ __forceinline__ void protrude_ff(const CellDev& c, int v, const ff4& X, ff& vh0, ff& vh1) {
    const ParamF& pf = c.pf;
    if ((pf.pv == 0.0f && pf.pv_lo == 0.0f) || c.bnd_rank[v] < 0) return;
    const float dx = ff_sub(ffx(X), {pf.pcx, pf.pcx_lo}).hi, dy = ff_sub(ffy(X), {pf.pcy, pf.pcy_lo}).hi;
    const float r = sqrtf(dx * dx + dy * dy);
    if (r == 0.0f) return;
    vh0 = ff_mul_f({pf.pv, pf.pv_lo}, dx / r);
    vh1 = ff_mul_f({pf.pv, pf.pv_lo}, dy / r);
}

// ===========================================================================
// mixed-form vertex phase: predict (triple-float positions), bond kinetics with FP32
// rates and float-float accumulation, the FP32 element records, and the cell area and
// area-weighted centroid from the boundary loop (shoelace over the directed
// boundary edges).  For a planar mesh without inverted elements that equals
// calculateAreaTot's sum of element areas.
// ===========================================================================
enum { VM_PREDICT = 1, VM_UPDATE_FA = 2, VM_EXPORT = 8, VM_IMPORT = 16, VM_NOAREA = 32 };

// The substrate's displacement under a bond's anchor (a rigid substrate mesh moved by the
// caller), subtracted from the bond vector (UL:2053-2099).  Out of line: few cells have
// one, and its FP64 point location would otherwise set the register budget of every block.
__device__ __noinline__ void substrate_move(const CellDev& c, const ff4& Xv, const ff4& f, ff& u0, ff& u1, ff& u2) {
    double wgt[3], Xd[3], fd[3];
    pos_d(Xv, Xd);
    vec_d(f, fd);
    const int e = locate(c.sub, xs(Xd[0], fd[0]), xs(Xd[1], fd[1]), xs(Xd[2], fd[2]), wgt);
    if (e >= 0) {
        const int4 t = c.sub.tri[e];
        const double4 a0 = ld4(c.sub.x + t.x), a1 = ld4(c.sub.x + t.y), a2 = ld4(c.sub.x + t.z);
        const double4 b0 = ld4(c.sub.X + t.x), b1 = ld4(c.sub.X + t.y), b2 = ld4(c.sub.X + t.z);
        u0 = ff_sub(u0, ff_from_d(wgt[0] * (a0.x - b0.x) + wgt[1] * (a1.x - b1.x) + wgt[2] * (a2.x - b2.x)));
        u1 = ff_sub(u1, ff_from_d(wgt[0] * (a0.y - b0.y) + wgt[1] * (a1.y - b1.y) + wgt[2] * (a2.y - b2.y)));
        u2 = ff_sub(u2, ff_from_d(wgt[0] * (a0.z - b0.z) + wgt[1] * (a1.z - b1.z) + wgt[2] * (a2.z - b2.z)));
    }
}

// The predicted in-plane position of vertex v from its step-start position Xv, velocity V
// and acceleration A: vh = V + (dt/2) A (or the protrusion driver), x = X + dt vh.
__device__ __forceinline__ void predict_xy(const CellDev& c, int v, const VertexArgs& va, const ff4& Xv, const ff4& V,
                                           const float4& A, tf& xn0, tf& xn1, ff& vh0, ff& vh1) {
    vh0 = ff_add(ffx(V), ff_mul_f(va.hdt, A.x));
    vh1 = ff_add(ffy(V), ff_mul_f(va.hdt, A.y));
    protrude_ff(c, v, Xv, vh0, vh1);
    xn0 = tf_add_ff(tfx(Xv), ff_mul(va.dt, vh0));
    xn1 = tf_add_ff(tfy(Xv), ff_mul(va.dt, vh1));
}

// The cell area and centroid of the positions pos(u, x) gives (shoelace over the directed
// boundary edges), then the step constants of the patch phase that follows.  Called by all
// threads of one block of any size that is a multiple of 32 dividing 256; the sum has one
// fixed order whatever the block size: boundary ranks strided over 256 virtual threads, the
// 32 lanes of each virtual warp by a butterfly, then the 8 virtual warps in order.  s_w: 24
// doubles of shared scratch.
template <class Pos>
__device__ void shoelace_step_const(const CellDev& c, Pos pos, double dt_real, double* s_w) {
    constexpr int kVW = kK1Threads / 32;
    const int lane = threadIdx.x & 31;
    for (int vw = threadIdx.x >> 5; vw < kVW; vw += blockDim.x >> 5) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int r = vw * 32 + lane; r < c.nb; r += kK1Threads) {
            double xi[3];
            pos(c.bnd_vert[r], xi);
            for (int k = c.bnd_optr[r]; k < c.bnd_optr[r + 1]; ++k) {
                double xj[3];
                pos(c.bnd_out[k], xj);
                const double cr = xi[0] * xj[1] - xj[0] * xi[1];
                s0 += 0.5 * cr;
                s1 += (1.0 / 6.0) * (xi[0] + xj[0]) * cr;
                s2 += (1.0 / 6.0) * (xi[1] + xj[1]) * cr;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            s_w[3 * vw] = s0; s_w[3 * vw + 1] = s1; s_w[3 * vw + 2] = s2;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double A = 0, Ax = 0, Ay = 0;
        for (int w = 0; w < kVW; ++w) {
            A += s_w[3 * w]; Ax += s_w[3 * w + 1]; Ay += s_w[3 * w + 2];
        }
        c.area4[0] = A;
        c.area4[1] = Ax / A;
        c.area4[2] = Ay / A;
        c.area4[3] = 0.0;
        *reinterpret_cast<StepConst*>(c.stepc) = make_step_const(c, dt_real, A, Ax / A, Ay / A);
    }
    __syncthreads();   // the scratch may be reused by the caller
}

// shoelace_step_const on positions stored in xo, after every store of them is visible (out of
// line, as is area_predicted: its FP64 registers stay off the vertices' path)
__device__ __noinline__ void area_shoelace(const CellDev& c, const double4* xo, double dt_real, double* s_w) {
    shoelace_step_const(c, [&](int u, double* x) { pos_d(ld_ff4(xo, c.nv, u), x); }, dt_real, s_w);
}

// shoelace_step_const on the predictions of the step at parity par, formed here from the
// step-start state with the arithmetic of vertex_predict (the same values its blocks store),
// so that it needs no store of this step's vertex phase
__device__ __noinline__ void area_predicted(const CellDev& c, int par, const VertexArgs& va, double* s_w) {
    shoelace_step_const(
        c,
        [&](int u, double* x) {
            const ff4 Xu = ldg_ff4(c.pos[par], c.nv, u);
            tf x0, x1;
            ff h0, h1;
            predict_xy(c, u, va, Xu, ldg_ff4(c.vel, c.nv, u), ld_acc(c.acc, u), x0, x1, h0, h1);
            pos_d(make_pos4(x0, x1, ffz(Xu)), x);
        },
        va.dtd, s_w);
}

// The vertex phase's cell area where this launch stores the positions it sums (imported
// ones): the last block of the cell to finish (ticket ctl[2]) reads the positions the other
// blocks wrote (through L2) and runs area_shoelace.
__device__ __forceinline__ void finish_area_boundary(const CellDev& c, const double4* xo, double dt_real) {
    __shared__ int s_last;
    __shared__ double s_w[3 * kK1Threads / 32];
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 2), 1u);
        s_last = ((int)t == c.nk1 - 1);
        if (s_last) c.ctl[2] = 0;
    }
    __syncthreads();
    if (!s_last) return;   // block-uniform
    __threadfence();
    area_shoelace(c, xo, dt_real, s_w);
}

// The prediction of vertex v at step parity par (predict_xy), stored in pos[par ^ 1] (and,
// for the exchange path, vh, and x as binary64 into xq[0..2]).
__device__ __forceinline__ void vertex_predict(const CellDev& c, int v, int par, const VertexArgs& va, const ff4& Xv,
                                               const ff4& V, const float4& A, tf& xn0, tf& xn1, ff& xn2,
                                               double* xq = nullptr) {
    ff vh0, vh1;
    predict_xy(c, v, va, Xv, V, A, xn0, xn1, vh0, vh1);
    xn2 = ffz(Xv);
    st_ff4(c.pos[par ^ 1], c.nv, v, make_pos4(xn0, xn1, xn2));
    if (va.flags & VM_EXPORT) {
        st_ff4(c.vhl, c.nv, v, make_ff4(vh0, vh1, {0.0f, 0.0f}));
        xq[0] = tf_to_d(xn0); xq[1] = tf_to_d(xn1); xq[2] = ff_to_d(xn2);
    }
}

// Bond kinetics of vertex v at step parity par on the step displacement x - X (bond vector
// f, bond density c_C = cold, c_A = cAv as loaded before), and its FP32 element record
// rec[par] (strain hi eh).
__device__ __forceinline__ void vertex_kinetics(const CellDev& c, int v, int par, const VertexArgs& va, const ff4& Xv,
                                                const ff4& f, ff cold, ff cAv, const float4& eh, const tf& xn0,
                                                const tf& xn1) {
    const int flags = va.flags;
    const ff cu0 = tf_sub(xn0, tfx(Xv)), cu1 = tf_sub(xn1, tfy(Xv));   // step displacement
    if (flags & VM_UPDATE_FA) {
        const ParamF& pf = c.pf;
        ff u0 = ff_add(ffx(f), cu0), u1 = ff_add(ffy(f), cu1), u2 = ffz(f);
        if (c.has_sub && c.sub.moving) substrate_move(c, Xv, f, u0, u1, u2);
        // Bell kinetics (UL:2137-2171): k_off from the float-float force, the c_C update in float-float
        const ff F = bell_ff(pf, u0, u1, u2);
        const ff xa = ff_mul(F, {pf.iFa, pf.iFa_lo}), xb = ff_mul(F, {pf.iFb, pf.iFb_lo});
        // the exponent is capped below FP32 overflow (e^88 ~ 1.7e38): any force that large already
        // gives dt k_off >> 1, i.e. the same decisions as the unbounded FP64 rate
        const float koff = pf.ka * expf(fminf(xa.hi, 88.0f)) * (1.0f + xa.lo) + pf.kb * expf(-xb.hi) * (1.0f - xb.lo);
        const float coldf = cold.hi, kon = pf.k_on, dtf = va.dtf;
        const ff rate = ff_sub(ff_mul_f(ff_sub({1.0f, 0.0f}, cold), kon), ff_mul_f(cold, koff));
        ff cn = ff_add(cold, ff_mul(va.dt, rate));
        if (cn.hi < 0.0f) cn = {0.0f, 0.0f};
        if (cAv.hi < 0.0f) st_ff(c.cA, c.nv, v, {0.0f, 0.0f});
        ff n0, n1, n2;
        const bool keep_pos = coldf > 0.0f && (1.0f - dtf * koff) > 0.0f;
        if (keep_pos && cn.hi > 0.0f) {
            // keep / c_new = 1 + ds with ds = -dt k_on (1 - c_old) / c_new exactly
            const float ds = -dtf * kon * (1.0f - coldf) / cn.hi;
            n0 = ff_add(u0, ff_mul_f(u0, ds)); n1 = ff_add(u1, ff_mul_f(u1, ds)); n2 = ff_add(u2, ff_mul_f(u2, ds));
        } else {
            n0 = {0.0f * u0.hi, 0.0f}; n1 = {0.0f * u1.hi, 0.0f}; n2 = {0.0f * u2.hi, 0.0f};
        }
        st_ff(c.cC, c.nv, v, cn);
        st_ff4(c.fau, c.nv, v, make_ff4(n0, n1, n2));
    }
    if (!(flags & VM_EXPORT)) {
        // r0 = (X.x h, X.y h, X.x m, X.y m), r1 = (u.x, u.y, exx, eyy), r2 = (exy, ezz, X.x l, X.y l)
        float4* r = c.rec[par] + kRec * (size_t)v;
        r[0] = make_float4(Xv.hx, Xv.hy, Xv.lx, Xv.ly);
        r[1] = make_float4(cu0.hi, cu1.hi, eh.x, eh.y);
        r[2] = make_float4(eh.w, eh.z, Xv.hw, Xv.lw);
    }
    // boundary positions are read by the block that finishes the area
    if (!(flags & VM_NOAREA) && c.bnd_rank[v] >= 0) __threadfence();
}

// One vertex of the vertex phase at step parity par: predict into pos[par ^ 1] (or take
// the caller's positions), bond kinetics with FP32 rates and float-float accumulation,
// and the FP32 element record rec[par].  xq: the vertex's three binary64 coordinates of
// the exchange (read with VM_IMPORT, written with VM_EXPORT).
__device__ __forceinline__ void vertex_mixed_body(const CellDev& c, int v, int par, const VertexArgs& va,
                                                  double* xq) {
    const int flags = va.flags;
    double4* __restrict__ xo = c.pos[par ^ 1];
    const ff4 Xv = ldg_ff4(c.pos[par], c.nv, v);
    // every load of this vertex's state up front: none depends on the prediction's stores
    const bool do_fa = (flags & VM_UPDATE_FA) != 0;
    const ff4 f = do_fa ? ldg_ff4(c.fau, c.nv, v) : ff4{};
    const ff cold = do_fa ? ld_ff(c.cC, c.nv, v) : ff{0.0f, 0.0f};
    const ff cAv = do_fa ? ld_ff(c.cA, c.nv, v) : ff{0.0f, 0.0f};
    const float4 eh = __ldg(reinterpret_cast<const float4*>(c.ea[par]) + v);   // (xx, yy, zz, xy) hi
    // positions are triple-float (wcfe_ff.cuh); the step displacement cu is float-float
    tf xn0, xn1;
    ff xn2 = ffz(Xv);
    if (flags & VM_IMPORT) {
        // a coordinate the caller returned as the binary64 rounding of the predicted one keeps
        // the predicted triple-float (so the exchange path steps exactly as the internal one);
        // any other value is taken as given
        const double* qq = xq;
        const ff4 pr = ld_ff4(xo, c.nv, v);
        const tf p0 = tfx(pr), p1 = tfy(pr);
        xn0 = tf_to_d(p0) == qq[0] ? p0 : tf_from_d(qq[0]);
        xn1 = tf_to_d(p1) == qq[1] ? p1 : tf_from_d(qq[1]);
        xn2 = ff_from_d(qq[2]);
        st_ff4(xo, c.nv, v, make_pos4(xn0, xn1, xn2));
    } else if (flags & VM_PREDICT) {
        vertex_predict(c, v, par, va, Xv, ldg_ff4(c.vel, c.nv, v), ld_acc(c.acc, v), xn0, xn1, xn2, xq);
    } else {
        const ff4 t = ld_ff4(xo, c.nv, v);
        xn0 = tfx(t); xn1 = tfy(t); xn2 = ffz(t);
    }
    vertex_kinetics(c, v, par, va, Xv, f, cold, cAv, eh, xn0, xn1);
}

// The next step's vertex-phase inputs of an owned vertex in a fused patch phase: its
// predicted position (the next step-start position), bond vector, c_C and c_A.
struct FusedIn {
    ff4 X, f;
    ff cold, cA;
};

// Explicit update of vertex v (UL:592-628): the acceleration in FP32 from the force; the
// velocity and the strain accumulate in float-float.  A boundary vertex (exact = true)
// brings a float-float force and forms F - drag vh - damp m V in float-float (its terms
// nearly cancel); an interior vertex brings its FP32 force (F0.lo = 0).  V, A and the
// strain (xx yy zz xy, hi and lo) come in from the caller (global memory or a staged copy).
// nx (fused patch phase): the vertex's next-step inputs; the next step's vertex phase then
// runs on it here, from the new velocity, acceleration and strain still in registers.
__device__ __forceinline__ void finish_vertex_core(const CellDev& c, const MixedArgs& a, int par, int v, ff F0,
                                                   ff F1, bool exact, float Q0, float Q1, float Q2, float Q3,
                                                   float MMf, const ff4& V, const float4& A, const float4& eh,
                                                   const float4& el, const FusedIn* nx = nullptr) {
    const ParamF& pf = c.pf;
    ff vh0, vh1;
    if (a.vh_from_buf) {
        const ff4 h = ldg_ff4(c.vhl, c.nv, v);
        vh0 = ffx(h); vh1 = ffy(h);
    } else {
        vh0 = ff_add(ffx(V), ff_mul_f(a.hdt, A.x));
        vh1 = ff_add(ffy(V), ff_mul_f(a.hdt, A.y));
        if (c.pf.pv != 0.0f && c.bnd_rank[v] >= 0) protrude_ff(c, v, ldg_ff4(c.pos[par], c.nv, v), vh0, vh1);
    }
    const float rhom = pf.rho;
    const float iM = 1.0f / (MMf * rhom);
    const float damp_m = pf.damp * MMf * rhom;
    float An0, An1;
    if (exact) {
        An0 = ff_mul_f(ff_sub(F0, ff_add(ff_mul_f(vh0, pf.drag), ff_mul_f(ffx(V), damp_m))), iM).hi;
        An1 = ff_mul_f(ff_sub(F1, ff_add(ff_mul_f(vh1, pf.drag), ff_mul_f(ffy(V), damp_m))), iM).hi;
    } else {
        An0 = (F0.hi - pf.drag * vh0.hi - damp_m * V.hx) * iM;
        An1 = (F1.hi - pf.drag * vh1.hi - damp_m * V.hy) * iM;
    }
    const float An2 = V.hz == 0.0f ? 0.0f : (-damp_m * V.hz) * iM;  // no force normal to the plane
    ff Vn0, Vn1, Vn2;
    if (a.half) {
        Vn0 = ff_add(vh0, ff_mul_f(a.cdt, An0));
        Vn1 = ff_add(vh1, ff_mul_f(a.cdt, An1));
        Vn2 = ff_mul_f(a.cdt, An2);
    } else {
        Vn0 = ff_add(ffx(V), ff_mul_f(a.dtr, An0));
        Vn1 = ff_add(ffy(V), ff_mul_f(a.dtr, An1));
        Vn2 = ff_add(ffz(V), ff_mul_f(a.dtr, An2));
    }
    float4* en = reinterpret_cast<float4*>(c.ea[par ^ 1]);   // (xz, yz) stay as set
    const float iMM = 1.0f / MMf;
    const ff exx = ff_add_f({eh.x, el.x}, Q0 * iMM), eyy = ff_add_f({eh.y, el.y}, Q1 * iMM);
    const ff ezz = ff_add_f({eh.z, el.z}, Q3 * iMM), exy = ff_add_f({eh.w, el.w}, Q2 * iMM);
    en[v] = make_float4(exx.hi, eyy.hi, ezz.hi, exy.hi);
    en[c.nv + v] = make_float4(exx.lo, eyy.lo, ezz.lo, exy.lo);
    st_acc(c.acc, v, make_float4(An0, An1, An2, 0.0f));
    st_ff4(c.vel, c.nv, v, make_ff4(Vn0, Vn1, Vn2));
    // NaN/Inf in the state shows up in the FP32 quantities derived from it
    const float chk = An0 + An1 + Q0 + Q1 + Q2 + vh0.hi + vh1.hi;
    if (!isfinite(chk)) atomicOr(c.status, 1u);
    if (nx) {   // the next step's vertex phase of v, on the values just stored
        tf xn0, xn1;
        ff xn2;
        vertex_predict(c, v, par ^ 1, a.va, nx->X, make_ff4(Vn0, Vn1, Vn2), make_float4(An0, An1, An2, 0.0f), xn0,
                       xn1, xn2);
        vertex_kinetics(c, v, par ^ 1, a.va, nx->X, nx->f, nx->cold, nx->cA,
                        make_float4(exx.hi, eyy.hi, ezz.hi, exy.hi), xn0, xn1);
    }
}

// the next-step inputs of vertex v of a fused patch phase at parity par
__device__ __forceinline__ FusedIn fused_in(const CellDev& c, int par, int v) {
    return {ldg_ff4(c.pos[par ^ 1], c.nv, v), ldg_ff4(c.fau, c.nv, v), ld_ff(c.cC, c.nv, v), ld_ff(c.cA, c.nv, v)};
}

__device__ __forceinline__ void finish_vertex(const CellDev& c, const MixedArgs& a, int par, int v, ff F0, ff F1,
                                              float Q0, float Q1, float Q2, float Q3, float MMf, bool fuse) {
    const float4* eo = reinterpret_cast<const float4*>(c.ea[par]);
    const float4 A = a.vh_from_buf ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_acc(c.acc, v);
    FusedIn nx;
    if (fuse) nx = fused_in(c, par, v);
    finish_vertex_core(c, a, par, v, F0, F1, true, Q0, Q1, Q2, Q3, MMf, ldg_ff4(c.vel, c.nv, v), A, __ldg(eo + v),
                       __ldg(eo + c.nv + v), fuse ? &nx : nullptr);
}

// kfa f - R as float-float (the boundary vertices' force before their boundary terms)
__device__ __forceinline__ ff net_force_ff(float kfa, float f, ff R) {
    const float p = kfa * f;
    return ff_sub({p, __fmaf_rn(kfa, f, -p)}, R);
}
constexpr int kBndRec = 10;   // floats per queued boundary vertex: index, F0 and F1 (hi, lo), Q0-Q3, MM

// MINB: the least CTAs of 128 threads per SM the register allocation must allow (5: 96
// registers; 6, 7, 8: 80, 72, 64 registers, with shared memory then limiting emax); the
// autotuner picks among them.
// FUSED: the fused form (MixedArgs::va), a separate instantiation so that its code does
// not weigh on the register allocation of the plain one.  EMAX > 0: the element-slot
// stride of the shared arrays as a constant (a.emax == EMAX), so that the field offsets
// are immediates; 0: a.emax at run time.  FF: the float-float element (element2d_ff).
template <int MINB, bool FUSED, int EMAX = 0, bool FF = false>
__global__ void __launch_bounds__(128, MINB) k_patch_phase_mixed(MixedArgs a, const CellDev* __restrict__ cells,
                                                                 const WorkItem* __restrict__ work) {
    extern __shared__ float smf[];
    const int emax = EMAX > 0 ? EMAX : a.emax;
    // structure of arrays: field k of slot j at smf[k * emax + j]
    // boundary-queue counts of alternate patches: a patch's count is cleared after the element
    // barrier of the patch before it, when every thread has read it, so no barrier ends a patch
    __shared__ int s_nb2[2], s_last;
    __shared__ float s_bnd[kBndRec * kBndSlots];
    if (threadIdx.x == 0) s_nb2[0] = s_nb2[1] = 0;
    __syncthreads();
    int kp = -1;   // patches this CTA has processed, less one
    for (int w = blockIdx.x; w < a.nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const CellDev& c = cells[it.cell];   // the table is read-only here: its fields stay in registers
        if (cell_done(c)) continue;   // block-uniform: a serving cell that ran its steps
        ++kp;
        int& s_nbnd = s_nb2[kp & 1];
        // fused: predict the cell's next step here unless this step is the last of its budget
        // (ctl[3] is counted down only after every patch of the cell took its ticket)
        const bool fuse = FUSED && c.ctl[3] != 1;
        const int4 pt = c.patch[it.idx];
        const int par = c.ctl[0];
        const double4* __restrict__ xp = c.pos[par ^ 1];
        const float4* __restrict__ rec = c.rec[par];
        const unsigned long long ap_call = c.ap[0];
        // the cell's constants of this step, formed by the vertex phase
        const StepConst& sc = *reinterpret_cast<const StepConst*>(c.stepc);
        const BndConst& s_bc = sc.b;
        const ElemParams q = sc.q;
        // this CTA's next patch: its owned element records and its element slots into L2
        // while this one computes (the records are gathered with dependent loads; the owned
        // state is read coalesced and gains nothing from a prefetch)
        if (threadIdx.x == blockDim.x - 32 && w + (int)gridDim.x < a.nwork) {
            const WorkItem nt = work[w + gridDim.x];
            const CellDev& cn = cells[nt.cell];
            const int4 pn = cn.patch[nt.idx];
            l2_prefetch(cn.rec[cn.ctl[0] & 1] + kRec * (size_t)pn.x, 16u * kRec * (size_t)pn.y);
            l2_prefetch(cn.patch_tri + pn.z, 16u * (size_t)pn.w);
        }
        // ---- elements of the patch -> shared memory ----
        for (int j = threadIdx.x; j < pt.w; j += blockDim.x) {
            const int4 t4 = __ldg(c.patch_tri + pt.z + j);   // (a, b, c, element id)
            const int e = t4.w;
            const int id[3] = {t4.x, t4.y, t4.z};
            float4 r[3][kRec];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int m = 0; m < kRec; ++m) r[k][m] = rec[kRec * (size_t)id[k] + m];
            Elem2 o;
            ElemParams qe = q;
            if (c.mu_e) qe.mu = __ldg(reinterpret_cast<const float*>(c.mu_e) + e);
            if (FF) element2d_ff(r, qe, o);
            else element2d(r, qe, o);
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
        if (threadIdx.x == 0) s_nb2[(kp + 1) & 1] = 0;   // the next patch's count
        // ---- owned vertices: forces and the acceleration in FP32, accumulations in float-float ----
        // Interior vertices finish here.  Boundary vertices queue their FP32 sums in shared
        // memory and finish in a second loop over consecutive threads, so that the float-float
        // boundary terms run on full warps instead of one or two lanes of many warps.
        const ParamF& pf = c.pf;
        const float rho_max = pf.rho_i_max;
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            // the vertex's own state first: these loads do not depend on the one-ring sums below
            const int kb = c.vt_ptr[v], ke = c.vt_ptr[v + 1];
            const ff4 f4 = ldg_ff4(c.fau, c.nv, v);
            const ff cCv = ld_ff(c.cC, c.nv, v);
            const float cCh = cCv.hi;
            const float rho = c.rho_w ? ld_rho(c.rho_w, v) : rho_max;
            const int rank = c.bnd_rank[v];
            const float4* eo = reinterpret_cast<const float4*>(c.ea[par]);
            const ff4 Vv = ldg_ff4(c.vel, c.nv, v);
            const float4 Av = a.vh_from_buf ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_acc(c.acc, v);
            const float4 eh = __ldg(eo + v), el = __ldg(eo + c.nv + v);
            float Q0 = 0, Q1 = 0, Q2 = 0, Q3 = 0, MMf = 0, Asf = 0;
            ff R0 = {0.0f, 0.0f}, R1 = {0.0f, 0.0f};   // compensated: the corner forces largely cancel
#pragma unroll 4
            for (int k = kb; k < ke; ++k) {
                const int code = c.vc_code[k];
                const int sl = code >> 2, cn = code & 3;
                R0 = ff_add_f(R0, smf[(2 * cn) * emax + sl]);
                R1 = ff_add_f(R1, smf[(2 * cn + 1) * emax + sl]);
                Q0 += smf[(6 + 4 * cn) * emax + sl];
                Q1 += smf[(7 + 4 * cn) * emax + sl];
                Q2 += smf[(8 + 4 * cn) * emax + sl];
                Q3 += smf[(9 + 4 * cn) * emax + sl];
                MMf += smf[18 * emax + sl];
                Asf += smf[19 * emax + sl];
            }
            const float Asum = Asf * (1.0f / 3.0f);
            // integrin force (UL:1241-1269) in FP32
            float fs[3];
            spring_force32(pf, f4.hx, f4.hy, f4.hz, f4.lx, f4.ly, f4.lz, fs);
            const float kfa = -cCh * Asum * rho;
            if (rank >= 0) {   // F = kfa fs - R in float-float, then the boundary terms
                ff G0 = net_force_ff(kfa, fs[0], R0), G1 = net_force_ff(kfa, fs[1], R1);
                const int slot = atomicAdd(&s_nbnd, 1);
                if (slot < kBndSlots) {
                    float* b = s_bnd + kBndRec * slot;
                    b[0] = __int_as_float(i); b[1] = G0.hi; b[2] = G0.lo; b[3] = G1.hi; b[4] = G1.lo;
                    b[5] = Q0; b[6] = Q1; b[7] = Q2; b[8] = Q3; b[9] = MMf;
                    continue;
                }
                boundary_force(c, s_bc, pt, rec, xp, v, rank, G0, G1);   // queue full: finish in place
                FusedIn nx;
                if (fuse) nx = {ldg_ff4(xp, c.nv, v), f4, cCv, ld_ff(c.cA, c.nv, v)};
                finish_vertex_core(c, a, par, v, G0, G1, true, Q0, Q1, Q2, Q3, MMf, Vv, Av, eh, el,
                                   fuse ? &nx : nullptr);
                continue;
            }
            // F = kfa fs - R with the product exact (TwoProduct) and one rounding at the end
            const float F0 = net_force(kfa, fs[0], R0), F1 = net_force(kfa, fs[1], R1);
            FusedIn nx;
            if (fuse) nx = {ldg_ff4(xp, c.nv, v), f4, cCv, ld_ff(c.cA, c.nv, v)};
            finish_vertex_core(c, a, par, v, {F0, 0.0f}, {F1, 0.0f}, false, Q0, Q1, Q2, Q3, MMf, Vv, Av, eh, el,
                               fuse ? &nx : nullptr);
        }
        __syncthreads();
        const int nq = min(s_nbnd, kBndSlots);
        for (int j = threadIdx.x; j < nq; j += blockDim.x) {
            const float* b = s_bnd + kBndRec * j;
            const int v = pt.x + __float_as_int(b[0]);
            ff F0 = {b[1], b[2]}, F1 = {b[3], b[4]};
            boundary_force(c, s_bc, pt, rec, xp, v, c.bnd_rank[v], F0, F1);
            finish_vertex(c, a, par, v, F0, F1, b[5], b[6], b[7], b[8], b[9], fuse);
        }
        // The next patch's element loop may start while boundary vertices finish: it writes
        // only the element slots, which nothing after the vertex loop's barrier reads.
        if (fuse) __syncthreads();
        if (threadIdx.x == 0) {
            // The ticket only counts the cell's patches, so that the last one advances the
            // parity, clock and AP counter, which the next launch reads; only the fused form's
            // last patch reads what the others stored (their predictions) and needs the
            // release fence before its ticket.
            if (fuse) __threadfence();
            const unsigned int done = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 1), 1u);
            const bool last = (int)done == c.np - 1;
            if (last) {
                c.ctl[1] = 0;
                c.ctl[0] = par ^ 1;
                c.clk[0] = c.clk[0] + a.dt_real;
                c.ap[0] = ap_call + 1ull;
                count_step(c);
            }
            s_last = last;
        }
        if (fuse) {
            // the cell's last patch: area and step constants of the next step from every patch's
            // predictions (the shared element slots are free until the next patch)
            __syncthreads();
            if (s_last) {
                __threadfence();
                area_shoelace(c, c.pos[par], a.va.dtd, reinterpret_cast<double*>(smf));
            }
        }
    }
}

// Mixed-form vertex phase, one block per work item (c.vb consecutive vertices of
// one cell): predict, bond kinetics with FP32 rates and float-float accumulation,
// and the FP32 element records.  No FP64 arithmetic outside the exchange
// conversions and the cell area.  The area and the step constants come from the
// cell's block 0, before its vertices, on predictions it forms itself (area_predicted)
// or on positions already in place, so no block waits for another; only positions this
// launch imports are summed after every block stored them (ticket, finish_area_boundary).
// MINB: the least blocks of 256 threads per SM the register allocation must allow (4, 5,
// 6, 8: 64, 48, 40, 32 registers, spilling more as the cap falls); the autotuner picks.
template <int MINB>
__global__ void __launch_bounds__(kK1Threads, MINB) k_vertex_phase_mixed(const CellDev* __restrict__ cells,
                                                                    const WorkItem* __restrict__ work,
                                                                    const VertexArgs va) {
    const WorkItem it = work[blockIdx.x];
    const CellDev& c = cells[it.cell];
    if (cell_done(c)) return;   // block-uniform: a serving cell that ran its steps
    const int v = it.idx * c.vb + threadIdx.x;
    const int par = c.ctl[0];
    const bool area = !(va.flags & VM_NOAREA), ticket = area && (va.flags & VM_IMPORT);
    if (area && !ticket && it.idx == 0) {   // block-uniform
        __shared__ double s_w[3 * kK1Threads / 32];
        if (va.flags & VM_PREDICT) area_predicted(c, par, va, s_w);
        else area_shoelace(c, c.pos[par ^ 1], va.dtd, s_w);
    }
    VertexArgs vb = va;
    if (!ticket) vb.flags |= VM_NOAREA;   // no block reads this launch's stored positions
    // The exchange coordinates of the block's vertices, 3 binary64 each, pass through shared
    // memory so that the exchange staging array is read and written in consecutive runs
    // (a warp's access covers 256 contiguous bytes instead of 32 doubles 24 bytes apart).
    __shared__ double s_x[3 * kK1Threads];
    const int v0 = it.idx * c.vb, nd = 3 * max(0, min(c.vb, c.nv - v0));
    if (va.flags & VM_IMPORT) {   // block-uniform
        const double* src = va.stage_in + 3 * ((size_t)c.hoff + v0);
        for (int k = threadIdx.x; k < nd; k += blockDim.x) s_x[k] = src[k];
        __syncthreads();
    }
    if (v < c.nv) vertex_mixed_body(c, v, par, vb, s_x + 3 * threadIdx.x);
    if (va.flags & VM_EXPORT) {
        __syncthreads();
        double* dst = va.stage_out + 3 * ((size_t)c.hoff + v0);
        for (int k = threadIdx.x; k < nd; k += blockDim.x) dst[k] = s_x[k];
    }
    if (ticket) finish_area_boundary(c, c.pos[par ^ 1], va.dtd);
}

void launch_vertex_mixed(const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
                         int threads, cudaStream_t st, const double* stage_in, double* stage_out, int kind) {
    if (nwork <= 0) return;
    (void)grid;   // one block per work item
    VertexArgs va;
    va.dt = ff_from_d(dt);
    va.hdt = ff_from_d(dt / 2.0);
    va.dtd = dt;
    va.dtf = (float)dt;
    va.flags = flags;
    va.stage_in = stage_in;
    va.stage_out = stage_out;
    switch (kind) {
        case 1: k_vertex_phase_mixed<4><<<nwork, threads, 0, st>>>(cells, work, va); break;
        case 2: k_vertex_phase_mixed<6><<<nwork, threads, 0, st>>>(cells, work, va); break;
        case 3: k_vertex_phase_mixed<8><<<nwork, threads, 0, st>>>(cells, work, va); break;
        default: k_vertex_phase_mixed<5><<<nwork, threads, 0, st>>>(cells, work, va); break;
    }
}

// ===========================================================================
// Staged patch phase: a persistent CTA walks its patches and, one patch ahead,
// copies everything the patch reads into shared memory with bulk asynchronous
// copies completing on an mbarrier (two stages).  Element records of the owned
// range and the owned vertices' state are contiguous ranges (one bulk copy each);
// the halo records are scattered 48-B rows, copied with 16-B cp.async by the lanes
// of warp 0, whose completion arrives on the same barrier.
// The arithmetic is that of k_patch_phase_mixed.
// ===========================================================================
struct StageLayout {
    uint32_t stage_bytes;   // bytes per stage
    uint32_t o_hdr, o_loc, o_rec, o_vt, o_code, o_fau, o_cc, o_rho, o_vhi, o_vlo, o_acc, o_eahi, o_ealo, o_rank;
    uint32_t smf_off;       // element outputs, after the two stages
    int32_t cap_ne, cap_nvp, cap_nh, cap_nc;
};

struct StageHdr {
    int32_t cell, idx, par, bad;
    int4 pt;                // (v0, nvp, e0, ne)
    int4 px;                // (h0, nh, c0, nc)
    int32_t vt_off, code_base, s_off, has_rho;
    unsigned long long ap_call;
    ElemParams q;
    BndConst bc;
};

constexpr long long kWaitLimit = 4000000000ll;   // SM clocks (about 2 s) before a stage wait gives up

__device__ __forceinline__ void stage_issue(const MixedArgs& a, const StageLayout& L, unsigned char* sm, int w, int s,
                                            uint64_t* bar) {
    unsigned char* st = sm + (size_t)s * L.stage_bytes;
    StageHdr* h = reinterpret_cast<StageHdr*>(st + L.o_hdr);
    const int lane = threadIdx.x & 31;
    fence_proxy_async_smem();   // the stage was last read through the generic proxy
    if (lane == 0) {
        const WorkItem it = a.work[w];
        const CellDev& c = a.cells[it.cell];
        const int4 pt = c.patch[it.idx];
        const int4 px = c.patch_x[it.idx];
        const int n = c.nv;
        const int par = c.ctl[0];
        h->cell = it.cell;
        h->idx = it.idx;
        h->par = par;
        h->pt = pt;
        h->px = px;
        h->ap_call = c.ap[0];
        h->has_rho = c.rho_w != nullptr;
        {   // element constants of this cell and step
            const wcfe_params& p = c.prm;
            const double t = isnan(a.t_override) ? c.clk[0] : a.t_override;
            const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
            h->q.mu = (float)p.mu;
            h->q.thick = (float)p.thick;
            h->q.grow = (float)(p.thetag_dot * a.dt_real);
            h->q.s_iso = (float)(p.kappa * t_act);
            h->q.t_an = (float)((1.0 - 2.0 * p.kappa) * t_act);
            h->q.cx = (float)c.area4[1];
            h->q.cy = (float)c.area4[2];
            h->bc = make_bnd_const(c, a, h->ap_call);
        }
        const bool bad = pt.w > L.cap_ne || pt.y > L.cap_nvp || px.y > L.cap_nh || px.w > L.cap_nc;
        const bool skip = cell_done(c);   // a serving cell that ran its steps: no copies, no work
        h->bad = skip ? 2 : (bad ? 1 : 0);
        if (bad || skip) {
            if (!skip) atomicOr(c.status, 4u);
            mbar_arrive_expect_tx(bar + s, 0);
        } else {
            const int v0 = pt.x, nvp = pt.y;
            const int a4 = v0 & ~3;                  // 16-B aligned start of the 4-byte per-vertex arrays
            const int cb = px.z & ~7;                // 16-B aligned start of the 2-byte codes
            h->vt_off = v0 - a4;
            h->s_off = v0 - a4;
            h->code_base = cb;
            const uint32_t b_loc = align16(8u * (uint32_t)pt.w);
            const uint32_t b_rec = 48u * (uint32_t)nvp;
            const uint32_t b_vt = align16(4u * (uint32_t)(v0 + nvp + 1 - a4));
            const uint32_t b_code = align16(2u * (uint32_t)(px.z + px.w - cb));
            const uint32_t b_v16 = 16u * (uint32_t)nvp;
            const uint32_t b_s4 = align16(4u * (uint32_t)(v0 + nvp - a4));
            const uint32_t total = b_loc + b_rec + b_vt + b_code + 6u * b_v16 + (h->has_rho ? 3u : 2u) * b_s4;
            mbar_arrive_expect_tx(bar + s, total);
            const float4* fau = reinterpret_cast<const float4*>(c.fau);
            const float4* vel = reinterpret_cast<const float4*>(c.vel);
            const float4* ea = reinterpret_cast<const float4*>(c.ea[par]);
            bulk_g2s(st + L.o_loc, c.patch_loc + 4 * (size_t)pt.z, b_loc, bar + s);
            if (b_rec) bulk_g2s(st + L.o_rec, c.rec[par] + 3 * (size_t)v0, b_rec, bar + s);
            bulk_g2s(st + L.o_vt, c.vt_ptr + a4, b_vt, bar + s);
            if (b_code) bulk_g2s(st + L.o_code, c.vc_code + cb, b_code, bar + s);
            if (b_v16) {
                bulk_g2s(st + L.o_fau, fau + v0, b_v16, bar + s);
                bulk_g2s(st + L.o_vhi, vel + v0, b_v16, bar + s);
                bulk_g2s(st + L.o_vlo, vel + n + v0, b_v16, bar + s);
                bulk_g2s(st + L.o_acc, reinterpret_cast<const float4*>(c.acc) + v0, b_v16, bar + s);
                bulk_g2s(st + L.o_eahi, ea + v0, b_v16, bar + s);
                bulk_g2s(st + L.o_ealo, ea + n + v0, b_v16, bar + s);
            }
            if (b_s4) {
                bulk_g2s(st + L.o_cc, reinterpret_cast<const float*>(c.cC) + a4, b_s4, bar + s);
                bulk_g2s(st + L.o_rank, c.bnd_rank + a4, b_s4, bar + s);
                if (h->has_rho) bulk_g2s(st + L.o_rho, reinterpret_cast<const float*>(c.rho_w) + a4, b_s4, bar + s);
            }
        }
    }
    __syncwarp();
    // halo records: scattered 48-B rows, three 16-B cp.async each, spread over the lanes; every
    // lane then arrives on the stage barrier when its copies have landed (32 of its 33 arrivals)
    if (!h->bad) {
        const CellDev& c = a.cells[h->cell];
        const int nvp = h->pt.y, h0 = h->px.x, nh = h->px.y;
        float4* rec_s = reinterpret_cast<float4*>(st + L.o_rec) + kRec * (size_t)nvp;
        for (int k = lane; k < nh; k += 32) {
            const float4* src = c.rec[h->par] + kRec * (size_t)c.patch_halo[h0 + k];
#pragma unroll
            for (int m = 0; m < kRec; ++m) cp_async16(rec_s + kRec * (size_t)k + m, src + m);
        }
    }
    cp_async_mbar_arrive(bar + s);
}

constexpr int kConsumers = 256;   // 8 consumer warps; warp 8 produces (stage_issue)

__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Warp-specialised: warp 8 walks the CTA's patches and fills stage k & 1 for patch k as
// soon as the consumers have released it (barrier empty[s]); warps 0-7 wait for the
// stage (barrier full[s]), compute, and release it.
__global__ void __launch_bounds__(kConsumers + 32) k_patch_mixed_staged(MixedArgs a, StageLayout L) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[2], empty[2];
    __shared__ int s_nbnd, s_ok;
    __shared__ float s_bnd[kBndRec * kBndSlots];
    float* smf = reinterpret_cast<float*>(sm + L.smf_off);
    const int emax = L.cap_ne;   // field stride of the element outputs
    if (threadIdx.x == 0) {
        // full: the producer lane 0's expect-tx arrival + one cp.async arrival per producer lane
        mbar_init(full, 33);
        mbar_init(full + 1, 33);
        mbar_init(empty, 1);
        mbar_init(empty + 1, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x >= kConsumers) {   // ---- producer warp ----
        int k = 0;
        for (int w = blockIdx.x; w < a.nwork; w += gridDim.x, ++k) {
            const int s = k & 1;
            if (k >= 2) {   // wait until the consumers released this stage (patch k - 2)
                int ok = 1;
                if ((threadIdx.x & 31) == 0)
                    ok = mbar_wait_bounded(empty + s, (uint32_t)((k >> 1) - 1) & 1u, kWaitLimit) ? 1 : 0;
                if (!__shfl_sync(0xffffffffu, ok, 0)) return;   // the consumers stopped (and flagged it)
            }
            stage_issue(a, L, sm, w, s, full);
        }
        return;
    }
    // ---- consumer warps ----
    int k = 0;
    for (int w = blockIdx.x; w < a.nwork; w += gridDim.x, ++k) {
        const int s = k & 1;
        if (threadIdx.x == 0) {
            s_nbnd = 0;
            s_ok = mbar_wait_bounded(full + s, (uint32_t)(k >> 1) & 1u, kWaitLimit) ? 1 : 0;
        }
        consumer_sync();
        if (!s_ok) {
            // a copy did not complete: flag the cell, wait (bounded) once more for the stage's copies, leave
            if (threadIdx.x == 0) {
                atomicOr(a.cells[a.work[w].cell].status, 8u);
                mbar_wait_bounded(full + s, (uint32_t)(k >> 1) & 1u, kWaitLimit);
            }
            return;
        }
        const unsigned char* st = sm + (size_t)s * L.stage_bytes;
        const StageHdr* h = reinterpret_cast<const StageHdr*>(st + L.o_hdr);
        if (h->bad) {   // capacity exceeded (status already flagged), or a serving cell that is done
            consumer_sync();
            if (threadIdx.x == 0) mbar_arrive(empty + s);
            continue;
        }
        const CellDev& c = a.cells[h->cell];
        const int4 pt = h->pt;
        const int par = h->par;
        const ElemParams q = h->q;
        const float4* rec_s = reinterpret_cast<const float4*>(st + L.o_rec);
        const uint2* loc_s = reinterpret_cast<const uint2*>(st + L.o_loc);
        // ---- elements of the patch -> shared memory ----
        for (int j = threadIdx.x; j < pt.w; j += kConsumers) {
            const uint2 l2 = loc_s[j];
            const int id[3] = {(int)(l2.x & 0xffffu), (int)(l2.x >> 16), (int)(l2.y & 0xffffu)};
            float4 r[3][kRec];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                for (int m = 0; m < kRec; ++m) r[kk][m] = rec_s[kRec * id[kk] + m];
            Elem2 o;
            ElemParams qe = q;
            if (c.mu_e) qe.mu = __ldg(reinterpret_cast<const float*>(c.mu_e) + c.patch_elems[pt.z + j]);
            element2d(r, qe, o);
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                smf[(2 * kk + 0) * emax + j] = o.re[kk][0];
                smf[(2 * kk + 1) * emax + j] = o.re[kk][1];
#pragma unroll
                for (int m = 0; m < 4; ++m) smf[(6 + 4 * kk + m) * emax + j] = o.rea[kk][m];
            }
            smf[18 * emax + j] = o.mm;
            smf[19 * emax + j] = o.acur;
        }
        consumer_sync();
        // ---- owned vertices (as k_patch_phase_mixed, state from the stage) ----
        const int32_t* vt_s = reinterpret_cast<const int32_t*>(st + L.o_vt) + h->vt_off;
        const uint16_t* code_s = reinterpret_cast<const uint16_t*>(st + L.o_code) - h->code_base;
        const float4* fau_s = reinterpret_cast<const float4*>(st + L.o_fau);
        const float* cc_s = reinterpret_cast<const float*>(st + L.o_cc) + h->s_off;
        const float* rho_s = reinterpret_cast<const float*>(st + L.o_rho) + h->s_off;
        const int32_t* rank_s = reinterpret_cast<const int32_t*>(st + L.o_rank) + h->s_off;
        const float4* vhi_s = reinterpret_cast<const float4*>(st + L.o_vhi);
        const float4* vlo_s = reinterpret_cast<const float4*>(st + L.o_vlo);
        const float4* acc_s = reinterpret_cast<const float4*>(st + L.o_acc);
        const float4* eahi_s = reinterpret_cast<const float4*>(st + L.o_eahi);
        const float4* ealo_s = reinterpret_cast<const float4*>(st + L.o_ealo);
        const ParamF& pf = c.pf;
        const float rho_max = pf.rho_i_max;
        const bool has_rho = h->has_rho;
        const double4* __restrict__ xp = c.pos[par ^ 1];
        for (int i = threadIdx.x; i < pt.y; i += kConsumers) {
            const int v = pt.x + i;
            float Q0 = 0, Q1 = 0, Q2 = 0, Q3 = 0, MMf = 0, Asf = 0;
            ff R0 = {0.0f, 0.0f}, R1 = {0.0f, 0.0f};   // compensated: the corner forces largely cancel
            for (int kk = vt_s[i]; kk < vt_s[i + 1]; ++kk) {
                const int code = code_s[kk];
                const int sl = code >> 2, cn = code & 3;
                R0 = ff_add_f(R0, smf[(2 * cn) * emax + sl]);
                R1 = ff_add_f(R1, smf[(2 * cn + 1) * emax + sl]);
                Q0 += smf[(6 + 4 * cn) * emax + sl];
                Q1 += smf[(7 + 4 * cn) * emax + sl];
                Q2 += smf[(8 + 4 * cn) * emax + sl];
                Q3 += smf[(9 + 4 * cn) * emax + sl];
                MMf += smf[18 * emax + sl];
                Asf += smf[19 * emax + sl];
            }
            const float Asum = Asf * (1.0f / 3.0f);
            const float4 f4 = fau_s[i];   // the high words; the MD branch also reads the low words
            const float4 f4l = pf.law == PF_MD ? __ldg(reinterpret_cast<const float4*>(c.fau) + c.nv + pt.x + i)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
            float fs[3];
            spring_force32(pf, f4.x, f4.y, f4.z, f4l.x, f4l.y, f4l.z, fs);
            const float rho = has_rho ? rho_s[i] : rho_max;
            const float kfa = -cc_s[i] * Asum * rho;
            const int rank = rank_s[i];
            const float4 vh = vhi_s[i], vl = vlo_s[i];
            if (rank >= 0) {   // F = kfa fs - R in float-float, then the boundary terms
                ff G0 = net_force_ff(kfa, fs[0], R0), G1 = net_force_ff(kfa, fs[1], R1);
                const int slot = atomicAdd(&s_nbnd, 1);
                if (slot < kBndSlots) {
                    float* b = s_bnd + kBndRec * slot;
                    b[0] = __int_as_float(i); b[1] = G0.hi; b[2] = G0.lo; b[3] = G1.hi; b[4] = G1.lo;
                    b[5] = Q0; b[6] = Q1; b[7] = Q2; b[8] = Q3; b[9] = MMf;
                    continue;
                }
                boundary_force(c, h->bc, pt, c.rec[par], xp, v, rank, G0, G1);   // queue full: finish in place
                finish_vertex_core(c, a, par, v, G0, G1, true, Q0, Q1, Q2, Q3, MMf,
                                   {vh.x, vh.y, vh.z, vh.w, vl.x, vl.y, vl.z, vl.w}, acc_s[i], eahi_s[i], ealo_s[i]);
                continue;
            }
            // F = kfa fs - R with the product exact (TwoProduct) and one rounding at the end
            const float F0 = net_force(kfa, fs[0], R0), F1 = net_force(kfa, fs[1], R1);
            finish_vertex_core(c, a, par, v, {F0, 0.0f}, {F1, 0.0f}, false, Q0, Q1, Q2, Q3, MMf,
                               {vh.x, vh.y, vh.z, vh.w, vl.x, vl.y, vl.z, vl.w}, acc_s[i], eahi_s[i], ealo_s[i]);
        }
        consumer_sync();
        const int nq = min(s_nbnd, kBndSlots);
        for (int j = threadIdx.x; j < nq; j += kConsumers) {
            const float* b = s_bnd + kBndRec * j;
            const int i = __float_as_int(b[0]);
            const int v = pt.x + i;
            ff F0 = {b[1], b[2]}, F1 = {b[3], b[4]};
            boundary_force(c, h->bc, pt, c.rec[par], xp, v, rank_s[i], F0, F1);
            const float4 vh = vhi_s[i], vl = vlo_s[i];
            finish_vertex_core(c, a, par, v, F0, F1, true, b[5], b[6], b[7], b[8], b[9],
                               {vh.x, vh.y, vh.z, vh.w, vl.x, vl.y, vl.z, vl.w}, acc_s[i], eahi_s[i], ealo_s[i]);
        }
        consumer_sync();
        if (threadIdx.x == 0) {
            const unsigned long long ap_call = h->ap_call;
            mbar_arrive(empty + s);   // stage s is free (everything it holds has been read)
            __threadfence();
            const unsigned int done = atomicAdd(reinterpret_cast<unsigned int*>(c.ctl + 1), 1u);
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

// Shared-memory plan of the staged kernel for the given capacities; false if it
// does not fit in max_smem bytes.
bool staged_layout(int cap_ne, int cap_nvp, int cap_nh, int cap_nc, size_t max_smem, StageLayout* L,
                   size_t* total) {
    cap_ne = (cap_ne + 1) & ~1;
    uint32_t o = 0;
    auto put = [&](uint32_t bytes) {
        const uint32_t at = o;
        o = (o + bytes + 127u) & ~127u;
        return at;
    };
    L->o_hdr = put((uint32_t)sizeof(StageHdr));
    L->o_loc = put(8u * cap_ne + 16u);
    L->o_rec = put(48u * (uint32_t)(cap_nvp + cap_nh));
    L->o_vt = put(4u * (uint32_t)(cap_nvp + 8));
    L->o_code = put(2u * (uint32_t)(cap_nc + 16));
    L->o_fau = put(16u * cap_nvp);
    L->o_vhi = put(16u * cap_nvp);
    L->o_vlo = put(16u * cap_nvp);
    L->o_acc = put(16u * cap_nvp);
    L->o_eahi = put(16u * cap_nvp);
    L->o_ealo = put(16u * cap_nvp);
    L->o_cc = put(4u * (uint32_t)(cap_nvp + 8));
    L->o_rho = put(4u * (uint32_t)(cap_nvp + 8));
    L->o_rank = put(4u * (uint32_t)(cap_nvp + 8));
    L->stage_bytes = o;
    L->smf_off = 2u * o;
    L->cap_ne = cap_ne;
    L->cap_nvp = cap_nvp;
    L->cap_nh = cap_nh;
    L->cap_nc = cap_nc;
    *total = (size_t)L->smf_off + sizeof(float) * (size_t)cap_ne * kSlot32;
    return *total <= max_smem;
}

static size_t g_staged_optin = 0;   // dynamic shared memory the staged kernel may use

cudaError_t configure_staged(size_t max_smem) {
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, (const void*)k_patch_mixed_staged);
    if (e != cudaSuccess) return e;
    size_t dyn = max_smem > at.sharedSizeBytes + 1024 ? max_smem - at.sharedSizeBytes - 1024 : 0;
    g_staged_optin = dyn;
    return cudaFuncSetAttribute((const void*)k_patch_mixed_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)dyn);
}

// Launch the staged kernel if its plan fits; returns false (nothing launched) otherwise.
bool launch_patch_staged(const CellDev* cells, const WorkItem* work, int nwork, int cap_ne, int cap_nvp, int cap_nh,
                         int cap_nc, double dt, double dt_real, double ap_thresh, double t_override, int vh_from_buf,
                         int num_sms, cudaStream_t st) {
    if (nwork <= 0) return true;
    StageLayout L;
    size_t smem = 0;
    if (!staged_layout(cap_ne, cap_nvp, cap_nh, cap_nc, g_staged_optin, &L, &smem)) return false;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_patch_mixed_staged, kConsumers + 32, smem) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    MixedArgs a;
    a.cells = cells;
    a.work = work;
    a.nwork = nwork;
    a.emax = L.cap_ne;
    a.dt_real = dt_real;
    a.hdt = ff_from_d(dt / 2.0);
    a.cdt = ff_from_d(dt_real - dt / 2.0);
    a.dtr = ff_from_d(dt_real);
    a.half = dt_real > dt / 2.0;
    a.ap_thresh = ap_thresh;
    a.t_override = t_override;
    a.vh_from_buf = vh_from_buf;
    const int grid = std::min(nwork, per_sm * num_sms);
    k_patch_mixed_staged<<<grid, kConsumers + 32, smem, st>>>(a, L);
    return true;
}

size_t mixed_smem_bytes(int emax) { return sizeof(float) * (size_t)emax * kSlot32; }

namespace {
// kinds 1-4: the plain kernel for 5-8 CTAs per SM; 5: the fused form (5 CTAs per SM)
const void* mixed_kernel(int kind) {
    switch (kind) {
        case 2: return (const void*)k_patch_phase_mixed<6, false>;
        case 3: return (const void*)k_patch_phase_mixed<7, false>;
        case 4: return (const void*)k_patch_phase_mixed<8, false>;
        case 5: return (const void*)k_patch_phase_mixed<5, true>;
        case 6: return (const void*)k_patch_phase_mixed<2, false, 0, true>;
        default: return (const void*)k_patch_phase_mixed<5, false>;
    }
}
}  // namespace

cudaError_t configure_mixed(size_t max_smem) {
    {   // the constant-stride instantiation of kind 1 (emax 512)
        const void* f = (const void*)k_patch_phase_mixed<5, false, 512>;
        cudaFuncAttributes at;
        cudaError_t e = cudaFuncGetAttributes(&at, f);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(max_smem > at.sharedSizeBytes ? max_smem - at.sharedSizeBytes : 0));
        if (e != cudaSuccess) return e;
    }
    for (int kind = 1; kind <= 6; ++kind) {
        cudaFuncAttributes at;
        cudaError_t e = cudaFuncGetAttributes(&at, mixed_kernel(kind));
        if (e != cudaSuccess) return e;
        size_t dyn = max_smem > at.sharedSizeBytes ? max_smem - at.sharedSizeBytes : 0;
        e = cudaFuncSetAttribute(mixed_kernel(kind), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    return configure_staged(max_smem);
}

// resident CTAs per SM of the plain kernel variant `kind` (1-4, see k_patch_phase_mixed; 5 fused;
// 6 the float-float element)
int mixed_occupancy(int threads, size_t smem, int kind) { return occupancy_cached(mixed_kernel(kind), threads, smem); }
int mixed_occupancy(int threads, size_t smem) { return mixed_occupancy(threads, smem, 1); }

void launch_patch_mixed(const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt, double dt_real,
                        double ap_thresh, double t_override, int vh_from_buf, int threads, int grid, cudaStream_t st,
                        int kind, int fused) {
    if (nwork <= 0) return;
    MixedArgs a;
    a.va.dt = ff_from_d(dt);
    a.va.hdt = ff_from_d(dt / 2.0);
    a.va.dtd = dt;
    a.va.dtf = (float)dt;
    a.va.flags = VM_PREDICT | VM_UPDATE_FA;
    a.va.stage_in = nullptr;
    a.va.stage_out = nullptr;
    a.cells = cells;
    a.work = work;
    a.nwork = nwork;
    a.emax = emax;
    a.dt_real = dt_real;
    a.hdt = ff_from_d(dt / 2.0);
    a.cdt = ff_from_d(dt_real - dt / 2.0);
    a.dtr = ff_from_d(dt_real);
    a.half = dt_real > dt / 2.0;
    a.ap_thresh = ap_thresh;
    a.t_override = t_override;
    a.vh_from_buf = vh_from_buf;
    const size_t smem = mixed_smem_bytes(emax);
    if (fused) {   // one fused instantiation (5 CTAs per SM) serves every plain kind
        k_patch_phase_mixed<5, true><<<grid, threads, smem, st>>>(a, cells, work);
        return;
    }
    switch (kind) {
        case 2: k_patch_phase_mixed<6, false><<<grid, threads, smem, st>>>(a, cells, work); break;
        case 3: k_patch_phase_mixed<7, false><<<grid, threads, smem, st>>>(a, cells, work); break;
        case 4: k_patch_phase_mixed<8, false><<<grid, threads, smem, st>>>(a, cells, work); break;
        case 6: k_patch_phase_mixed<2, false, 0, true><<<grid, threads, smem, st>>>(a, cells, work); break;
        default:
            if (emax == 512) k_patch_phase_mixed<5, false, 512><<<grid, threads, smem, st>>>(a, cells, work);
            else k_patch_phase_mixed<5, false><<<grid, threads, smem, st>>>(a, cells, work);
            break;
    }
}
void launch_patch_mixed(const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt, double dt_real,
                        double ap_thresh, double t_override, int vh_from_buf, int threads, int grid, cudaStream_t st) {
    launch_patch_mixed(cells, work, nwork, emax, dt, dt_real, ap_thresh, t_override, vh_from_buf, threads, grid, st, 1, 0);
}

}  // namespace wcfe
