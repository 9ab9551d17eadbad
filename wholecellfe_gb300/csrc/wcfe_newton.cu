// wcfe_newton.cu — implicit (Newton) step of the membrane on FP64 engines.
//
// There is no counterpart in the reference, which integrates explicitly
// (UL:889).  The step is backward Euler of the same equations of motion the
// explicit step integrates (UL:592-628), with the membrane implicit and the
// adhesion and boundary forces evaluated at the predicted positions:
//
//   G(x) = m (x - X) / dt^2 - m V / dt + (drag + damp m)(x - X) / dt - F_ext + Res(X, x, ea) = 0
//   J(x) = diag(m / dt^2 + (drag + damp m) / dt) + dRes/dx          (in-plane, 2N x 2N)
//
// with m = MM rho the lumped mass, F_ext = F_FA + F_AP + F_bend + F_area at the
// predicted positions and Res the FP64 membrane residual (calculateRes,
// UL:632-707).  Per Newton iteration: the FP64 residual G, the FP32 element
// tangents (forward-mode derivatives of the planar increment-form element, six
// directions at once), a dense FP32 J assembled row by row in one-ring order
// (deterministic), its LU factorisation with the trailing updates on the tensor
// cores in TF32, and the solve J d = -G refined in FP64 against the sparse
// element-by-element J until the correction's residual is 1e-10 of |G|.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "wcfe_common.cuh"

namespace wcfe {

// ===========================================================================
// forward-mode derivatives: value + ND directional derivatives
// ===========================================================================
template <int ND>
struct Dual {
    float v;
    float d[ND];
};
template <int ND>
__device__ __forceinline__ Dual<ND> dconst(float a) {
    Dual<ND> r;
    r.v = a;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = 0.0f;
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator+(const Dual<ND>& a, const Dual<ND>& b) {
    Dual<ND> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator-(const Dual<ND>& a, const Dual<ND>& b) {
    Dual<ND> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator-(const Dual<ND>& a) {
    Dual<ND> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator*(const Dual<ND>& a, const Dual<ND>& b) {
    Dual<ND> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator*(const Dual<ND>& a, float b) {
    Dual<ND> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator*(float b, const Dual<ND>& a) { return a * b; }
template <int ND>
__device__ __forceinline__ Dual<ND> operator+(const Dual<ND>& a, float b) {
    Dual<ND> r = a;
    r.v += b;
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator+(float b, const Dual<ND>& a) { return a + b; }
template <int ND>
__device__ __forceinline__ Dual<ND> operator-(const Dual<ND>& a, float b) {
    Dual<ND> r = a;
    r.v -= b;
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> operator-(float b, const Dual<ND>& a) {
    Dual<ND> r;
    r.v = b - a.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> inv(const Dual<ND>& a) {   // 1 / a
    Dual<ND> r;
    r.v = 1.0f / a.v;
    const float s = -r.v * r.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * s;
    return r;
}
template <int ND>
__device__ __forceinline__ Dual<ND> rsqrt(const Dual<ND>& a) {   // a^-1/2
    Dual<ND> r;
    r.v = rsqrtf(a.v);
    const float s = -0.5f * r.v / a.v;
#pragma unroll
    for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * s;
    return r;
}
__device__ __forceinline__ float inv(float a) { return 1.0f / a; }
__device__ __forceinline__ float rsqrt(float a) { return rsqrtf(a); }

struct TanParams {   // per-cell constants of the planar element
    float mu, thick, grow, s_iso, t_an;
};

// In-plane element residual of the planar increment form (the re part of the mixed
// form's element; UL:710-928 restated with F = I + H):
//   G1, G2 reference edges; d1, d2 the edge increments of the displacement x - X;
//   e = strain (xx, yy, xy, zz) at the integration point; (ax, ay) the element
//   centroid minus the cell centroid (direction of the anisotropic active stress).
template <class T>
__device__ __forceinline__ void element_re_planar(float G1x, float G1y, float G2x, float G2y, const T& d1x,
                                                  const T& d1y, const T& d2x, const T& d2y, const float e[4],
                                                  const T& ax_in, const T& ay_in, const TanParams& q, T re[3][2]) {
    const float Gc = G1x * G2y - G1y * G2x;
    const float iG = 1.0f / Gc;
    const float b1x = G2y * iG, b1y = -G2x * iG;
    const float b2x = -G1y * iG, b2y = G1x * iG;
    const float b0x = -b1x - b2x, b0y = -b1y - b2y;
    const T H00 = d1x * b1x + d2x * b2x, H01 = d1x * b1y + d2x * b2y;
    const T H10 = d1y * b1x + d2y * b2x, H11 = d1y * b1y + d2y * b2y;
    const float exx = e[0], eyy = e[1], exy = e[2], ezz = e[3];
    const float m00 = 1.0f - 2.0f * exx, m11 = 1.0f - 2.0f * eyy, m01 = -2.0f * exy;
    const float dm1 = -2.0f * (exx + eyy) + 4.0f * (exx * eyy - exy * exy);
    const float idM = 1.0f / (1.0f + dm1);
    const float i00 = m11 * idM, i01 = -m01 * idM, i11 = m00 * idM;
    const float be00 = 2.0f * (exx * i00 + exy * i01), be01 = 2.0f * (exx * i01 + exy * i11);
    const float be11 = 2.0f * (exy * i01 + eyy * i11);
    const float de = dm1 - 2.0f * ezz * (1.0f + dm1);
    const T c00 = 2.0f * H00 + (H00 * H00 + H10 * H10);
    const T c11 = 2.0f * H11 + (H01 * H01 + H11 * H11);
    const T c01 = H01 + H10 + (H00 * H01 + H10 * H11);
    const T dC = (1.0f + c00) * (1.0f + c11) - c01 * c01;
    const T iC = inv(dC);
    const T ci00 = (1.0f + c11) * iC, ci01 = -c01 * iC, ci11 = (1.0f + c00) * iC;
    const T ga00 = -(c00 * ci00 + c01 * ci01), ga01 = -(c00 * ci01 + c01 * ci11);
    const T ga11 = -(c01 * ci01 + c11 * ci11);
    const T dth = (H00 + H11) + (H00 * H11 - H01 * H10);
    const float g = q.grow, thg = 1.0f + g, gg2 = 2.0f * g + g * g;
    const T one_dth = 1.0f + dth;
    const T eta = (gg2 + thg * thg * de - 2.0f * dth - dth * dth) * inv(one_dth * one_dth);
    const T c0 = -(gg2 + thg * thg * eta) * (1.0f / thg);
    const float ith = 1.0f / thg;
    const T tge = thg * (1.0f + eta);
    T S00 = q.mu * (c0 + be00 * ith - tge * ga00);
    T S01 = q.mu * (be01 * ith - tge * ga01);
    T S11 = q.mu * (c0 + be11 * ith - tge * ga11);
    if (q.t_an != 0.0f) {
        const T ia = rsqrt(ax_in * ax_in + ay_in * ay_in);
        const T ax = ax_in * ia, ay = ay_in * ia;
        S00 = S00 + q.t_an * (ax * ax);
        S01 = S01 + q.t_an * (ax * ay);
        S11 = S11 + q.t_an * (ay * ay);
    }
    const T T00 = q.s_iso * H00 + S00 + (H00 * S00 + H01 * S01);
    const T T01 = q.s_iso * H01 + S01 + (H00 * S01 + H01 * S11);
    const T T10 = q.s_iso * H10 + S01 + (H10 * S00 + H11 * S01);
    const T T11 = q.s_iso * H11 + S11 + (H10 * S01 + H11 * S11);
    const float wA = 0.5f * Gc * q.thick;
    re[0][0] = wA * (T00 * b0x + T01 * b0y); re[0][1] = wA * (T10 * b0x + T11 * b0y);
    re[1][0] = wA * (T00 * b1x + T01 * b1y); re[1][1] = wA * (T10 * b1x + T11 * b1y);
    re[2][0] = wA * (T00 * b2x + T01 * b2y); re[2][1] = wA * (T10 * b2x + T11 * b2y);
}

// element tangents and dense assembly, one CTA per patch of a cell (work list of
// the patch phase); elements computed once per patch into shared memory
constexpr int kTanThreads = 128;

__global__ void __launch_bounds__(kTanThreads) k_newton_tangent(const CellDev* __restrict__ cells,
                                                               const NewtonCell* __restrict__ nc,
                                                               const int* __restrict__ cell_slot,
                                                               const WorkItem* __restrict__ work, int nwork, int emax,
                                                               double dt, int dense) {
    extern __shared__ float ke_s[];   // [emax][36]
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const int slot = cell_slot[it.cell];
        if (slot < 0) continue;
        const NewtonCell& N = nc[slot];
        if (!N.active) continue;
        const CellDev& c = cells[it.cell];
        const wcfe_params& p = c.prm;
        const int4 pt = c.patch[it.idx];
        const int par = c.ctl[0];
        const double4* __restrict__ X = c.pos[par];
        const double4* __restrict__ xp = c.pos[par ^ 1];
        const double* __restrict__ ea = c.ea[par];
        const double t = c.clk[0];
        const double t_act = t < p.tact_t1 ? t * p.tact_rate : p.tact_max;
        TanParams q;
        q.mu = (float)p.mu;
        q.thick = (float)p.thick;
        q.grow = (float)(p.thetag_dot * dt);
        q.s_iso = (float)(p.kappa * t_act);
        q.t_an = (float)((1.0 - 2.0 * p.kappa) * t_act);
        const double cx = c.area4[1], cy = c.area4[2];
        for (int j = threadIdx.x; j < pt.w; j += blockDim.x) {
            const int e = c.patch_elems[pt.z + j];
            const int4 t4 = c.tri[e];
            const int id[3] = {t4.x, t4.y, t4.z};
            double Xd[3][2], ud[3][2];
            float ev[4] = {0, 0, 0, 0};
            double axd = 0, ayd = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double4 a = ld4(X + id[k]), b = ld4v(xp + id[k]);
                Xd[k][0] = a.x; Xd[k][1] = a.y;
                ud[k][0] = b.x - a.x; ud[k][1] = b.y - a.y;
                axd += b.x; ayd += b.y;
                const double* q6 = ea + 6 * (size_t)id[k];
                ev[0] += (float)q6[0]; ev[1] += (float)q6[1]; ev[2] += (float)q6[3]; ev[3] += (float)q6[2];
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) ev[m] *= (1.0f / 3.0f);
            // seeds: direction 2k + i is the displacement of corner k, component i
            Dual<6> u[3][2];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    u[k][i] = dconst<6>((float)ud[k][i]);
                    u[k][i].d[2 * k + i] = 1.0f;
                }
            const Dual<6> d1x = u[1][0] - u[0][0], d1y = u[1][1] - u[0][1];
            const Dual<6> d2x = u[2][0] - u[0][0], d2y = u[2][1] - u[0][1];
            Dual<6> ax = dconst<6>((float)(axd / 3.0 - cx)), ay = dconst<6>((float)(ayd / 3.0 - cy));
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                ax.d[2 * k] = 1.0f / 3.0f;
                ay.d[2 * k + 1] = 1.0f / 3.0f;
            }
            Dual<6> re[3][2];
            TanParams qe = q;
            if (c.mu_e) qe.mu = (float)c.mu_e[e];
            element_re_planar((float)(Xd[1][0] - Xd[0][0]), (float)(Xd[1][1] - Xd[0][1]), (float)(Xd[2][0] - Xd[0][0]),
                              (float)(Xd[2][1] - Xd[0][1]), d1x, d1y, d2x, d2y, ev, ax, ay, qe, re);
            float* o = ke_s + 36 * j;
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int l = 0; l < 6; ++l) o[(2 * k + i) * 6 + l] = re[k][i].d[l];
            float* og = N.Ke + 36 * (size_t)e;   // duplicates across patches carry the same values
#pragma unroll 4
            for (int l = 0; l < 36; ++l) og[l] = o[l];
        }
        __syncthreads();
        // rows 2v, 2v+1 of the owned vertices: diagonal, then the one-ring in mesh order
        const double idt = 1.0 / dt;
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            const double m = N.MM[v] * p.rho;
            const double dg = m * idt * idt + (p.drag + p.damp * m) * idt;
            N.diag[v] = dg;
            if (!dense) continue;   // element tangents and the diagonal only (the factors are reused)
            float* row0 = N.J + (size_t)(2 * v) * N.ld;
            float* row1 = row0 + N.ld;
            row0[2 * v] += (float)dg;
            row1[2 * v + 1] += (float)dg;
            for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                const int code = c.vc_code[k];
                const int sl = code >> 2, cv = code & 3;
                const int e = c.patch_elems[pt.z + sl];
                const int4 t4 = c.tri[e];
                const int id[3] = {t4.x, t4.y, t4.z};
                const float* o = ke_s + 36 * sl;
#pragma unroll
                for (int l = 0; l < 3; ++l) {
                    const int col = 2 * id[l];
                    row0[col] += o[(2 * cv) * 6 + 2 * l];
                    row0[col + 1] += o[(2 * cv) * 6 + 2 * l + 1];
                    row1[col] += o[(2 * cv + 1) * 6 + 2 * l];
                    row1[col + 1] += o[(2 * cv + 1) * 6 + 2 * l + 1];
                }
            }
        }
        __syncthreads();
    }
}

// Newton residual G (FP64) per owned vertex, and per cell |G|inf and the force scale
__global__ void k_newton_residual(const CellDev* __restrict__ cells, const NewtonCell* __restrict__ nc,
                                  const int* __restrict__ cell_of_slot, int nslots, double dt) {
    const int slot = blockIdx.y;
    if (slot >= nslots) return;
    const NewtonCell& N = nc[slot];
    if (!N.active) return;
    const CellDev& c = cells[cell_of_slot[slot]];
    const wcfe_params& p = c.prm;
    const double idt = 1.0 / dt;
    double gmax = 0.0, fscale = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N.n; v += gridDim.x * blockDim.x) {
        const double m = N.MM[v] * p.rho;
        const double4 Vv = ld4(c.vel + v);
        const double dx[2] = {N.d[2 * (size_t)v], N.d[2 * (size_t)v + 1]}, V[2] = {Vv.x, Vv.y};
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const double f = N.Fext[3 * (size_t)v + i], res = N.Res[3 * (size_t)v + i];
            const double inert = m * dx[i] * idt * idt, mom = m * V[i] * idt;
            const double g = inert - mom + (p.drag + p.damp * m) * dx[i] * idt - f + res;
            N.G[2 * (size_t)v + i] = g;
            gmax = fmax(gmax, fabs(g));
            // the scale of the terms G sums (its rounding floor is relative to the largest)
            fscale = fmax(fscale, fmax(fmax(fabs(f), fabs(res)), fmax(fabs(inert), fabs(mom))));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        gmax = fmax(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
        fscale = fmax(fscale, __shfl_xor_sync(0xffffffffu, fscale, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(reinterpret_cast<unsigned long long*>(N.norms + 0), (unsigned long long)__double_as_longlong(gmax));
        atomicMax(reinterpret_cast<unsigned long long*>(N.norms + 1), (unsigned long long)__double_as_longlong(fscale));
    }
}

// ===========================================================================
// Dense LU without pivoting (J is strongly diagonally dominant: the mass term
// m / dt^2 exceeds the membrane stiffness by orders of magnitude for explicit-size
// steps; a pivot that is not finite or not above 1e-30 of the diagonal's scale
// flags the cell).  Right-looking, 64-wide blocks; the trailing update
// A22 -= L21 U12 runs on the tensor cores (mma m16n8k8, TF32 in, FP32 accumulate).
// ===========================================================================
constexpr int kNb = 64;

// The diagonal block, padded to 64 x 64 with the identity, factored in shared memory
// by a 16 x 16 thread grid (no divisions or modulos in the inner loops).
__device__ __forceinline__ void load_block_padded(const NewtonCell& N, int k0, int kb, float (*A)[kNb + 1]) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int i = ty; i < kNb; i += 16)
        for (int j = tx; j < kNb; j += 16)
            A[i][j] = (i < kb && j < kb) ? N.J[(size_t)(k0 + i) * N.ld + k0 + j] : (i == j ? 1.0f : 0.0f);
}

__global__ void __launch_bounds__(256) k_lu_diag(NewtonCell* nc, int nslots, int k0) {
    NewtonCell& N = nc[blockIdx.x];
    const int m = 2 * N.n;
    if (blockIdx.x >= nslots || !N.active || k0 >= m) return;
    const int kb = min(kNb, m - k0);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    __shared__ float A[kNb][kNb + 1];
    load_block_padded(N, k0, kb, A);
    __syncthreads();
    for (int j = 0; j < kNb; ++j) {
        const float piv = A[j][j];
        if (threadIdx.x == 0 && j < kb && !(fabsf(piv) > 1e-30f)) N.norms[3] = 1.0;
        if (threadIdx.x > j && threadIdx.x < kNb) A[threadIdx.x][j] /= piv;
        __syncthreads();
        for (int i = j + 1 + ty; i < kNb; i += 16) {
            const float l = A[i][j];
            for (int k = j + 1 + tx; k < kNb; k += 16) A[i][k] -= l * A[j][k];
        }
        __syncthreads();
    }
    for (int i = ty; i < kb; i += 16)
        for (int j = tx; j < kb; j += 16) N.J[(size_t)(k0 + i) * N.ld + k0 + j] = A[i][j];
    // explicit inverses of the (identity-padded) unit-lower and upper factors, one column per
    // thread: L X = I forward, U Y = I backward.  Rolled loops: fully unrolled, the two
    // substitutions were about 8k instructions that each launch's four warps ran once, from
    // a cold instruction cache.  Both inverses share one array Z: column j of Linv below
    // the diagonal (its diagonal is 1, the rest 0) and column j of Uinv on and above it, so
    // each thread reads only entries of its own column that it wrote.  The zero terms the
    // substitutions skip contribute exact zeros.  Stored as Linv and Uinv^T (row-major), the
    // K-major operands of the tensor-core panels.
    __shared__ float Z[kNb][kNb + 1];
    float* Li = N.Dinv + (size_t)(k0 / kNb) * 2 * kNb * kNb;
    float* Ui = Li + kNb * kNb;
    if (threadIdx.x < kNb) {
        const int j = threadIdx.x;
        for (int i = j + 1; i < kNb; ++i) {
            float s = -A[i][j];
#pragma unroll 4
            for (int k = j + 1; k < i; ++k) s -= A[i][k] * Z[k][j];
            Z[i][j] = s;
        }
    } else if (threadIdx.x < 2 * kNb) {
        const int j = threadIdx.x - kNb;
        for (int i = j; i >= 0; --i) {
            float s = i == j ? 1.0f : 0.0f;
#pragma unroll 4
            for (int k = i + 1; k <= j; ++k) s -= A[i][k] * Z[k][j];
            Z[i][j] = s / A[i][i];
        }
    }
    __syncthreads();
    // coalesced stores: Li[r][c] = Linv[r][c]; Ui[r][c] = Uinv[c][r]
    for (int e = threadIdx.x; e < kNb * kNb; e += blockDim.x) {
        const int r = e / kNb, cc = e % kNb;
        Li[e] = r > cc ? Z[r][cc] : (r == cc ? 1.0f : 0.0f);
        Ui[e] = cc <= r ? Z[cc][r] : 0.0f;
    }
}

// U12 = L11^-1 A12 (block x: column chunks) and L21 = A21 U11^-1 (block x: row chunks
// after the column chunks), in place, with the explicit inverses of the diagonal block's
// factors: one column or one row per thread, held in registers, and 64 independent dot
// products (no serial substitution chain).  The U rows also go, transposed, to
// Ut[col][kbase + i] (the tensor-core update's K-major operand).
__global__ void __launch_bounds__(256, 1) k_lu_panels(NewtonCell* nc, int nslots, int k0, int nchunks, int kbase) {
    const int slot = blockIdx.y;
    if (slot >= nslots) return;
    NewtonCell& N = nc[slot];
    const int m = 2 * N.n;
    if (!N.active || k0 >= m) return;
    const int kb = min(kNb, m - k0);
    const int r0 = k0 + kb;
    if (r0 >= m) return;
    const int half = nchunks / 2;
    const bool cols = (int)blockIdx.x < half;
    __shared__ __align__(16) float D[kNb][kNb];   // Linv for the columns, Uinv for the rows
    {
        const float* src = N.Dinv + (size_t)(k0 / kNb) * 2 * kNb * kNb;
        if (cols) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            float4* dst = reinterpret_cast<float4*>(&D[0][0]);
            for (int i = threadIdx.x; i < kNb * kNb / 4; i += blockDim.x) dst[i] = s4[i];
        } else {   // Uinv from its stored transpose
            for (int i = threadIdx.x; i < kNb * kNb; i += blockDim.x) D[i & (kNb - 1)][i >> 6] = src[kNb * kNb + i];
        }
    }
    __syncthreads();
    // kb == 64 here: a partial diagonal block is the last one and has no panels
    float a[kNb];
    if (cols) {   // u = Linv a (Linv unit lower): u_i = a_i + sum_{j < i} Linv[i][j] a_j
        for (int col = r0 + blockIdx.x * blockDim.x + threadIdx.x; col < m; col += half * blockDim.x) {
#pragma unroll
            for (int i = 0; i < kNb; ++i) a[i] = N.J[(size_t)(k0 + i) * N.ld + col];
            float4* ut = N.Ut ? reinterpret_cast<float4*>(N.Ut + (size_t)col * N.utld + kbase) : nullptr;
#pragma unroll
            for (int ig = 0; ig < kNb / 4; ++ig) {
                float u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int i = 4 * ig + q;
                    const float4* d4 = reinterpret_cast<const float4*>(&D[i][0]);
                    float s = a[i];
#pragma unroll
                    for (int jg = 0; jg < (i + 3) / 4; ++jg) {   // Linv[i][j] = 0 for j >= i
                        const float4 d = d4[jg];
                        s += d.x * a[4 * jg] + (4 * jg + 1 < i ? d.y * a[4 * jg + 1] : 0.0f) +
                             (4 * jg + 2 < i ? d.z * a[4 * jg + 2] : 0.0f) + (4 * jg + 3 < i ? d.w * a[4 * jg + 3] : 0.0f);
                    }
                    u[q] = s;
                    N.J[(size_t)(k0 + i) * N.ld + col] = s;
                }
                if (ut) ut[ig] = make_float4(u[0], u[1], u[2], u[3]);
                asm volatile("" ::: "memory");   // keep the next group's loads from being hoisted (registers)
            }
        }
    } else {      // l = a Uinv (Uinv upper): l_j = sum_{i <= j} a_i Uinv[i][j]
        for (int row = r0 + (blockIdx.x - half) * blockDim.x + threadIdx.x; row < m; row += half * blockDim.x) {
            float4* ar = reinterpret_cast<float4*>(N.J + (size_t)row * N.ld + k0);
#pragma unroll
            for (int ig = 0; ig < kNb / 4; ++ig) {
                const float4 v = ar[ig];
                a[4 * ig] = v.x; a[4 * ig + 1] = v.y; a[4 * ig + 2] = v.z; a[4 * ig + 3] = v.w;
            }
#pragma unroll
            for (int jg = 0; jg < kNb / 4; ++jg) {
                float l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int i = 0; i < 4 * jg + 4; ++i) {   // Uinv[i][j] = 0 for i > j
                    const float4 d = *reinterpret_cast<const float4*>(&D[i][4 * jg]);
                    l[0] += i <= 4 * jg ? a[i] * d.x : 0.0f;
                    l[1] += i <= 4 * jg + 1 ? a[i] * d.y : 0.0f;
                    l[2] += i <= 4 * jg + 2 ? a[i] * d.z : 0.0f;
                    l[3] += a[i] * d.w;
                }
                ar[jg] = make_float4(l[0], l[1], l[2], l[3]);
                asm volatile("" ::: "memory");
            }
        }
    }
}

// At[c][k] = J[k0 + k][c] for the columns c >= k0 + 64 (the row panel A12, transposed
// through shared memory: coalesced reads and writes)
__global__ void __launch_bounds__(256) k_lu_transpose_a12(NewtonCell* nc, int nslots, int k0) {
    NewtonCell& N = nc[blockIdx.y];
    const int m = 2 * N.n;
    if (blockIdx.y >= nslots || !N.active || k0 + kNb >= m) return;
    const int c0 = k0 + kNb + blockIdx.x * kNb;
    if (c0 >= m) return;
    __shared__ float T[kNb][kNb + 1];
    const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;   // 64 x 4
    for (int k = ty; k < kNb; k += 4) {
        const int c = c0 + tx;
        T[k][tx] = c < m ? N.J[(size_t)(k0 + k) * N.ld + c] : 0.0f;
    }
    __syncthreads();
    for (int cc = ty; cc < kNb; cc += 4) {
        const int c = c0 + cc;
        if (c < m) N.At[(size_t)c * kNb + tx] = T[tx][cc];
    }
}

__device__ __forceinline__ uint32_t to_tf32(float f) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
    return r;
}

// A22 -= L21 U12 for one 64 x 128 tile of the trailing matrix; 8 warps as 2 x 4, each
// a 32 x 32 block of 2 x 4 m16n8 tiles; K = the block width (<= 64).
constexpr int kTileM = 64, kTileN = 128;
__global__ void __launch_bounds__(256) k_lu_update(NewtonCell* nc, int nslots, int k0) {
    const int slot = blockIdx.z;
    if (slot >= nslots) return;
    NewtonCell& N = nc[slot];
    const int m = 2 * N.n;
    if (!N.active || k0 >= m) return;
    const int kb = min(kNb, m - k0);
    const int r0 = k0 + kb;
    const int tm = r0 + blockIdx.y * kTileM, tn = r0 + blockIdx.x * kTileN;
    if (tm >= m || tn >= m) return;
    extern __shared__ float smu[];
    const int lda = kNb + 4, ldb = kTileN + 8;
    float* As = smu;                 // [64][kNb + 4]: L21 rows tm.., columns k0..
    float* Bs = smu + kTileM * lda;  // [kNb][128 + 8]: U12 rows k0.., columns tn..
    for (int idx = threadIdx.x; idx < kTileM * kNb; idx += blockDim.x) {
        const int i = idx >> 6, k = idx & (kNb - 1);
        const int row = tm + i;
        As[i * lda + k] = (row < m && k < kb) ? N.J[(size_t)row * N.ld + k0 + k] : 0.0f;
    }
    for (int idx = threadIdx.x; idx < kNb * kTileN; idx += blockDim.x) {
        const int k = idx >> 7, j = idx & (kTileN - 1);
        const int col = tn + j;
        Bs[k * ldb + j] = (col < m && k < kb) ? N.J[(size_t)(k0 + k) * N.ld + col] : 0.0f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 2) * 32, wn = (warp & 3) * 32;   // warp block origin in the tile
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            const int rA = tm + wm + mi * 16 + g, cA = tn + wn + ni * 8 + 2 * t;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = rA + 8 * h;
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int col = cA + q;
                    acc[mi][ni][2 * h + q] = (row < m && col < m) ? N.J[(size_t)row * N.ld + col] : 0.0f;
                }
            }
        }
#pragma unroll
    for (int ks = 0; ks < kNb; ks += 8) {
        uint32_t af[2][4], bf[4][2];
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
            const float* a = As + (wm + mi * 16) * lda + ks;
            // -L21: the product is subtracted
            af[mi][0] = to_tf32(-a[g * lda + t]);
            af[mi][1] = to_tf32(-a[(g + 8) * lda + t]);
            af[mi][2] = to_tf32(-a[g * lda + t + 4]);
            af[mi][3] = to_tf32(-a[(g + 8) * lda + t + 4]);
        }
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            const float* b = Bs + ks * ldb + wn + ni * 8;
            bf[ni][0] = to_tf32(b[t * ldb + g]);
            bf[ni][1] = to_tf32(b[(t + 4) * ldb + g]);
        }
#pragma unroll
        for (int mi = 0; mi < 2; ++mi)
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                float* d = acc[mi][ni];
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                    : "r"(af[mi][0]), "r"(af[mi][1]), "r"(af[mi][2]), "r"(af[mi][3]), "r"(bf[ni][0]), "r"(bf[ni][1]));
            }
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) {
            const int rA = tm + wm + mi * 16 + g, cA = tn + wn + ni * 8 + 2 * t;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = rA + 8 * h;
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int col = cA + q;
                    if (row < m && col < m) N.J[(size_t)row * N.ld + col] = acc[mi][ni][2 * h + q];
                }
            }
        }
}

// ===========================================================================
// Triangular solves with the LU factors, z = U^-1 L^-1 r (FP32), blocked by 64 rows.
// ===========================================================================
__global__ void k_trsv_init(NewtonCell* nc, int nslots) {
    NewtonCell& N = nc[blockIdx.y];
    if (blockIdx.y >= nslots || !N.active) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * N.n; i += gridDim.x * blockDim.x) N.z[i] = (float)N.r[i];
}

// The triangular solves in one launch per direction (a sweep): persistent CTAs take the
// 64-row blocks of every cell from a shared counter, in an order in which each cell's
// blocks come in dependency order (forward: first to last; backward: last to first), so a
// block only ever waits for blocks that running CTAs took before it.  For its block a CTA
// subtracts the contributions of the solved blocks as their solutions are published (a
// warp per eight rows, each row's 64 entries read coalesced: the factor is read once),
// solves the diagonal block with its explicit inverse and publishes the solution with the
// sweep's epoch in the cell's flag of that block.  Row r's right-hand side takes the solved
// blocks' contributions one block at a time in solve order, each a 64-entry dot product
// reduced across the warp.  Every wait is bounded: on a timeout the CTA flags the cell
// (norms[3] = 3) and raises the sweep's abort word, which ends every other wait (and flags
// the waiting cells too).
// sweep[0]: the block counter (zero before the launch); sweep[1]: the abort word.
constexpr long long kSweepWait = 2000000000ll;   // SM clocks (about 1 s) before a wait gives up

// 8 warps of 8 rows each; 32 registers, so that 8 CTAs (8 blocks in flight) fit on an SM:
// measured on the 512-cell implicit step, the sweeps take 84, 75 and 64 ms per step at 5, 6
// and 8 CTAs per SM, and 75 ms with CTAs of 4 warps at 12 per SM.
constexpr int kSweepThreads = 256;

// withhold >= 0 (tests of the timeout path only): that block of every cell is solved but its
// flag is never published, so every block after it waits until wait_limit clocks run out.
__global__ void __launch_bounds__(kSweepThreads, 8) k_trsv_sweep(NewtonCell* nc, int nslots, int maxblk, int upper,
                                                                 int epoch, int* sweep, int withhold,
                                                                 long long wait_limit) {
    constexpr int kW = kSweepThreads / 32;   // warps
    constexpr int kR = kNb / kW;             // rows per warp
    __shared__ int s_t;
    __shared__ float T[kNb][kNb + 1];
    __shared__ float rb[kNb];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = maxblk * nslots;
    volatile int* abort_w = sweep + 1;
    for (;;) {
        __syncthreads();   // the previous block's shared arrays are free
        if (threadIdx.x == 0) s_t = atomicAdd(sweep, 1);
        __syncthreads();
        const int t = s_t;
        if (t >= total) break;
        const int slot = t % nslots, rt = t / nslots;   // by block rank, then cell
        NewtonCell& N = nc[slot];
        const int m = 2 * N.n, nblk = (m + kNb - 1) / kNb;
        if (!N.active || rt >= nblk) continue;
        const int b = upper ? nblk - 1 - rt : rt;
        const int b0 = b * kNb, kb = min(kNb, m - b0);
        const float* in = upper ? N.zt : N.z;   // this pass's right-hand side
        float* out = upper ? N.z : N.zt;        // this pass's solution
        volatile int* flag = N.flags;
        const float* inv = N.Dinv + (size_t)b * 2 * kNb * kNb + (upper ? kNb * kNb : 0);
        if (!upper)
            for (int i = threadIdx.x; i < kNb * kNb; i += blockDim.x) T[i >> 6][i & (kNb - 1)] = inv[i];
        else   // Uinv from its stored transpose
            for (int i = threadIdx.x; i < kNb * kNb; i += blockDim.x) T[i & (kNb - 1)][i >> 6] = inv[i];
        // this warp's rows: b0 + warp + kW u, u < kR
        float acc[kR];
#pragma unroll
        for (int u = 0; u < kR; ++u) {
            const int r = warp + kW * u;
            acc[u] = r < kb ? in[b0 + r] : 0.0f;
        }
        // the solved blocks j, in solve order
        const int jstep = upper ? -1 : 1;
        int j = upper ? nblk - 1 : 0;
        while (j != b) {
            // lane 0 finds how far the consecutive published blocks reach (waiting, bounded,
            // for the first one), then the warp applies them
            int ready = j;
            if (lane == 0) {
                const long long t0 = clock64();
                bool stop = false;
                while (flag[ready] != epoch) {
                    if (*abort_w) stop = true;
                    else if (clock64() - t0 > wait_limit) {
                        *abort_w = 1;
                        stop = true;
                    }
                    if (stop) break;
                    __nanosleep(64);
                }
                if (stop) {
                    N.norms[3] = 3.0;   // this cell's solution is not valid
                    ready = b;          // apply nothing more
                } else {
                    while (ready != b && flag[ready] == epoch) ready += jstep;
                }
                __threadfence();        // the solutions published before the flags
            }
            ready = __shfl_sync(0xffffffffu, ready, 0);
            for (; j != ready; j += jstep) {
                const int j0 = j * kNb, kj = min(kNb, m - j0);
                const float x0 = lane < kj ? __ldcg(out + j0 + lane) : 0.0f;
                const float x1 = lane + 32 < kj ? __ldcg(out + j0 + lane + 32) : 0.0f;
#pragma unroll
                for (int h = 0; h < kR / 8; ++h) {   // eight rows at a time
                    float sp[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int r = warp + kW * (8 * h + u);
                        const float* Ai = N.J + (size_t)(b0 + r) * N.ld + j0;
                        sp[u] = r < kb ? (lane < kj ? Ai[lane] * x0 : 0.0f) +
                                             (lane + 32 < kj ? Ai[lane + 32] * x1 : 0.0f)
                                       : 0.0f;
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                        for (int u = 0; u < 8; ++u) sp[u] += __shfl_xor_sync(0xffffffffu, sp[u], o);
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[8 * h + u] -= sp[u];
                }
            }
        }
        if (lane == 0)
#pragma unroll
            for (int u = 0; u < kR; ++u) rb[warp + kW * u] = warp + kW * u < kb ? acc[u] : 0.0f;
        __syncthreads();
        if (threadIdx.x < kb) {
            float s = 0.0f;
#pragma unroll 16
            for (int k = 0; k < kNb; ++k) s += T[threadIdx.x][k] * rb[k];
            out[b0 + threadIdx.x] = s;
            __threadfence();
        }
        __syncthreads();
        if (threadIdx.x == 0 && b != withhold) flag[b] = epoch;
    }
}

// per-iteration clears, one launch each over all cells: the correction and the FP32
// workspace of active cells; entries [first, first + count) of every cell's norms;
// the dense tangent of active cells before its assembly
__global__ void k_newton_clear(NewtonCell* nc, int nslots) {
    NewtonCell& N = nc[blockIdx.y];
    if (blockIdx.y >= nslots || !N.active) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * N.n; i += gridDim.x * blockDim.x) {
        N.dx[i] = 0.0;
        N.z[i] = 0.0f;
    }
}
__global__ void k_norms_clear(double* norms, int nslots, int first, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nslots * count; i += gridDim.x * blockDim.x)
        norms[8 * (size_t)(i / count) + first + i % count] = 0.0;
}
__global__ void k_dense_clear(NewtonCell* nc, int nslots) {
    NewtonCell& N = nc[blockIdx.y];
    if (blockIdx.y >= nslots || !N.active) return;
    float4* J = reinterpret_cast<float4*>(N.J);   // 2n rows of ld floats, ld a multiple of 4
    const size_t n4 = (size_t)2 * N.n * N.ld / 4;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x)
        J[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// dx += z; r = -G - J dx in FP64 with J element by element (diagonal + the FP32 element
// tangents promoted), one CTA per patch; |r|inf per cell
__global__ void __launch_bounds__(kTanThreads) k_newton_refine(const CellDev* __restrict__ cells, NewtonCell* nc,
                                                              const int* __restrict__ cell_slot,
                                                              const WorkItem* __restrict__ work, int nwork,
                                                              int add_z) {
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const WorkItem it = work[w];
        const int slot = cell_slot[it.cell];
        if (slot < 0) continue;
        NewtonCell& N = nc[slot];
        if (!N.active) continue;
        const CellDev& c = cells[it.cell];
        const int4 pt = c.patch[it.idx];
        double rmax = 0.0;
        for (int i = threadIdx.x; i < pt.y; i += blockDim.x) {
            const int v = pt.x + i;
            double jd[2] = {0.0, 0.0};
            for (int k = c.vt_ptr[v]; k < c.vt_ptr[v + 1]; ++k) {
                const int code = c.vc_code[k];
                const int cv = code & 3;
                const int e = c.patch_elems[pt.z + (code >> 2)];
                const int4 t4 = c.tri[e];
                const int id[3] = {t4.x, t4.y, t4.z};
                const float* o = N.Ke + 36 * (size_t)e;
#pragma unroll
                for (int l = 0; l < 3; ++l)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const int col = 2 * id[l] + j;
                        const double dcol = N.dx[col] + (add_z ? (double)N.z[col] : 0.0);
                        jd[0] += (double)o[(2 * cv) * 6 + 2 * l + j] * dcol;
                        jd[1] += (double)o[(2 * cv + 1) * 6 + 2 * l + j] * dcol;
                    }
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int row = 2 * v + q;
                const double dr = N.dx[row] + (add_z ? (double)N.z[row] : 0.0);
                const double rr = -N.G[row] - (N.diag[v] * dr + jd[q]);
                N.r[row] = rr;
                rmax = fmax(rmax, fabs(rr));
            }
        }
        for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        if ((threadIdx.x & 31) == 0)
            atomicMax(reinterpret_cast<unsigned long long*>(N.norms + 2), (unsigned long long)__double_as_longlong(rmax));
    }
}

// dx += z (after every refine pass reads it)
__global__ void k_newton_accumulate(NewtonCell* nc, int nslots) {
    NewtonCell& N = nc[blockIdx.y];
    if (blockIdx.y >= nslots || !N.active) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * N.n; i += gridDim.x * blockDim.x) N.dx[i] += (double)N.z[i];
}

// d += dx (in-plane displacement), x = X + d in pos[par ^ 1]; init: d = x_pred - X
__global__ void k_newton_apply(const CellDev* __restrict__ cells, NewtonCell* nc, const int* __restrict__ cell_of_slot,
                               int nslots, int init) {
    NewtonCell& N = nc[blockIdx.y];
    if (blockIdx.y >= nslots || (!init && !N.active)) return;
    const CellDev& c = cells[cell_of_slot[blockIdx.y]];
    const int par = c.ctl[0];
    const double4* X = c.pos[par];
    double4* xp = c.pos[par ^ 1];
    double dxm = 0.0, dm = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N.n; v += gridDim.x * blockDim.x) {
        const double4 Xv = ld4(X + v);
        double4 q = ld4v(xp + v);
        if (init) {
            N.d[2 * v] = q.x - Xv.x;
            N.d[2 * v + 1] = q.y - Xv.y;
            continue;
        }
        const double d0 = N.d[2 * v] + N.dx[2 * v], d1 = N.d[2 * v + 1] + N.dx[2 * v + 1];
        N.d[2 * v] = d0;
        N.d[2 * v + 1] = d1;
        st4(xp + v, Xv.x + d0, Xv.y + d1, q.z);
        dxm = fmax(dxm, fmax(fabs(N.dx[2 * v]), fabs(N.dx[2 * v + 1])));
        dm = fmax(dm, fmax(fabs(d0), fabs(d1)));
    }
    if (init) return;
    for (int o = 16; o > 0; o >>= 1) {
        dxm = fmax(dxm, __shfl_xor_sync(0xffffffffu, dxm, o));
        dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(reinterpret_cast<unsigned long long*>(N.norms + 4), (unsigned long long)__double_as_longlong(dxm));
        atomicMax(reinterpret_cast<unsigned long long*>(N.norms + 5), (unsigned long long)__double_as_longlong(dm));
    }
}

// Finish the step at the converged x: V = (x - X)/dt, A = (V - V_old)/dt, ea += Res_ea / MM;
// the last block of a cell advances parity, clock and AP counter
__global__ void k_newton_finish(const CellDev* __restrict__ cells, NewtonCell* nc, const int* __restrict__ cell_of_slot,
                                int nslots, const double* __restrict__ res_ea, double dt, unsigned int* tickets) {
    const int slot = blockIdx.y;
    if (slot >= nslots) return;
    NewtonCell& N = nc[slot];
    const CellDev& c = cells[cell_of_slot[slot]];
    const int par = c.ctl[0];
    const double* eo = c.ea[par];
    double* en = c.ea[par ^ 1];
    const double* Rq = res_ea + 6 * (size_t)c.hoff;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N.n; v += gridDim.x * blockDim.x) {
        const double4 Vo = ld4(c.vel + v);
        const double Vn[2] = {N.d[2 * (size_t)v] / dt, N.d[2 * (size_t)v + 1] / dt};
        st4(c.acc + v, (Vn[0] - Vo.x) / dt, (Vn[1] - Vo.y) / dt, 0.0);
        st4(c.vel + v, Vn[0], Vn[1], 0.0);
        const double iMM = 1.0 / N.MM[v];
#pragma unroll
        for (int q = 0; q < 6; ++q) en[6 * (size_t)v + q] = eo[6 * (size_t)v + q] + Rq[6 * (size_t)v + q] * iMM;
        if (!isfinite(Vn[0] + Vn[1])) atomicOr(c.status, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int done = atomicAdd(tickets + slot, 1u);
        if ((int)done == (int)gridDim.x - 1) {
            tickets[slot] = 0;
            c.ctl[0] = par ^ 1;
            c.clk[0] = c.clk[0] + dt;
            c.ap[0] = c.ap[0] + 1ull;
        }
    }
}

// F_ext = F_FA + F_AP + F_bend + F_area (packed [3 n_total])
__global__ void k_sum4(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                       const double* __restrict__ d, double* __restrict__ o, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        o[i] = a[i] + b[i] + c[i] + d[i];
}

// ---------------------------------------------------------------------------- host launchers
static int g_num_sms = 0;

cudaError_t configure_lu_tc(int num_sms);
int lu_update_prefix(const NewtonCell* h, int nslots, const LuUpdateArgs& a, int* pref);
bool launch_lu_update_tc(NewtonCell* nc, const LuMaps* maps, const int* d_prefix, int nslots, int total,
                         const LuUpdateArgs& a, cudaStream_t st);
bool launch_lu_panels_tc(NewtonCell* nc, const LuMaps* maps, const int* d_prefix, int nslots, int total,
                         const LuUpdateArgs& a, cudaStream_t st);
LuUpdateArgs lu_panel_args(int k0, int kbase);

cudaError_t configure_newton(size_t max_smem, int num_sms) {
    g_num_sms = num_sms;
    cudaError_t ce = configure_lu_tc(num_sms);
    if (ce != cudaSuccess) return ce;
    cudaError_t e = cudaFuncSetAttribute((const void*)k_lu_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(float) * (kTileM * (kNb + 4) + kNb * (kTileN + 8))));
    if (e != cudaSuccess) return e;
    cudaFuncAttributes at;
    if ((e = cudaFuncGetAttributes(&at, (const void*)k_newton_tangent)) != cudaSuccess) return e;
    return cudaFuncSetAttribute((const void*)k_newton_tangent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(max_smem - at.sharedSizeBytes - 1024));
}

size_t newton_tangent_smem(int emax) { return sizeof(float) * 36 * (size_t)emax; }

void launch_newton_residual(const CellDev* cells, const NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n,
                            double dt, cudaStream_t st) {
    dim3 grid((unsigned)std::max(1, std::min((max_n + 255) / 256, 64)), (unsigned)nslots);
    k_newton_residual<<<grid, 256, 0, st>>>(cells, nc, cell_of_slot, nslots, dt);
}
void launch_newton_tangent(const CellDev* cells, const NewtonCell* nc, const int* cell_slot, const WorkItem* work,
                           int nwork, int emax, double dt, int dense, cudaStream_t st) {
    if (nwork <= 0) return;
    const int grid = std::min(nwork, std::max(1, g_num_sms) * 8);
    k_newton_tangent<<<grid, kTanThreads, newton_tangent_smem(emax), st>>>(cells, nc, cell_slot, work, nwork, emax, dt,
                                                                               dense);
}
// The blocked LU of every active cell, in lockstep over the largest matrix.  kind 1: the
// 64-wide right-looking algorithm with mma.sync updates (nb must be 64).  kind 0:
// outer blocks of nb columns (a multiple of 64 up to 1024), each factored recursively by
// halves: 64-wide leaves factor the diagonal block and the two panels, and each split
// updates its right half's column strip and row strip with K = the left half's width;
// the trailing matrix then takes one update with K = nb.  All updates and panels run on
// the tcgen05 tensor cores.  The per-launch tile counts go to the device in one copy
// (d_prefix, lu_prefix_capacity ints).
// A non-empty split update implies a 64-wide leaf inside the matrix (the leftmost of its
// right half), so there are at most two launches of two regions each per 64 columns, plus
// per outer block one update of one region.
size_t lu_prefix_capacity(int nslots, int max_m) {
    return (size_t)3 * ((size_t)(max_m + kNb - 1) / kNb + 1) * (2 * (size_t)nslots + 1);
}

// The kind-0 schedule for matrices of order up to max_m with outer blocks of nb columns.
// Columns [s, s + w) of the outer block starting at K0, recursively: factor the left half,
// update the right half's columns below it and the right half's rows to the right of the
// block with K = the left half's width, then factor the right half.  The strips inside an
// outer block thus run with K = 64, 128, ... instead of all with 64; the trailing matrix
// then takes one update with K = nb.  A 64-wide step at the matrix's end has no panels.
std::vector<LuOp> lu_schedule(int max_m, int nb) {
    std::vector<LuOp> ops;
    auto block = [&](auto&& self, int K0, int s, int w) -> void {
        if (s >= max_m) return;
        if (w == kNb) {
            ops.push_back({0, s, {}});
            if (max_m - s - kNb > 0) ops.push_back({1, s, lu_panel_args(s, s - K0)});
            return;
        }
        const int h = kNb * ((w / kNb + 1) / 2);
        self(self, K0, s, h);
        LuUpdateArgs a{};
        a.nreg = 2;
        a.rlo[0] = s + h; a.rhi[0] = -1; a.clo[0] = s + h; a.chi[0] = s + w;
        a.rlo[1] = s + h; a.rhi[1] = s + w; a.clo[1] = s + w; a.chi[1] = -1;
        a.ka = s;
        a.kb = s - K0;
        a.K = h;
        ops.push_back({2, s, a});
        self(self, K0, s + h, w - h);
    };
    for (int K0 = 0; K0 < max_m; K0 += nb) {
        block(block, K0, K0, nb);
        LuUpdateArgs a{};   // the trailing matrix, K = nb
        a.nreg = 1;
        a.rlo[0] = K0 + nb; a.rhi[0] = -1; a.clo[0] = K0 + nb; a.chi[0] = -1;
        a.ka = K0;
        a.kb = 0;
        a.K = nb;
        ops.push_back({2, K0, a});
    }
    return ops;
}

// side, ev[2] (optional): a second stream and two events of the caller.  The transpose of a
// leaf's row panel then runs on the side stream beside the leaf's diagonal factor (which
// reads and writes only the diagonal block and its inverses): the factor is latency-bound
// with one CTA per cell, the transpose bandwidth-bound, and both only follow the update
// before them.  The next leaf's transpose follows this leaf's panels in stream order (the
// side stream waits for an event recorded after them), so At is never overwritten early.
const char* launch_newton_lu(NewtonCell* nc, const NewtonCell* h_nc, int nslots, int max_m, const LuMaps* maps,
                             int* d_prefix, int nb, int kind, cudaStream_t st, cudaStream_t side,
                             const cudaEvent_t* ev) {
    const char* failed = nullptr;
    auto checked = [&](const char* name) {
        if (!failed && cudaGetLastError() != cudaSuccess) failed = name;
    };
    auto panels = [&](int k0, int kbase) {
        const int rest = max_m - k0 - kNb;
        const int half = std::max(1, std::min((rest + 255) / 256, 32));
        k_lu_panels<<<dim3(2 * half, nslots), 256, 0, st>>>(nc, nslots, k0, 2 * half, kbase);
    };
    if (kind == 1) {
        const size_t usm = sizeof(float) * (kTileM * (kNb + 4) + kNb * (kTileN + 8));
        for (int k0 = 0; k0 < max_m; k0 += kNb) {
            k_lu_diag<<<nslots, 256, 0, st>>>(nc, nslots, k0);
            const int rest = max_m - k0 - kNb;
            if (rest <= 0) break;
            panels(k0, 0);
            k_lu_update<<<dim3((rest + kTileN - 1) / kTileN, (rest + kTileM - 1) / kTileM, nslots), 256, usm, st>>>(
                nc, nslots, k0);
            checked("k_lu_diag, k_lu_panels or k_lu_update");
        }
        return failed;
    }
    struct Op {
        int type, k0, kbase, pref, total;   // type 0 diag, 1 panels (A12 transpose + tcgen05 panels), 2 update
        LuUpdateArgs a;
    };
    std::vector<Op> ops;
    std::vector<int> pref;
    for (const LuOp& o : lu_schedule(max_m, nb)) {
        if (o.type == 0) {
            ops.push_back({0, o.k0, 0, 0, 0, {}});
            continue;
        }
        const size_t at = pref.size();
        pref.resize(at + (size_t)nslots * o.a.nreg + 1);
        const int total = lu_update_prefix(h_nc, nslots, o.a, pref.data() + at);
        if (!total) {
            pref.resize(at);
            continue;
        }
        ops.push_back({o.type, o.k0, o.a.kb, (int)at, total, o.a});
    }
    if (pref.size() > lu_prefix_capacity(nslots, max_m)) return "tile lists (capacity)";
    if (!pref.empty()) cudaMemcpyAsync(d_prefix, pref.data(), sizeof(int) * pref.size(), cudaMemcpyHostToDevice, st);
    const bool overlap = side && ev;
    auto transpose = [&](int k0, cudaStream_t s) {
        const int rest = max_m - k0 - kNb;
        k_lu_transpose_a12<<<dim3((unsigned)((rest + kNb - 1) / kNb), (unsigned)nslots), 256, 0, s>>>(nc, nslots, k0);
        checked("k_lu_transpose_a12");
    };
    for (size_t i = 0; i < ops.size(); ++i) {
        const Op& o = ops[i];
        if (o.type == 0) {
            // a leaf with panels: its transpose on the side stream beside the diagonal factor
            const bool pair = overlap && i + 1 < ops.size() && ops[i + 1].type == 1 && ops[i + 1].k0 == o.k0;
            if (pair) {
                cudaEventRecord(ev[0], st);
                cudaStreamWaitEvent(side, ev[0], 0);
                transpose(o.k0, side);
                cudaEventRecord(ev[1], side);
            }
            k_lu_diag<<<nslots, 256, 0, st>>>(nc, nslots, o.k0);
            checked("k_lu_diag");
            if (pair) {
                cudaStreamWaitEvent(st, ev[1], 0);
                if (!launch_lu_panels_tc(nc, maps, d_prefix + ops[i + 1].pref, nslots, ops[i + 1].total, ops[i + 1].a,
                                         st) &&
                    !failed)
                    failed = "k_lu_panels_tc";
                ++i;
            }
        } else if (o.type == 1) {
            transpose(o.k0, st);
            if (!launch_lu_panels_tc(nc, maps, d_prefix + o.pref, nslots, o.total, o.a, st) && !failed)
                failed = "k_lu_panels_tc";
        } else {
            if (!launch_lu_update_tc(nc, maps, d_prefix + o.pref, nslots, o.total, o.a, st) && !failed)
                failed = "k_lu_update_tc";
        }
    }
    return failed;
}
void launch_newton_clear(NewtonCell* nc, int nslots, int max_n, cudaStream_t st) {
    k_newton_clear<<<dim3((unsigned)std::max(1, std::min((2 * max_n + 255) / 256, 32)), (unsigned)nslots), 256, 0, st>>>(
        nc, nslots);
}
void launch_norms_clear(double* norms, int nslots, int first, int count, cudaStream_t st) {
    const int n = nslots * count;
    k_norms_clear<<<std::max(1, std::min((n + 255) / 256, 64)), 256, 0, st>>>(norms, nslots, first, count);
}
void launch_dense_clear(NewtonCell* nc, int nslots, int max_n, cudaStream_t st) {
    const size_t n4 = (size_t)2 * max_n * (2 * max_n + 4) / 4;
    const unsigned gx = (unsigned)std::max<size_t>(1, std::min<size_t>((n4 + 255) / 256, 1024));
    k_dense_clear<<<dim3(gx, (unsigned)nslots), 256, 0, st>>>(nc, nslots);
}

// z = U^-1 L^-1 r for every active cell.  sweep: 2 ints of device scratch; *epoch: the last
// epoch used by this cell set's flags (advanced by two); withhold, wait_limit: see
// k_trsv_sweep (-1 and 0: the normal solve with waits of about 1 s).
void launch_newton_solve(NewtonCell* nc, int nslots, int max_n, int* sweep, int* epoch, cudaStream_t st,
                         int withhold, long long wait_limit) {
    if (wait_limit <= 0) wait_limit = kSweepWait;
    const int m = 2 * max_n, nblk = (m + kNb - 1) / kNb;
    k_trsv_init<<<dim3((unsigned)std::max(1, std::min((m + 255) / 256, 32)), (unsigned)nslots), 256, 0, st>>>(nc, nslots);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_trsv_sweep, kSweepThreads, 0) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int grid = std::max(1, std::min(nblk * nslots, std::max(1, g_num_sms) * per_sm));
    for (int upper = 0; upper < 2; ++upper) {   // forward with L, then backward with U
        *epoch += 1;
        cudaMemsetAsync(sweep, 0, 2 * sizeof(int), st);
        k_trsv_sweep<<<grid, kSweepThreads, 0, st>>>(nc, nslots, nblk, upper, *epoch, sweep, withhold, wait_limit);
    }
}
void launch_newton_refine(const CellDev* cells, NewtonCell* nc, const int* cell_slot, const WorkItem* work, int nwork,
                          int add_z, cudaStream_t st) {
    if (nwork <= 0) return;
    const int grid = std::min(nwork, std::max(1, g_num_sms) * 8);
    k_newton_refine<<<grid, kTanThreads, 0, st>>>(cells, nc, cell_slot, work, nwork, add_z);
}
void launch_newton_accumulate(NewtonCell* nc, int nslots, int max_n, cudaStream_t st) {
    dim3 grid((unsigned)std::max(1, std::min((2 * max_n + 255) / 256, 64)), (unsigned)nslots);
    k_newton_accumulate<<<grid, 256, 0, st>>>(nc, nslots);
}
void launch_newton_apply(const CellDev* cells, NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n, int init,
                         cudaStream_t st) {
    dim3 grid((unsigned)std::max(1, std::min((max_n + 255) / 256, 64)), (unsigned)nslots);
    k_newton_apply<<<grid, 256, 0, st>>>(cells, nc, cell_of_slot, nslots, init);
}
void launch_newton_finish(const CellDev* cells, NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n,
                          const double* res_ea, double dt, unsigned int* tickets, cudaStream_t st) {
    dim3 grid((unsigned)std::max(1, std::min((max_n + 255) / 256, 64)), (unsigned)nslots);
    k_newton_finish<<<grid, 256, 0, st>>>(cells, nc, cell_of_slot, nslots, res_ea, dt, tickets);
}
void launch_sum4(const double* a, const double* b, const double* c, const double* d, double* o, size_t n,
                 cudaStream_t st) {
    if (n == 0) return;
    const int grid = (int)std::min<size_t>((n + 255) / 256, 4096);
    k_sum4<<<grid, 256, 0, st>>>(a, b, c, d, o, n);
}

}  // namespace wcfe
