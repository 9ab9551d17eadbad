// wcfe_device.cuh — device-side data layout and math of the per-step
// mechanics (sm_103a).  Shared by the kernels (wcfe_kernels.cu) and by the host
// engine (wcfe_engine.cu) for the layout structs.
//
// Layout in HBM, per cell (one arena block per cell, 256-B aligned arrays):
//   pos[2][nv]   double4 (x, y, z, 0)  ping-pong: pos[par] = X (step start), pos[par^1] = x (step end)
//   vel, acc, vhl [nv] double4         V, A, and V_hlf of the last drop-in predict
//   ea[2][nv][6] double                ping-pong Euler-Almansi strain (Voigt xx yy zz xy xz yz)
//   cA, cC [nv] double, fau [nv] double4
//   tri [nt] int4 (a, b, c, 0); vt_ptr [nv+1], vc_code [3nt] uint16 one-ring in mesh order
//   patches: patch [np] int4 (v0, nv, e0, ne), patch_elems [sum ne] int32
//   boundary: bnd_rank [nv] int32 (-1 interior), bnd_cptr [nb+1], bnd_cand [..] int2 (nj, nint)
//   bnd_optr [nb+1], bnd_out: directed boundary edges; bnd_vert [nb] boundary vertices by rank
//   k1_part [nk1][4] double: per-block partial sums of area and area-weighted centroid
//   area4 [4] double: cell area and centroid of the predicted positions (written by the vertex phase)
//   rec[2][nv][3] float4: mixed form only, the FP32 element inputs of each vertex, by step parity
#pragma once
#include <cstdint>

#include <cuda.h>

#include "../../include/wcfe.h"

namespace wcfe {

constexpr int kK1Threads = 256;  // largest vertex-phase block (vertices per block = threads = CellDev::vb)

struct CellDev;
struct SubDev {                 // substrate mesh + uniform grid for point location
    int32_t nv, nt;
    const double4* X;           // previous positions (point location)
    const double4* x;           // current positions (displacement interpolation)
    const int4* tri;
    const int32_t* cell_ptr;    // [gx*gy+1]
    const int32_t* cell_tri;    // triangle ids, ascending within a grid cell
    double ox, oy, inv_h;
    int32_t gx, gy;
    int32_t moving;             // 0: x == X (rigid), the interpolated displacement is exactly 0
    // deformable substrate simulated by the same engine (A10): its table entry, whose step-start
    // positions and predicted displacement replace X and x above, and its reaction accumulator
    const CellDev* scell;
    unsigned long long* fext;   // [nv_s][4] fixed-point (2^-40) reaction forces of the cell's bonds
};

// FP32 copies of the per-cell constants the mixed form uses per vertex, converted
// once on the host so that the kernels do no FP64 -> FP32 parameter conversions.
enum { PF_LINEAR0 = 0, PF_MD = 1, PF_LINEAR = 2, PF_POLY = 3 };
struct ParamF {
    float k_lin, rest_len, poly_k0, poly_c3;   // poly_c3 = 1 / (3 x0^2)
    float ka, kb, iFa, iFb, k_on, rho_i_max;
    float drag, damp, rho;
    int32_t law;                               // PF_*: linear with zero rest length, MD table, linear, polynomial
    int32_t norm2d;
    // low parts (x - RN(x)) of the constants the Bell force and rate use in float-float
    float k_lin_lo, rest_len_lo, poly_k0_lo, poly_c3_lo, iFa_lo, iFb_lo;
    // the radial protrusion driver (wcfe_params.protrude_v, _cx, _cy) as float-float pairs
    float pv, pv_lo, pcx, pcx_lo, pcy, pcy_lo;
};

struct CellDev {
    int32_t nv, nt, nb, np, nk1;
    int32_t vb;                 // vertices per vertex-phase block (= its thread count); 2 vb elements per block
    int32_t has_sub;
    int32_t material;           // 1 cell membrane, 2 substrate (mat 2: no active stress, integrins, boundary
                                // terms or drag; external forces from fext_in)
    int64_t hoff;               // first vertex of this cell in the engine's packed host exchange arrays
    double4* pos[2];
    double4* vel;
    double4* acc;
    double4* vhl;
    double* ea[2];
    double* cA;
    double* cC;
    double4* fau;
    const double* rho_w;        // optional per-vertex integrin density (nullptr: rho_i_max); floats in a mixed engine
    const double* mu_e;         // optional per-element shear modulus (nullptr: prm.mu); floats in a mixed engine
    const int4* tri;
    const int32_t* vt_ptr;
    const uint16_t* vc_code;    // (slot << 2) | corner, slot local to the owner's patch
    const int4* patch;
    const int32_t* patch_elems;
    const int4* patch_x;        // per patch (h0, nh, c0, nc): halo list and one-ring code range (mixed form staging)
    const int32_t* patch_halo;  // halo vertices of each patch, ascending
    const uint16_t* patch_loc;  // [4 per element slot] corners as patch-local vertex indices
    const int4* patch_tri;      // [per element slot] (vertex a, b, c, element id)
    float4* stepc;              // [8] the mixed form's per-step cell constants (element and boundary terms)
    const int32_t* bnd_rank;
    const int32_t* bnd_cptr;
    const int2* bnd_cand;
    const int32_t* bnd_optr;    // [nb+1] directed boundary edges leaving each boundary vertex
    const int32_t* bnd_out;     //        and their end vertices (the boundary loop, mixed-form area)
    double* k1_part;
    double* area4;              // {A, cx, cy, cz} of the positions after predict, reduced by the vertex phase
    float4* rec[2];             // mixed form: per-vertex FP32 element inputs [nv][3] by step parity (wcfe_mixed.cu)
    const int32_t* bnd_vert;    // [nb] boundary vertices in rank order (the inverse of bnd_rank)
    // control words, advanced by the last patch-phase CTA of the cell to finish a step:
    int32_t* ctl;               // [0] parity (which pos/ea buffer holds the step-start state), [1] patch-phase
                                //     CTA ticket, [2] vertex-phase block ticket (FP64 form; the mixed form
                                //     only for imported positions), [3] step budget (serving):
                                //     0 unlimited, n > 0 steps left, -1 done (every kernel skips the cell)
    double* clk;                // [0] simulation time at the start of the next step
    unsigned long long* ap;     // [0] calculateForce_AP calls made (the AP counter of the next step)
    uint32_t* status;
    unsigned long long* fext_in;  // substrate cells: [nv][4] fixed-point reactions accumulated this step
    double ap_thresh;           // ap_rate dt exp(-ap_rate dt) for the engine's current dt (UL:1552)
    SubDev sub;
    wcfe_params prm;
    ParamF pf;
};

#ifdef __CUDACC__
// The step budget ctl[3] of a cell.  A kernel reads it before any work on the cell; the
// last patch-phase CTA of the cell's step (after every other CTA of that cell finished the
// step) counts it down, so all work of one launch sees the same value and a cell with n
// steps left runs exactly n more steps, however many are queued.
__device__ __forceinline__ bool cell_done(const CellDev& c) { return c.ctl[3] < 0; }
__device__ __forceinline__ void count_step(const CellDev& c) {
    const int32_t b = c.ctl[3];
    if (b > 0) c.ctl[3] = b > 1 ? b - 1 : -1;
}
#endif

inline ParamF make_paramf(const wcfe_params& p) {
    ParamF f{};
    f.k_lin = (float)p.k_lin;
    f.rest_len = (float)p.rest_len;
    f.poly_k0 = (float)p.poly_k0;
    f.poly_c3 = (float)(1.0 / (3.0 * p.poly_x0 * p.poly_x0));
    f.ka = (float)p.ka;
    f.kb = (float)p.kb;
    f.iFa = (float)(1.0 / p.Fa);
    f.iFb = (float)(1.0 / p.Fb);
    f.k_on = (float)p.k_on;
    f.rho_i_max = (float)p.rho_i_max;
    f.drag = (float)p.drag;
    f.damp = (float)p.damp;
    f.rho = (float)p.rho;
    f.law = p.force_law == WCFE_LAW_MD_TABLE ? PF_MD
          : p.force_law == WCFE_LAW_LINEAR ? (p.rest_len == 0.0 ? PF_LINEAR0 : PF_LINEAR)
          : PF_POLY;
    f.norm2d = p.linear_norm2d ? 1 : 0;
    auto lo = [](double x) { return (float)(x - (double)(float)x); };
    f.pv = (float)p.protrude_v;
    f.pv_lo = lo(p.protrude_v);
    f.pcx = (float)p.protrude_cx;
    f.pcx_lo = lo(p.protrude_cx);
    f.pcy = (float)p.protrude_cy;
    f.pcy_lo = lo(p.protrude_cy);
    f.k_lin_lo = lo(p.k_lin);
    f.rest_len_lo = lo(p.rest_len);
    f.poly_k0_lo = lo(p.poly_k0);
    f.poly_c3_lo = lo(1.0 / (3.0 * p.poly_x0 * p.poly_x0));
    f.iFa_lo = lo(1.0 / p.Fa);
    f.iFb_lo = lo(1.0 / p.Fb);
    return f;
}

// Newton work of one cell (implicit step, wcfe_newton.cu); device array, one entry per cell
struct NewtonCell {
    float* J;            // dense 2n x 2n tangent, row-major, leading dimension ld (FP32); LU factors in place
    float* Ke;           // [nt][36] element tangents: (2 k + i) * 6 + 2 l + j = d re[k][i] / d u[l][j]
    double* diag;        // [n] mass and damping diagonal m / dt^2 + (drag + damp m) / dt
    double* G;           // [2n] Newton residual
    double* dx;          // [2n] Newton correction
    double* d;           // [2n] the iterate as displacement x - X (keeps the inertia term free of the
                         //      rounding of x: m / dt^2 times ulp(x) would floor |G|)
    double* r;           // [2n] residual of the linear solve
    float* z;            // [2n] FP32 solve workspace
    const double* Fext;  // [3n] external forces at the predicted positions
    const double* Res;   // [3n] membrane residual at the iterate
    const double* MM;    // [n] lumped mass
    double* norms;       // [8]: |G|inf, force scale, |r|inf, non-finite or zero pivot flag, |dx|inf of the
                         //      last update, |d|inf
    int n, ld, active, pad;
    float* Ut;           // [2n][utld] transposed U rows of the current outer LU block (tensor-core operand)
    int utld, pad2;
    float* Dinv;         // [ceil(2n/64)][2][64][64] inverses of the 64 x 64 diagonal blocks' unit-lower and
                         //      upper factors (identity-padded), row-major
    float* zt;           // [2n] FP32 solve workspace (the forward solve's result)
    float* At;           // [2n][64] the current row panel A12, transposed (tensor-core operand)
    int* flags;          // [ceil(2n/64)] the triangular sweeps' published blocks (the sweep's epoch)
};

// TMA descriptors of one cell's dense LU (fp32, 128-byte swizzled boxes)
struct LuMaps {
    CUtensorMap jmap;    // J: 32 columns x 128 rows
    CUtensorMap umap;    // Ut: 32 columns x 128 rows
    CUtensorMap amap;    // At: 32 columns x 128 rows
    CUtensorMap dmap;    // the diagonal blocks' Linv / Uinv^T (Dinv as [nblk * 128][64]): 32 columns x 64 rows
};

// One trailing-update launch of the blocked LU: per cell, C[rows, cols] -= J[rows, ka:ka+K]
// Ut[cols, kb:kb+K]^T over up to two regions, each bound clamped to the cell's 2n (a
// negative upper bound means 2n)
struct LuUpdateArgs {
    int rlo[2], rhi[2], clo[2], chi[2];
    int nreg, ka, kb, K;
};

// One step of the tensor-core LU's schedule (host side): type 0 factors the 64 x 64
// diagonal block at k0 and forms its inverses; type 1 computes that step's panels (L21 for
// the rows below, U12 for the columns to the right; a = lu_panel_args); type 2 updates up
// to two regions, C[rlo:rhi, clo:chi] -= J[rows, ka:ka+K] U[K0+kb : K0+kb+K, cols] (a bound
// of -1 is the matrix's order).
struct LuOp {
    int type, k0;
    LuUpdateArgs a;
};

struct WorkItem {               // one block of a phase: (cell index into the table, block/patch index)
    int32_t cell, idx;
};

// Philox4x32-10, Salmon et al. SC'11 (the counter-based stream of include/wcfe.h)
__host__ __device__ inline void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__host__ __device__ inline uint32_t ap_draw(uint32_t seed, uint32_t stream, unsigned long long call, uint32_t k) {
    uint32_t ctr[4] = {k, (uint32_t)call, (uint32_t)(call >> 32), 0u};
    uint32_t key[2] = {seed, stream};
    uint32_t o[4];
    philox4x32_10(ctr, key, o);
    return o[0] >> 1;
}

}  // namespace wcfe
