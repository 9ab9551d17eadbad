// wcfe_lu_tc.cu — trailing updates of the implicit step's blocked LU on the
// 5th-generation tensor cores (tcgen05, TF32 inputs, FP32 accumulation in TMEM).
//
// One launch updates, for every active cell, C[rows, cols] -= L Ut^T with
// L = J[rows, ka:ka+K] (the L21 panel, K-major as stored) and Ut the transposed U rows
// of the current outer block (Ut[c][k] = U[K0 + k][c], written by the panel kernel).
// The MMA computes the transposed product D = Ut L^T with M = 128 columns of C and
// N = TM rows of C, so a TMEM lane is a column of C and a TMEM column is a row of C:
// each epilogue thread owns one column of the tile and reads and writes C one row at a
// time, a warp covering 32 consecutive floats (coalesced, no staging buffer).
//
// Persistent CTAs, one per SM, walk a flat list of TM x 128 tiles over all cells (the
// host gives the per-cell tile counts as a prefix sum); TM = 256 rows for the updates
// with K >= 512, whose operand reads from L2 bound them (a 256-row tile reads a quarter
// fewer operand bytes per flop), 128 for the narrower strips.  Every CTA loads all of its
// own operands (no cluster sharing), so no CTA waits on another.  Warp 0 streams the
// operand boxes with TMA into a 4-stage ring (K = 32 per stage, 128-byte swizzled); one thread of
// warp 1 issues the MMAs into two TMEM accumulators, so tile t + 1 multiplies while tile t
// is written back; 16 epilogue warps, four per TMEM lane quadrant (TM / 4 rows of C each,
// in slices of 32), prefetch each slice's C values before its product is needed, then
// subtract and store.
//
// Every wait is bounded: on a timeout the CTA flags the cell it was working on (norms[3],
// the LU's failure flag), stops issuing work, waits (bounded) for its copies and MMAs in
// flight, frees its TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "wcfe_device.cuh"
#include "wcfe_tc.cuh"

namespace wcfe {
namespace {

constexpr int kTile = 128;                         // tile columns of C (and rows, but for wide updates)
constexpr int kBK = 32;                            // K per pipeline stage (one 128-B swizzle atom of fp32)
constexpr int kStages = 4;
constexpr int kEpiWarps = 16;                     // four per TMEM lane quadrant, 32 rows of C each
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kBoxBytes = 128u * 128u;        // 128 rows x 128 B
// update tiles of TM rows x 128 columns of C: TM = 256 for the K >= 512 updates (a quarter
// fewer operand bytes per flop), 128 for the narrower strip updates
template <int TM>
__host__ __device__ constexpr uint32_t stage_bytes() { return (1 + TM / 128) * kBoxBytes; }   // Ut box, then TM / 128 L boxes
template <int TM>
__host__ __device__ constexpr size_t update_smem() { return 1024 + (size_t)kStages * stage_bytes<TM>() + 256; }
constexpr uint32_t kStageBytes = stage_bytes<128>();
constexpr long long kWait = 2000000000ll;          // SM clocks (about 1 s) before a wait gives up

struct Tile {
    int slot, reg, tm, tn, rhi, chi;
};

__device__ __forceinline__ void region_of(const LuUpdateArgs& a, int r, int m, int& rlo, int& rhi, int& clo,
                                          int& chi) {
    rlo = min(a.rlo[r], m);
    rhi = a.rhi[r] < 0 ? m : min(a.rhi[r], m);
    clo = min(a.clo[r], m);
    chi = a.chi[r] < 0 ? m : min(a.chi[r], m);
}

// flat tile f -> cell, tile origin; groups are (cell, region) pairs in cell-major order;
// tiles of TM rows x 128 columns
template <int TM = kTile>
__device__ __forceinline__ Tile decode_tile(const NewtonCell* nc, const int* __restrict__ prefix, int ngroups, const LuUpdateArgs& a,
                            int f) {
    int lo = 0, hi = ngroups;   // prefix[lo] <= f < prefix[hi]; empty groups are skipped
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= f) lo = mid;
        else hi = mid;
    }
    Tile t;
    t.slot = lo / a.nreg;
    const int reg = lo - t.slot * a.nreg;
    t.reg = reg;
    const int m = 2 * nc[t.slot].n;
    int rlo, rhi, clo, chi;
    region_of(a, reg, m, rlo, rhi, clo, chi);
    const int tiles_n = (chi - clo + kTile - 1) / kTile;
    const int local = f - __ldg(prefix + lo);
    t.tm = rlo + (local / tiles_n) * TM;
    t.tn = clo + (local % tiles_n) * kTile;
    t.rhi = rhi;
    t.chi = chi;
    return t;
}

template <int TM>
__global__ void __launch_bounds__(kThreads, 1) k_lu_update_tc(NewtonCell* nc, const LuMaps* __restrict__ maps,
                                                             const int* __restrict__ prefix, int ngroups,
                                                             LuUpdateArgs a) {
    constexpr int NH = TM / 128;                        // 32-row slices of C per epilogue warp
    constexpr uint32_t kSB = stage_bytes<TM>();
    constexpr uint32_t kCols = 2 * TM;                  // two TM-column fp32 accumulators
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* sm = tc_smem_raw + ((1024u - (smem_addr(tc_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + kStages * kSB);
    uint64_t* empty = full + kStages;
    uint64_t* tfull = empty + kStages;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint32_t* tbase_s = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_s = reinterpret_cast<volatile int*>(tbase_s + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = __ldg(prefix + ngroups);   // units
    const int nch = a.K / kBK;
    const int unit0 = blockIdx.x, nunits = gridDim.x;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort_s = 0;
        mbar_init_fence();
    }
    if (warp == 1) {
        tc_alloc(tbase_s, kCols);
        tc_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tbase_s;

    if (warp == 0) {
        // ---------------------------------------------------------------- TMA producer
        if (lane == 0) {
            int g = 0;   // chunks issued so far
            for (int f = unit0; f < total && !*abort_s; f += nunits) {
                const Tile t = decode_tile<TM>(nc, prefix, ngroups, a, f);
                const LuMaps* mp = maps + t.slot;
                tmap_acquire(&mp->umap);
                tmap_acquire(&mp->jmap);
                for (int c = 0; c < nch; ++c, ++g) {
                    const int s = g % kStages;
                    const uint32_t u = (uint32_t)(g / kStages);
                    if (!mbar_wait_bounded(empty + s, (u & 1u) ^ 1u, kWait)) {
                        *abort_s = 1;
                        nc[t.slot].norms[3] = 2.0;
                        break;
                    }
                    uint8_t* st = sm + s * kSB;
                    mbar_arrive_expect_tx(full + s, kSB);
                    tma_load_2d(st, &mp->umap, a.kb + c * kBK, t.tn, full + s);
#pragma unroll
                    for (int j = 0; j < NH; ++j)   // rows past the matrix read as zeros
                        tma_load_2d(st + (1 + j) * kBoxBytes, &mp->jmap, a.ka + c * kBK, t.tm + 128 * j, full + s);
                }
            }
            // every stage's last fill has landed before the CTA may exit
            for (int s = 0; s < kStages && s < g; ++s) {
                const uint32_t ulast = (uint32_t)((g - 1 - s) / kStages);
                mbar_wait_bounded(full + s, ulast & 1u, kWait);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = tc_idesc_tf32(kTile, TM);
            int g = 0, it = 0;
            for (int f = unit0; f < total && !*abort_s; f += nunits, ++it) {
                const int b = it & 1;
                const uint32_t v = (uint32_t)(it >> 1);
                if (!mbar_wait_bounded(tempty + b, (v & 1u) ^ 1u, kWait)) {
                    *abort_s = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tbase + (uint32_t)(b * TM);
                bool ok = true;
                for (int c = 0; c < nch; ++c, ++g) {
                    const int s = g % kStages;
                    const uint32_t u = (uint32_t)(g / kStages);
                    if (!mbar_wait_bounded(full + s, u & 1u, kWait)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_addr(sm + s * kSB);
                    const uint64_t da = tc_desc_k_sw128(sa), db = tc_desc_k_sw128(sa + kBoxBytes);
#pragma unroll
                    for (int k = 0; k < kBK / 8; ++k)
                        tc_mma_tf32(d, da + 2u * (uint32_t)k, db + 2u * (uint32_t)k, idesc, (uint32_t)(c | k));
                    tc_commit(empty + s);   // the stage is free once these MMAs have read it
                }
                if (!ok) {
                    *abort_s = 1;
                    break;
                }
                tc_commit(tfull + b);
            }
            tc_commit(drain);   // all MMAs issued by this thread have completed
            mbar_wait_bounded(drain, 0u, kWait);
        }
        __syncwarp();
    } else {
        // ---------------------------------------------------------------- epilogue: C -= D^T
        const int q = warp & 3;                   // the TMEM lane quadrant this warp may access
        const int g = (warp - 2) >> 2;            // this warp's NH slices of 32 rows: rows 32 (NH g + h)
        const uint32_t lane_field = (uint32_t)(32 * q) << 16;
        // Software-pipelined: once a slice's product is subtracted, the following slice's C
        // values (the same tile's next slice, or the next tile's first) are requested between
        // this slice's stores, so their latency overlaps the stores and the next product.  The
        // tiles of one launch are disjoint, so a load never reads what a store of this launch
        // writes.  A slice: rows r0 + r of column col, r < nrows valid.
        Tile t{};
        int ld = 0, nrows = 0;
        float* __restrict__ Cb = nullptr;
        auto slice = [&](int h) {
            const int col = t.tn + 32 * q + lane;
            const int r0 = t.tm + 32 * (NH * g + h);
            nrows = col < t.chi ? min(32, t.rhi - r0) : 0;
            Cb = nc[t.slot].J + (size_t)r0 * ld + col;
        };
        auto locate = [&](int ff) {
            t = decode_tile<TM>(nc, prefix, ngroups, a, ff);
            ld = nc[t.slot].ld;
            slice(0);
        };
        int f = unit0;
        float c[32];
        if (f < total) {
            locate(f);
#pragma unroll
            for (int r = 0; r < 32; ++r) c[r] = r < nrows ? Cb[r * ld] : 0.0f;
        }
        for (int it = 0; f < total; f += nunits, ++it) {
            const int b = it & 1;
            const uint32_t v = (uint32_t)(it >> 1);
            const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(tfull + b, v & 1u, kWait));
            if (!ok) {
                if (lane == 0) nc[t.slot].norms[3] = 2.0;
                *abort_s = 1;
                break;
            }
            tc_fence_after();
#pragma unroll 1
            for (int h = 0; h < NH; ++h) {
                float p[32];
                tc_ld_32x32b_x32(tbase + (uint32_t)(b * TM + 32 * (NH * g + h)) + lane_field, p);
                if (h == NH - 1) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(tempty + b);   // the accumulator may be overwritten
                }
#pragma unroll
                for (int r = 0; r < 32; ++r) p[r] = c[r] - p[r];
                // row r of this slice is stored, then row r of the following slice requested:
                // about 32 values stay live instead of 64
                float* __restrict__ Cs = Cb;
                const int lds = ld, ns = nrows;
                if (h + 1 < NH) slice(h + 1);
                else if (f + nunits < total) locate(f + nunits);
                else nrows = 0;
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    if (r < ns) *Cs = p[r];
                    Cs += lds;
                    c[r] = r < nrows ? Cb[r * ld] : 0.0f;
                }
            }
            if (*abort_s) break;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tc_dealloc(tbase, kCols);
    }
}

// ---------------------------------------------------------------------------- panels
// The two panels of a 64-wide LU step as tcgen05 GEMMs with N = 64, K = 64, from the
// diagonal block's explicit inverses (Dinv block b: Linv rows, then Uinv^T rows):
//   region 0, 128-row tiles of L21:  L21 = A21 Uinv     (A: J rows, B: Uinv^T)
//        D[i][j] in TMEM lane i: the thread of row i writes J[i][k0 + j], 64 B per slice;
//   region 1, 128-column tiles of U12:  U12^T = A12^T Linv^T   (A: At rows, B: Linv)
//        D[c][i] in TMEM lane c: Ut[c][kbase + i] (64 B per slice) and J[k0 + i][c]
//        (coalesced across the warp's columns).
// Same pipeline as the update kernel; 16 epilogue warps, each 16 TMEM columns of a quadrant.
constexpr int kPN = 64;                                  // panel width (N)
constexpr uint32_t kPBoxA = 128u * 128u, kPBoxB = 64u * 128u;
constexpr uint32_t kPStageBytes = kPBoxA + kPBoxB;       // 24 KB, a multiple of 1024
constexpr uint32_t kPTmemCols = 128;                     // two 64-column accumulators
constexpr size_t kPSmemBytes = 1024 + (size_t)kStages * kPStageBytes + 256;

__global__ void __launch_bounds__(kThreads, 1) k_lu_panels_tc(NewtonCell* nc, const LuMaps* __restrict__ maps,
                                                             const int* __restrict__ prefix, int ngroups,
                                                             LuUpdateArgs a) {
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* sm = tc_smem_raw + ((1024u - (smem_addr(tc_smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + kStages * kPStageBytes);
    uint64_t* empty = full + kStages;
    uint64_t* tfull = empty + kStages;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint32_t* tbase_s = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_s = reinterpret_cast<volatile int*>(tbase_s + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = __ldg(prefix + ngroups);
    const int k0 = a.ka, kbase = a.kb;
    const int dblk = (k0 / kPN) * 2 * kPN;   // the block's first row in the Dinv map
    constexpr int nch = kPN / kBK;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort_s = 0;
        mbar_init_fence();
    }
    if (warp == 1) {
        tc_alloc(tbase_s, kPTmemCols);
        tc_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tbase_s;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;
            for (int f = blockIdx.x; f < total && !*abort_s; f += gridDim.x) {
                const Tile t = decode_tile(nc, prefix, ngroups, a, f);
                const LuMaps* mp = maps + t.slot;
                const bool lpanel = t.reg == 0;
                const CUtensorMap* amap = lpanel ? &mp->jmap : &mp->amap;
                tmap_acquire(amap);
                tmap_acquire(&mp->dmap);
                for (int c = 0; c < nch; ++c, ++g) {
                    const int s = g % kStages;
                    const uint32_t u = (uint32_t)(g / kStages);
                    if (!mbar_wait_bounded(empty + s, (u & 1u) ^ 1u, kWait)) {
                        *abort_s = 1;
                        nc[t.slot].norms[3] = 2.0;
                        break;
                    }
                    uint8_t* st = sm + s * kPStageBytes;
                    mbar_arrive_expect_tx(full + s, kPStageBytes);
                    if (lpanel) tma_load_2d(st, amap, k0 + c * kBK, t.tm, full + s);   // A21 rows
                    else tma_load_2d(st, amap, c * kBK, t.tn, full + s);                // At rows
                    tma_load_2d(st + kPBoxA, &mp->dmap, c * kBK, dblk + (lpanel ? kPN : 0), full + s);
                }
            }
            for (int s = 0; s < kStages && s < g; ++s) {
                const uint32_t ulast = (uint32_t)((g - 1 - s) / kStages);
                mbar_wait_bounded(full + s, ulast & 1u, kWait);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tc_idesc_tf32(kTile, kPN);
            int g = 0, it = 0;
            for (int f = blockIdx.x; f < total && !*abort_s; f += gridDim.x, ++it) {
                const int b = it & 1;
                const uint32_t v = (uint32_t)(it >> 1);
                if (!mbar_wait_bounded(tempty + b, (v & 1u) ^ 1u, kWait)) {
                    *abort_s = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tbase + (uint32_t)(b * kPN);
                bool ok = true;
                for (int c = 0; c < nch; ++c, ++g) {
                    const int s = g % kStages;
                    const uint32_t u = (uint32_t)(g / kStages);
                    if (!mbar_wait_bounded(full + s, u & 1u, kWait)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_addr(sm + s * kPStageBytes);
                    const uint64_t da = tc_desc_k_sw128(sa), db = tc_desc_k_sw128(sa + kPBoxA);
#pragma unroll
                    for (int k = 0; k < kBK / 8; ++k)
                        tc_mma_tf32(d, da + 2u * (uint32_t)k, db + 2u * (uint32_t)k, idesc, (uint32_t)(c | k));
                    tc_commit(empty + s);
                }
                if (!ok) {
                    *abort_s = 1;
                    break;
                }
                tc_commit(tfull + b);
            }
            tc_commit(drain);
            mbar_wait_bounded(drain, 0u, kWait);
        }
        __syncwarp();
    } else {
        const int q = warp & 3;
        const int j0 = 16 * ((warp - 2) >> 2);   // the 16 TMEM columns (panel entries) of this warp
        const uint32_t lane_field = (uint32_t)(32 * q) << 16;
        __shared__ float stage_rows[kEpiWarps][32][17];   // per warp: 32 rows of 16 entries (padded)
        float (*S)[17] = stage_rows[warp - 2];
        int it = 0;
        for (int f = blockIdx.x; f < total; f += gridDim.x, ++it) {
            const int b = it & 1;
            const uint32_t v = (uint32_t)(it >> 1);
            const Tile t = decode_tile(nc, prefix, ngroups, a, f);
            const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(tfull + b, v & 1u, kWait));
            if (!ok) {
                if (lane == 0) nc[t.slot].norms[3] = 2.0;
                *abort_s = 1;
                break;
            }
            tc_fence_after();
            float p[16];
            tc_ld_32x32b_x16(tbase + (uint32_t)(b * kPN + j0) + lane_field, p);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty + b);
            NewtonCell& N = nc[t.slot];
            const int m = 2 * N.n;
            // Rows of 16 entries (this warp's TMEM columns) go out two rows per store
            // instruction, each a whole 64-byte segment, through the warp's staging tile:
            // lane l writes row (l >> 4) + 2 r2, entry l & 15.
            const int rl0 = lane >> 4, cl = lane & 15;
            if (t.reg == 0) {   // L21 rows t.tm + 32 q + i, entries k0 + j0 + 0..15 of each
#pragma unroll
                for (int r = 0; r < 16; ++r) S[lane][r] = p[r];
                __syncwarp();
                const int rbase = t.tm + 32 * q;
#pragma unroll 4
                for (int r2 = 0; r2 < 16; ++r2) {
                    const int rl = rl0 + 2 * r2, row = rbase + rl;
                    if (row < m) N.J[(size_t)row * N.ld + k0 + j0 + cl] = S[rl][cl];
                }
                __syncwarp();
            } else {            // U12 columns t.tn + 32 q + i: rows k0 + j0 + 0..15 of J, and Ut rows
                const int col = t.tn + 32 * q + lane;
                if (col < m) {
                    float* dst = N.J + (size_t)(k0 + j0) * N.ld + col;
#pragma unroll
                    for (int r = 0; r < 16; ++r) dst[(size_t)r * N.ld] = p[r];
                }
                if (N.Ut) {
#pragma unroll
                    for (int r = 0; r < 16; ++r) S[lane][r] = p[r];
                    __syncwarp();
                    const int cbase = t.tn + 32 * q;
#pragma unroll 4
                    for (int r2 = 0; r2 < 16; ++r2) {
                        const int rl = rl0 + 2 * r2, c = cbase + rl;
                        if (c < m) N.Ut[(size_t)c * N.utld + kbase + j0 + cl] = S[rl][cl];
                    }
                    __syncwarp();
                }
            }
            if (*abort_s) break;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tc_dealloc(tbase, kPTmemCols);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
int g_sms = 0;
int g_lu_tc_regs = 0, g_lu_tc_max_threads = 0;

int encode_f32_2d(CUtensorMap* map, const float* base, uint64_t cols, uint64_t rows, uint64_t row_bytes,
                  uint32_t box_rows = 128) {
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {32, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : -1;
}

}  // namespace

// driver entry point for tensor-map encoding, the kernel's shared-memory size, the SM count
cudaError_t configure_lu_tc(int num_sms) {
    g_sms = num_sms;
    if (!g_encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    cudaError_t e = cudaFuncSetAttribute((const void*)k_lu_update_tc<128>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)update_smem<128>());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute((const void*)k_lu_update_tc<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)update_smem<256>());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute((const void*)k_lu_panels_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kPSmemBytes);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes at;
    if ((e = cudaFuncGetAttributes(&at, (const void*)k_lu_update_tc<128>)) != cudaSuccess) return e;
    g_lu_tc_regs = at.numRegs;
    g_lu_tc_max_threads = at.maxThreadsPerBlock;
    if ((e = cudaFuncGetAttributes(&at, (const void*)k_lu_update_tc<256>)) != cudaSuccess) return e;
    g_lu_tc_regs = std::max(g_lu_tc_regs, at.numRegs);
    g_lu_tc_max_threads = std::min(g_lu_tc_max_threads, at.maxThreadsPerBlock);
    return cudaSuccess;
}

// registers per thread and the largest block the compiled update kernel can launch with
void lu_tc_attributes(int* regs, int* max_threads) {
    *regs = g_lu_tc_regs;
    *max_threads = g_lu_tc_max_threads;
}

// tensor maps of J and Ut for every cell (host copies of the NewtonCell entries); cells of
// 64 or fewer rows have no trailing update and get an empty entry.  0 on success.
int encode_lu_maps(const NewtonCell* h, int nslots, LuMaps* out) {
    if (!g_encode) return -1;
    for (int s = 0; s < nslots; ++s) {
        std::memset(&out[s], 0, sizeof(LuMaps));
        const uint64_t m = 2 * (uint64_t)h[s].n;
        if (m <= 64) continue;
        if (!h[s].Ut || h[s].utld % 32 != 0) return -1;
        if (encode_f32_2d(&out[s].jmap, h[s].J, m, m, sizeof(float) * (uint64_t)h[s].ld)) return -1;
        if (encode_f32_2d(&out[s].umap, h[s].Ut, (uint64_t)h[s].utld, m, sizeof(float) * (uint64_t)h[s].utld))
            return -1;
        if (!h[s].At || !h[s].Dinv) return -1;
        if (encode_f32_2d(&out[s].amap, h[s].At, 64, m, sizeof(float) * 64)) return -1;
        const uint64_t nblk = (m + 63) / 64;
        if (encode_f32_2d(&out[s].dmap, h[s].Dinv, 64, nblk * 128, sizeof(float) * 64, 64)) return -1;
    }
    return 0;
}

// tiles of one update launch per (cell, region) group, as a prefix sum (ngroups + 1 entries);
// returns the total
// rows of an update tile: 256 for the updates with K >= 512, else 128 (the kernel
// instantiation and the host's tile counts both follow this)
int lu_tile_rows(const LuUpdateArgs& a) { return a.K >= 512 ? 256 : kTile; }

int lu_update_prefix(const NewtonCell* h, int nslots, const LuUpdateArgs& a, int* pref) {
    const int tm = lu_tile_rows(a), tw = kTile;
    int acc = 0;
    for (int s = 0; s < nslots; ++s)
        for (int r = 0; r < a.nreg; ++r) {
            pref[s * a.nreg + r] = acc;
            if (!h[s].active) continue;
            const int m = 2 * h[s].n;
            const int rlo = std::min(a.rlo[r], m), rhi = a.rhi[r] < 0 ? m : std::min(a.rhi[r], m);
            const int clo = std::min(a.clo[r], m), chi = a.chi[r] < 0 ? m : std::min(a.chi[r], m);
            if (rhi > rlo && chi > clo) acc += ((rhi - rlo + tm - 1) / tm) * ((chi - clo + tw - 1) / tw);
        }
    pref[nslots * a.nreg] = acc;
    return acc;
}

bool launch_lu_update_tc(NewtonCell* nc, const LuMaps* maps, const int* d_prefix, int nslots, int total,
                         const LuUpdateArgs& a, cudaStream_t st) {
    if (g_lu_tc_max_threads < kThreads) return false;
    if (total <= 0) return true;
    const int grid = std::max(1, std::min(total, g_sms > 0 ? g_sms : 1));
    if (lu_tile_rows(a) == 256)
        k_lu_update_tc<256><<<grid, kThreads, update_smem<256>(), st>>>(nc, maps, d_prefix, nslots * a.nreg, a);
    else
        k_lu_update_tc<128><<<grid, kThreads, update_smem<128>(), st>>>(nc, maps, d_prefix, nslots * a.nreg, a);
    return cudaGetLastError() == cudaSuccess;
}

// the panels of the 64-wide step at a.ka = k0 (a.kb = its offset in Ut); regions as
// lu_panel_args builds them
bool launch_lu_panels_tc(NewtonCell* nc, const LuMaps* maps, const int* d_prefix, int nslots, int total,
                         const LuUpdateArgs& a, cudaStream_t st) {
    if (g_lu_tc_max_threads < kThreads) return false;
    if (total <= 0) return true;
    const int grid = std::max(1, std::min(total, g_sms > 0 ? g_sms : 1));
    k_lu_panels_tc<<<grid, kThreads, kPSmemBytes, st>>>(nc, maps, d_prefix, nslots * a.nreg, a);
    return cudaGetLastError() == cudaSuccess;
}

// region 0: 128-row tiles of L21 (rows k0 + 64 .. 2n); region 1: 128-column tiles of U12
LuUpdateArgs lu_panel_args(int k0, int kbase) {
    LuUpdateArgs a{};
    a.nreg = 2;
    a.rlo[0] = k0 + 64; a.rhi[0] = -1; a.clo[0] = 0; a.chi[0] = 1;
    a.rlo[1] = 0; a.rhi[1] = 1; a.clo[1] = k0 + 64; a.chi[1] = -1;
    a.ka = k0;
    a.kb = kbase;
    a.K = 64;
    return a;
}

}  // namespace wcfe
