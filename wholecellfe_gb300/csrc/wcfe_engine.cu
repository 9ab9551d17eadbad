// wcfe_engine.cu — host engine behind the C ABI (include/wcfe.h): cells in
// HBM, batched work lists, CUDA-graph replay, the shape autotuner and the
// serving loop.  Single device, one stream per engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/wcfe.h"
#include "wcfe_device.cuh"
#include "wcfe_frames.h"
#include "wcfe_serving.h"
#include "wcfe_topology.h"

namespace wcfe {
struct PatchArgs;
void launch_vertex_phase(const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
                         int threads, cudaStream_t st, const double* stage_in = nullptr, double* stage_out = nullptr);
void launch_predict(const CellDev* cells, int cell, double dt, double* xout, double* vhout, int nv, cudaStream_t st);
cudaError_t configure_kernels(size_t max_smem);
bool launch_patch_staged(const CellDev* cells, const WorkItem* work, int nwork, int cap_ne, int cap_nvp, int cap_nh,
                         int cap_nc, double dt, double dt_real, double ap_thresh, double t_override, int vh_from_buf,
                         int num_sms, cudaStream_t st);
size_t patch_smem_bytes(int prec, int mode, int emax);
size_t mixed_smem_bytes(int emax);
int mixed_occupancy(int threads, size_t smem, int kind);
void launch_patch_mixed(const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt, double dt_real,
                        double ap_thresh, double t_override, int vh_from_buf, int threads, int grid, cudaStream_t st,
                        int kind, int fused);
int patch_occupancy(int prec, int threads, size_t smem);
int vertex_occupancy(int threads);
bool mixed_available();
void launch_vertex_mixed(const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
                         int threads, cudaStream_t st, const double* stage_in, double* stage_out, int kind = 0);
void launch_patch(int prec, int mode, const CellDev* cells, const WorkItem* work, int nwork, int emax, double dt,
                  double dt_real, double ap_thresh, double t_override, int vh_from_buf, const double* centroid_dev,
                  double* o0, double* o1, double* o2, double* o3, double* o4, int threads, int grid, cudaStream_t st,
                  int packed = 0);
cudaError_t configure_newton(size_t max_smem, int num_sms);
size_t newton_tangent_smem(int emax);
void launch_newton_residual(const CellDev* cells, const NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n,
                            double dt, cudaStream_t st);
void launch_newton_tangent(const CellDev* cells, const NewtonCell* nc, const int* cell_slot, const WorkItem* work,
                           int nwork, int emax, double dt, int dense, cudaStream_t st);
const char* launch_newton_lu(NewtonCell* nc, const NewtonCell* h_nc, int nslots, int max_m, const LuMaps* maps,
                             int* d_prefix, int nb, int kind, cudaStream_t st, cudaStream_t side = nullptr,
                             const cudaEvent_t* ev = nullptr);
void lu_tc_attributes(int* regs, int* max_threads);
void launch_newton_clear(NewtonCell* nc, int nslots, int max_n, cudaStream_t st);
void launch_norms_clear(double* norms, int nslots, int first, int count, cudaStream_t st);
void launch_dense_clear(NewtonCell* nc, int nslots, int max_n, cudaStream_t st);
std::string lu_attr_note() {
    int regs = 0, mt = 0;
    lu_tc_attributes(&regs, &mt);
    return " (tensor-core update kernel: " + std::to_string(regs) + " registers, at most " + std::to_string(mt) +
           " threads per block)";
}
size_t lu_prefix_capacity(int nslots, int max_m);
std::vector<LuOp> lu_schedule(int max_m, int nb);
int encode_lu_maps(const NewtonCell* h, int nslots, LuMaps* out);
void launch_newton_solve(NewtonCell* nc, int nslots, int max_n, int* sweep, int* epoch, cudaStream_t st,
                         int withhold = -1, long long wait_limit = 0);
void launch_newton_refine(const CellDev* cells, NewtonCell* nc, const int* cell_slot, const WorkItem* work, int nwork,
                          int add_z, cudaStream_t st);
void launch_newton_accumulate(NewtonCell* nc, int nslots, int max_n, cudaStream_t st);
void launch_newton_apply(const CellDev* cells, NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n, int init,
                         cudaStream_t st);
void launch_newton_finish(const CellDev* cells, NewtonCell* nc, const int* cell_of_slot, int nslots, int max_n,
                          const double* res_ea, double dt, unsigned int* tickets, cudaStream_t st);
void launch_sum4(const double* a, const double* b, const double* c, const double* d, double* o, size_t n,
                 cudaStream_t st);
void launch_remesh_pack(const CellDev& c, int mixed, const void* rho, double* ext, unsigned long long* hdr,
                        cudaStream_t st);
void launch_remesh_split(double* ext, int n_old, const int* ks, int cnt, const int2* ab, cudaStream_t st);
void launch_remesh_unpack(const CellDev& c, int mixed, const double* ext, const int* keep, const double* x, void* rho,
                          const unsigned long long* hdr, cudaStream_t st);
}  // namespace wcfe

using namespace wcfe;

namespace {

enum { VP_PREDICT = 1, VP_UPDATE_FA = 2, VP_RECORD = 4, VP_EXPORT = 8, VP_IMPORT = 16, VP_NOAREA = 32 };
enum { PP_STEP = 0, PP_RESIDUAL = 1, PP_FORCES = 2 };

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

thread_local std::string g_last_error;
#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            g_last_error = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return WCFE_ERR_CUDA;                                                                       \
        }                                                                                               \
    } while (0)

double ap_threshold(const wcfe_params& p, double dt_real) { return p.ap_rate * dt_real * std::exp(-p.ap_rate * dt_real); }

// ---------------------------------------------------------------------------
struct Cell {
    int32_t id = -1;
    Topology topo;
    Patches patches;
    wcfe_params prm{};
    // device memory
    void* state_block = nullptr;
    size_t state_bytes = 0;
    void* patch_block = nullptr;
    size_t patch_bytes = 0;
    void* sub_block = nullptr;
    size_t sub_bytes = 0;
    double* rho_dev = nullptr;      // integrin density (floats for a mixed engine)
    size_t rho_size = 0;            // its allocation
    double* mu_dev = nullptr;       // per-element shear modulus (floats for a mixed engine)
    size_t mu_size = 0;
    // deformable substrate coupling (A10): a cell names its substrate cell; the substrate cell
    // owns the reaction accumulator; the cell owns the point-location grid over the substrate
    int32_t couple_sub = -1;
    bool is_sub = false;
    void* fext_block = nullptr;
    size_t fext_bytes = 0;
    void* cgrid_block = nullptr;
    size_t cgrid_bytes = 0;
    SubGrid cgrid;
    CellDev dev{};
    int32_t sub_nv = 0, sub_nt = 0;
    std::vector<int32_t> sub_tri;
    std::vector<double> sub_X, sub_x;
    bool sub_moving = false;
};

struct Graph {
    cudaGraphExec_t exec = nullptr;
    double dt = 0;
    int steps = 0;
    int kind = 0;                 // the step kind captured (STEP_FULL or STEP_MID)
    uint64_t version = 0;
};

// One group of the exchange path: consecutive cells of the table (also consecutive in the
// work lists and in the packed exchange array), their work-list ranges and vertex range.
struct XChunk {
    int k1_lo, k1_hi, k2_lo, k2_hi;
    size_t v_lo, v_hi;
};

}  // namespace

struct wcfe_engine {
    int device = 0;
    int prec = WCFE_PREC_FP64;
    uint64_t budget = 0;
    uint64_t used = 0;
    cudaStream_t stream = nullptr;
    // The exchange path (wcfe_engine_predict / _update) splits the cells into xchunks
    // groups.  Each group's phases run on its own stream (cstream), its copies on xstream,
    // so one group's predict and copy-out overlap another's update.  A group depends only
    // on its own earlier work (cells are independent), so the main stream joins the group
    // streams lazily: xpending marks group work the main stream has not waited for, and
    // every other entry point waits for it first (xjoin).  Events: xin copy-in of a group
    // done, xout a group predicted, cdone a group's work done, xprev the main stream's work.
    static constexpr int kXMax = 8;
    int xchunks = 8;
    std::vector<XChunk> xch;                 // the groups, kept for (xch_version, xch_count)
    uint64_t xch_version = ~0ull;
    int xch_count = 0;
    bool xpending = false;
    cudaStream_t xstream = nullptr;
    cudaStream_t cstream[kXMax] = {};
    cudaEvent_t xin[kXMax] = {}, xout[kXMax] = {}, cdone[kXMax] = {}, xprev = nullptr;
    int num_sms = 0;
    std::map<int32_t, std::unique_ptr<Cell>> cells;
    int32_t next_id = 0;
    // batched tables
    uint64_t version = 1;         // bumps on any change of the live set / topology / params
    uint64_t table_version = 0;
    double table_dt = -1.0;       // dt the per-cell AP thresholds in the table were computed for
    std::vector<int32_t> order;   // table index -> cell id
    std::vector<CellDev> table;
    std::vector<WorkItem> k1, k2;
    // k1 with every cell's block 0 first (the mixed vertex phase's area blocks start in
    // the first wave), stored on the device right after k1 in d_k1
    std::vector<WorkItem> k1a;
    int64_t total_nv = 0;         // vertices of all live cells (packed exchange arrays)
    double* d_xchg = nullptr;     // packed [total_nv][3] exchange buffer on the device
    size_t d_xchg_cap = 0;
    CellDev* d_table = nullptr;
    size_t d_table_cap = 0;
    WorkItem* d_k1 = nullptr;
    size_t d_k1_cap = 0;
    WorkItem* d_k2 = nullptr;
    size_t d_k2_cap = 0;
    // per-cell single-cell work lists for the drop-in calls (rebuilt on demand)
    WorkItem* d_one = nullptr;
    size_t d_one_cap = 0;
    // staging
    double* d_stage = nullptr;
    size_t d_stage_cap = 0;
    void* h_stage = nullptr;
    size_t h_stage_cap = 0;
    // shapes
    int patch_threads = 128;
    int patch_emax = 320;
    int vblock = 256;             // vertices (threads) per vertex-phase block
    int vertex_kind = 0;          // mixed form: vertex-phase kernel for 5 (0), 4 (1), 6 (2) or 8 (3) blocks per SM
    bool element_ff = false;      // mixed form: the float-float element (wcfe_engine_set_element_precision)
    int patch_kernel = 1;         // mixed form: 0 staged (bulk copies) where its plan fits, 1 plain
    bool fused = false;           // mixed form: runs of steps fold each next vertex phase into the patch phase
    // the implicit step's workspace (dense tangents, factors, solve vectors), kept between
    // calls while the cell set and the LU's outer block stay the same
    void* newton_plan = nullptr;
    uint64_t newton_version = 0;
    int newton_nb = 0;
    int lu_nb = 1024, lu_kind = 0; // implicit step's LU: outer block width, 0 tcgen05 / 1 mma.sync updates
    int lu_reuse = 1;             // 1: factor once per implicit step, 0: every Newton iteration
    int cap_ne = 0, cap_nvp = 0, cap_nh = 0, cap_nc = 0;   // largest patch over the cells (staging plan)
    int n2_sub = 0;               // patch work items of substrate cells, at the end of k2 (second launch)
    bool tuned = false;
    // graphs
    bool use_graphs = false;
    Graph graph;
    // timing
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> tev;  // per-step events of the last timed wcfe_engine_step: 3 per step
    int timed_steps = 0;
    float ms_v = 0, ms_p = 0, ms_span = 0;
    std::vector<float> step_ms;
    uint64_t launches = 0;
    // serving: tables uploaded without a host synchronisation, from two pinned buffers
    void* h_tab[2] = {nullptr, nullptr};
    size_t h_tab_cap[2] = {0, 0};
    cudaEvent_t tab_ev[2] = {nullptr, nullptr};
    int tab_buf = 0;
};

namespace {

int fail(const std::string& msg, int code) {
    g_last_error = msg;
    return code;
}

// kind 0 (tcgen05 updates): outer blocks of 64 to 1024 columns in steps of 64; kind 1: 64
bool lu_block_ok(int block, int kind) {
    if (kind == 1) return block == 64;
    return kind == 0 && block >= 64 && block <= 1024 && block % 64 == 0;
}

Cell* find(wcfe_engine* e, int32_t id) {
    auto it = e->cells.find(id);
    return it == e->cells.end() ? nullptr : it->second.get();
}

// ---- device memory of a cell -------------------------------------------------
size_t state_layout(int32_t nv, int32_t nt, int32_t nb, int32_t ncand, int32_t nk1, bool rec, size_t* off /* 28 */) {
    size_t o = 0;
    int i = 0;
    auto put = [&](size_t bytes) { off[i++] = o; o = align_up(o + bytes); };
    put(sizeof(double4) * nv);   // 0 pos0
    put(sizeof(double4) * nv);   // 1 pos1
    put(sizeof(double4) * nv);   // 2 vel
    put(sizeof(double4) * nv);   // 3 acc
    put(sizeof(double4) * nv);   // 4 vhl
    put(sizeof(double) * 6 * nv);  // 5 ea0
    put(sizeof(double) * 6 * nv);  // 6 ea1
    put(sizeof(double) * nv);    // 7 cA
    put(sizeof(double) * nv);    // 8 cC
    put(sizeof(double4) * nv);   // 9 fau
    put(sizeof(int4) * nt);      // 10 tri
    put(sizeof(int32_t) * (nv + 1));  // 11 vt_ptr
    put(sizeof(int32_t) * nv);   // 12 bnd_rank
    put(sizeof(int32_t) * (nb + 1));  // 13 bnd_cptr
    put(sizeof(int2) * std::max(ncand, 1));  // 14 bnd_cand
    put(sizeof(double) * 4 * nk1);  // 15 k1_part
    put(sizeof(int32_t) * 4);    // 16 ctl
    put(sizeof(double) * 2);     // 17 clk
    put(sizeof(unsigned long long) * 2);  // 18 ap
    put(sizeof(uint32_t) * 2);   // 19 status
    put(rec ? sizeof(float4) * 3 * (size_t)nv : 0);  // 20 mixed-form element records (3 float4 per vertex)
    put(sizeof(int32_t) * (nb + 1));  // 21 bnd_optr
    put(sizeof(int32_t) * std::max(2 * nb, 1));  // 22 bnd_out (at most a few edges per boundary vertex)
    put(sizeof(double) * 4);     // 23 area4
    put(sizeof(int32_t) * std::max(nb, 1));  // 24 bnd_vert: boundary vertices in rank order
    put(128);                    // 25 step constants of the mixed form (written by its vertex phase)
    put(rec ? sizeof(float4) * 3 * (size_t)nv : 0);  // 26 the second buffer of element records (by step parity)
    put(64);                     // 27 slack: 16-B-rounded bulk copies of the last arrays stay in the block
    return o;
}

// patch arrays; every array ends with 64 B of slack so that 16-B-rounded bulk copies stay in the block
size_t patch_layout(int32_t np, size_t nelems, size_t ncodes, size_t nhalo, size_t* off /* 7 */) {
    size_t o = 0;
    int i = 0;
    auto put = [&](size_t bytes) { off[i++] = o; o = align_up(o + bytes + 64); };
    put(sizeof(int4) * np);                               // 0 patch (v0, nvp, e0, ne)
    put(sizeof(int32_t) * std::max<size_t>(nelems, 1));   // 1 element ids
    put(sizeof(uint16_t) * std::max<size_t>(ncodes, 1));  // 2 one-ring slot codes
    put(sizeof(int4) * np);                               // 3 staging info (h0, nh, c0, nc)
    put(sizeof(int32_t) * std::max<size_t>(nhalo, 1));    // 4 halo vertices
    put(sizeof(uint16_t) * 4 * std::max<size_t>(nelems, 1));  // 5 element corners, patch-local
    put(sizeof(int4) * std::max<size_t>(nelems, 1));      // 6 element vertices and id per slot
    return o;
}

// per-vertex integrin density (double for FP64 engines, float for mixed ones) + slack
size_t rho_bytes(int32_t nv) { return sizeof(double) * (size_t)nv + 64; }

int32_t nk1_of(int32_t nv, int32_t nt, int32_t vb) {
    return std::max((nv + vb - 1) / vb, (nt + 2 * vb - 1) / (2 * vb));
}

int dev_alloc(wcfe_engine* e, void** p, size_t bytes) {
    if (e->budget && e->used + bytes > e->budget) return fail("HBM budget exceeded", WCFE_ERR_BUDGET);
    cudaError_t r = cudaMallocAsync(p, bytes, e->stream);
    if (r != cudaSuccess) {
        cudaGetLastError();
        return fail(std::string("cudaMallocAsync: ") + cudaGetErrorString(r), WCFE_ERR_NOMEM);
    }
    e->used += bytes;
    return WCFE_OK;
}
void dev_free(wcfe_engine* e, void*& p, size_t& bytes) {
    if (p) {
        cudaFreeAsync(p, e->stream);
        e->used -= bytes;
    }
    p = nullptr;
    bytes = 0;
}

void* host_stage(wcfe_engine* e, size_t bytes) {
    if (bytes > e->h_stage_cap) {
        if (e->h_stage) cudaFreeHost(e->h_stage);
        e->h_stage = nullptr;
        if (cudaMallocHost(&e->h_stage, bytes) != cudaSuccess) {
            e->h_stage_cap = 0;
            return nullptr;
        }
        e->h_stage_cap = bytes;
    }
    return e->h_stage;
}
double* dev_stage(wcfe_engine* e, size_t bytes) {
    if (bytes > e->d_stage_cap) {
        if (e->d_stage) cudaFree(e->d_stage);
        e->d_stage = nullptr;
        if (cudaMalloc(&e->d_stage, bytes) != cudaSuccess) {
            e->d_stage_cap = 0;
            return nullptr;
        }
        e->d_stage_cap = bytes;
    }
    return e->d_stage;
}

// the device pointers of a cell's state block (layout state_layout)
void bind_state(Cell* c, char* b, const size_t* off, int32_t nk1, int32_t vblock, bool mixed) {
    const Topology& T = c->topo;
    CellDev& d = c->dev;
    d.nv = T.nv;
    d.nt = T.nt;
    d.nb = T.nb;
    d.nk1 = nk1;
    d.vb = vblock;
    d.pos[0] = (double4*)(b + off[0]);
    d.pos[1] = (double4*)(b + off[1]);
    d.vel = (double4*)(b + off[2]);
    d.acc = (double4*)(b + off[3]);
    d.vhl = (double4*)(b + off[4]);
    d.ea[0] = (double*)(b + off[5]);
    d.ea[1] = (double*)(b + off[6]);
    d.cA = (double*)(b + off[7]);
    d.cC = (double*)(b + off[8]);
    d.fau = (double4*)(b + off[9]);
    d.tri = (const int4*)(b + off[10]);
    d.vt_ptr = (const int32_t*)(b + off[11]);
    d.bnd_rank = (const int32_t*)(b + off[12]);
    d.bnd_cptr = (const int32_t*)(b + off[13]);
    d.bnd_cand = (const int2*)(b + off[14]);
    d.k1_part = (double*)(b + off[15]);
    d.ctl = (int32_t*)(b + off[16]);
    d.clk = (double*)(b + off[17]);
    d.ap = (unsigned long long*)(b + off[18]);
    d.status = (uint32_t*)(b + off[19]);
    d.rec[0] = mixed ? (float4*)(b + off[20]) : nullptr;
    d.rec[1] = mixed ? (float4*)(b + off[26]) : nullptr;
    d.area4 = (double*)(b + off[23]);
    d.bnd_vert = (const int32_t*)(b + off[24]);
    d.stepc = (float4*)(b + off[25]);
    d.bnd_optr = (const int32_t*)(b + off[21]);
    d.bnd_out = (const int32_t*)(b + off[22]);
}

// host images of a cell's derived static arrays
void tri4_of(const Topology& T, std::vector<int4>& t4) {
    t4.resize(T.nt);
    for (int t = 0; t < T.nt; ++t) t4[t] = make_int4(T.tri[3 * t], T.tri[3 * t + 1], T.tri[3 * t + 2], 0);
}
void bnd_vert_of(const Topology& T, std::vector<int32_t>& bv) {
    bv.assign(T.nb, 0);
    for (int v = 0; v < T.nv; ++v)
        if (T.bnd_rank[v] >= 0) bv[T.bnd_rank[v]] = v;
}
// c_A = 100 at the start (cellBP/main.cpp:674-677), in the engine's layout: binary64, or a
// float-float hi plane then lo plane
void ca_init_of(int32_t nv, bool mixed, std::vector<double>& buf) {
    if (!mixed) {
        buf.assign(nv, 100.0);
        return;
    }
    buf.assign(nv, 0.0);   // 2 nv floats in the same bytes
    float* f = reinterpret_cast<float*>(buf.data());
    for (int v = 0; v < nv; ++v) f[v] = 100.0f;
}

// topology arrays of the bound state block, copied on stream st; the host sources must
// stay unchanged until the copies have run
int upload_state_arrays(Cell* c, cudaStream_t st, const std::vector<int4>& t4, const std::vector<int32_t>& bv,
                        const std::vector<double>& ca) {
    const Topology& T = c->topo;
    CellDev& d = c->dev;
    const int32_t ncand = (int32_t)(T.bnd_cand.size() / 2);
    CK(cudaMemcpyAsync((void*)d.bnd_optr, T.bnd_optr.data(), sizeof(int32_t) * (T.nb + 1), cudaMemcpyHostToDevice, st));
    if (!T.bnd_out.empty())
        CK(cudaMemcpyAsync((void*)d.bnd_out, T.bnd_out.data(), sizeof(int32_t) * T.bnd_out.size(), cudaMemcpyHostToDevice, st));
    if (T.nb > 0) CK(cudaMemcpyAsync((void*)d.bnd_vert, bv.data(), sizeof(int32_t) * T.nb, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)d.tri, t4.data(), sizeof(int4) * T.nt, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)d.vt_ptr, T.vt_ptr.data(), sizeof(int32_t) * (T.nv + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)d.bnd_rank, T.bnd_rank.data(), sizeof(int32_t) * T.nv, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)d.bnd_cptr, T.bnd_cptr.data(), sizeof(int32_t) * (T.nb + 1), cudaMemcpyHostToDevice, st));
    if (ncand) CK(cudaMemcpyAsync((void*)d.bnd_cand, T.bnd_cand.data(), sizeof(int2) * ncand, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d.cA, ca.data(), sizeof(double) * T.nv, cudaMemcpyHostToDevice, st));
    return WCFE_OK;
}

// upload the whole static part of a cell (topology) and zero the state
int upload_cell_topology(wcfe_engine* e, Cell* c) {
    const Topology& T = c->topo;
    int32_t ncand = (int32_t)(T.bnd_cand.size() / 2);
    int32_t nk1 = nk1_of(T.nv, T.nt, e->vblock);
    size_t off[32];
    const bool mixed = e->prec == WCFE_PREC_MIXED;
    size_t bytes = state_layout(T.nv, T.nt, T.nb, ncand, nk1, mixed, off);
    if (c->state_block && c->state_bytes != bytes) dev_free(e, c->state_block, c->state_bytes);
    if (!c->state_block) {
        int r = dev_alloc(e, &c->state_block, bytes);
        if (r) return r;
        c->state_bytes = bytes;
    }
    char* b = (char*)c->state_block;
    CK(cudaMemsetAsync(b, 0, bytes, e->stream));
    bind_state(c, b, off, nk1, e->vblock, mixed);
    if ((int64_t)T.bnd_out.size() > std::max<int64_t>(2 * (int64_t)T.nb, 1)) return fail("non-manifold boundary", WCFE_ERR_TOPOLOGY);
    std::vector<int4> t4;
    std::vector<int32_t> bv;
    std::vector<double> ca;
    tri4_of(T, t4);
    bnd_vert_of(T, bv);
    ca_init_of(T.nv, mixed, ca);
    int r = upload_state_arrays(c, e->stream, t4, bv, ca);
    if (r) return r;
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

// the device pointers of a cell's patch block (layout patch_layout)
void bind_patches(Cell* c, char* b, const size_t* off) {
    c->dev.np = c->patches.np;
    c->dev.patch = (const int4*)(b + off[0]);
    c->dev.patch_elems = (const int32_t*)(b + off[1]);
    c->dev.vc_code = (const uint16_t*)(b + off[2]);
    c->dev.patch_x = (const int4*)(b + off[3]);
    c->dev.patch_halo = (const int32_t*)(b + off[4]);
    c->dev.patch_loc = (const uint16_t*)(b + off[5]);
    c->dev.patch_tri = (const int4*)(b + off[6]);
}
// each element slot with its triangle's vertices (one load instead of two dependent ones)
void patch_tri_of(const Patches& P, const Topology& T, std::vector<int4>& pt) {
    pt.resize(P.elems.size());
    for (size_t k = 0; k < P.elems.size(); ++k) {
        const int32_t el = P.elems[k];
        pt[k] = make_int4(T.tri[3 * el], T.tri[3 * el + 1], T.tri[3 * el + 2], el);
    }
}
int upload_patch_arrays(Cell* c, cudaStream_t st, const std::vector<int4>& pt) {
    const Patches& P = c->patches;
    if (!pt.empty())
        CK(cudaMemcpyAsync((void*)c->dev.patch_tri, pt.data(), sizeof(int4) * pt.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)c->dev.patch, P.patch.data(), sizeof(int32_t) * P.patch.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)c->dev.patch_elems, P.elems.data(), sizeof(int32_t) * P.elems.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)c->dev.vc_code, P.vc_code.data(), sizeof(uint16_t) * P.vc_code.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)c->dev.patch_x, P.xinfo.data(), sizeof(int32_t) * P.xinfo.size(), cudaMemcpyHostToDevice, st));
    if (!P.halo.empty())
        CK(cudaMemcpyAsync((void*)c->dev.patch_halo, P.halo.data(), sizeof(int32_t) * P.halo.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void*)c->dev.patch_loc, P.loc.data(), sizeof(uint16_t) * P.loc.size(), cudaMemcpyHostToDevice, st));
    return WCFE_OK;
}

int upload_cell_patches(wcfe_engine* e, Cell* c) {
    std::string err = build_patches(c->patches, c->topo, e->patch_emax);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    const Patches& P = c->patches;
    size_t off[7];
    size_t bytes = patch_layout(P.np, P.elems.size(), P.vc_code.size(), P.halo.size(), off);
    if (c->patch_block && c->patch_bytes != bytes) dev_free(e, c->patch_block, c->patch_bytes);
    if (!c->patch_block) {
        int r = dev_alloc(e, &c->patch_block, bytes);
        if (r) return r;
        c->patch_bytes = bytes;
    }
    char* b = (char*)c->patch_block;
    CK(cudaMemsetAsync(b, 0, bytes, e->stream));
    bind_patches(c, b, off);
    std::vector<int4> pt;
    patch_tri_of(P, c->topo, pt);
    int r = upload_patch_arrays(c, e->stream, pt);
    if (r) return r;
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int upload_substrate(wcfe_engine* e, Cell* c) {
    dev_free(e, c->sub_block, c->sub_bytes);
    c->dev.has_sub = 0;
    std::memset(&c->dev.sub, 0, sizeof(SubDev));
    if (c->sub_nt <= 0) return WCFE_OK;
    SubGrid G;
    build_subgrid(G, c->sub_nv, c->sub_nt, c->sub_tri.data(), c->sub_X.data());
    size_t o = 0, off[6];
    auto put = [&](int i, size_t bytes) { off[i] = o; o = align_up(o + bytes); };
    put(0, sizeof(double4) * c->sub_nv);
    put(1, sizeof(double4) * c->sub_nv);
    put(2, sizeof(int4) * c->sub_nt);
    put(3, sizeof(int32_t) * G.cell_ptr.size());
    put(4, sizeof(int32_t) * std::max<size_t>(G.cell_tri.size(), 1));
    int r = dev_alloc(e, &c->sub_block, o);
    if (r) return r;
    c->sub_bytes = o;
    char* b = (char*)c->sub_block;
    SubDev& s = c->dev.sub;
    s.nv = c->sub_nv;
    s.nt = c->sub_nt;
    s.X = (const double4*)(b + off[0]);
    s.x = (const double4*)(b + off[1]);
    s.tri = (const int4*)(b + off[2]);
    s.cell_ptr = (const int32_t*)(b + off[3]);
    s.cell_tri = (const int32_t*)(b + off[4]);
    s.ox = G.ox;
    s.oy = G.oy;
    s.inv_h = G.inv_h;
    s.gx = G.gx;
    s.gy = G.gy;
    CK(cudaMemcpy2DAsync((void*)s.X, sizeof(double4), c->sub_X.data(), 3 * sizeof(double), 3 * sizeof(double), c->sub_nv,
                         cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpy2DAsync((void*)s.x, sizeof(double4), c->sub_x.data(), 3 * sizeof(double), 3 * sizeof(double), c->sub_nv,
                         cudaMemcpyHostToDevice, e->stream));
    std::vector<int4> t4(c->sub_nt);
    for (int t = 0; t < c->sub_nt; ++t) t4[t] = make_int4(c->sub_tri[3 * t], c->sub_tri[3 * t + 1], c->sub_tri[3 * t + 2], 0);
    CK(cudaMemcpyAsync((void*)s.tri, t4.data(), sizeof(int4) * c->sub_nt, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync((void*)s.cell_ptr, G.cell_ptr.data(), sizeof(int32_t) * G.cell_ptr.size(), cudaMemcpyHostToDevice, e->stream));
    if (!G.cell_tri.empty())
        CK(cudaMemcpyAsync((void*)s.cell_tri, G.cell_tri.data(), sizeof(int32_t) * G.cell_tri.size(), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    s.moving = c->sub_moving ? 1 : 0;
    c->dev.has_sub = 1;
    return WCFE_OK;
}

void free_cell(wcfe_engine* e, Cell* c) {
    dev_free(e, c->fext_block, c->fext_bytes);
    dev_free(e, c->cgrid_block, c->cgrid_bytes);
    if (c->mu_dev) {
        void* p = c->mu_dev;
        size_t b = c->mu_size;
        dev_free(e, p, b);
        c->mu_dev = nullptr;
    }
    dev_free(e, c->state_block, c->state_bytes);
    dev_free(e, c->patch_block, c->patch_bytes);
    dev_free(e, c->sub_block, c->sub_bytes);
    if (c->rho_dev) {
        size_t b = c->rho_size;
        void* p = c->rho_dev;
        dev_free(e, p, b);
        c->rho_dev = nullptr;
    }
}

// ---- batched tables -----------------------------------------------------------
void invalidate_graph(wcfe_engine* e);

template <class T>
int ensure_dev(T** p, size_t* cap, size_t n) {
    if (n > *cap) {
        if (*p) cudaFree(*p);
        *p = nullptr;
        size_t c = std::max<size_t>(n, 2 * *cap);
        if (cudaMalloc((void**)p, sizeof(T) * c) != cudaSuccess) {
            *cap = 0;
            return fail("cudaMalloc of a work list failed", WCFE_ERR_NOMEM);
        }
        *cap = c;
    }
    return WCFE_OK;
}

int table_index(wcfe_engine* e, int32_t id);

int build_tables(wcfe_engine* e);

int sync_tables(wcfe_engine* e, double dt = -1.0) {
    if (dt > 0 && dt != e->table_dt) {
        e->table_dt = dt;
        e->version++;
        invalidate_graph(e);
    }
    if (e->table_version == e->version) return WCFE_OK;
    int r = build_tables(e);
    if (r) return r;
    if ((r = ensure_dev(&e->d_table, &e->d_table_cap, std::max<size_t>(e->table.size(), 1)))) return r;
    if ((r = ensure_dev(&e->d_k1, &e->d_k1_cap, std::max<size_t>(2 * e->k1.size(), 1)))) return r;
    if ((r = ensure_dev(&e->d_k2, &e->d_k2_cap, std::max<size_t>(e->k2.size(), 1)))) return r;
    // coupled cells point at their substrate's table entry (device address, known now)
    for (size_t ti = 0; ti < e->table.size(); ++ti) {
        const Cell* c = e->cells.at(e->order[ti]).get();
        if (c->couple_sub < 0) continue;
        auto it = e->cells.find(c->couple_sub);
        if (it == e->cells.end()) return fail("coupled substrate cell no longer exists", WCFE_ERR_STATE);
        const int ts = table_index(e, c->couple_sub);
        SubDev& sd = e->table[ti].sub;
        sd.scell = e->d_table + ts;
        sd.fext = (unsigned long long*)it->second->fext_block;
    }
    if (!e->table.empty())
        CK(cudaMemcpyAsync(e->d_table, e->table.data(), sizeof(CellDev) * e->table.size(), cudaMemcpyHostToDevice, e->stream));
    if (!e->k1.empty()) {
        CK(cudaMemcpyAsync(e->d_k1, e->k1.data(), sizeof(WorkItem) * e->k1.size(), cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(e->d_k1 + e->k1.size(), e->k1a.data(), sizeof(WorkItem) * e->k1a.size(),
                           cudaMemcpyHostToDevice, e->stream));
    }
    if (!e->k2.empty())
        CK(cudaMemcpyAsync(e->d_k2, e->k2.data(), sizeof(WorkItem) * e->k2.size(), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    e->table_version = e->version;
    return WCFE_OK;
}

// the host tables of the live cells: the table entries, the work lists, the staging caps
int build_tables(wcfe_engine* e) {
    e->order.clear();
    e->table.clear();
    e->total_nv = 0;
    e->k1.clear();
    e->k2.clear();
    e->cap_ne = e->cap_nvp = e->cap_nh = e->cap_nc = 0;
    for (auto& kv : e->cells) {
        const Patches& P = kv.second->patches;
        e->cap_ne = std::max(e->cap_ne, P.max_ne);
        e->cap_nvp = std::max(e->cap_nvp, P.max_nvp);
        e->cap_nh = std::max(e->cap_nh, P.max_nh);
        e->cap_nc = std::max(e->cap_nc, P.max_nc);
    }
    std::vector<WorkItem> k2_sub;
    for (auto& kv : e->cells) {
        Cell* c = kv.second.get();
        c->dev.prm = c->prm;
        c->dev.pf = make_paramf(c->prm);
        c->dev.rho_w = c->rho_dev;
        c->dev.mu_e = c->mu_dev;
        c->dev.material = c->is_sub ? 2 : 1;
        c->dev.fext_in = (unsigned long long*)c->fext_block;
        c->dev.ap_thresh = e->table_dt > 0 ? ap_threshold(c->prm, e->table_dt) : 0.0;
        c->dev.hoff = e->total_nv;
        e->total_nv += c->topo.nv;
        int32_t ti = (int32_t)e->table.size();
        e->order.push_back(c->id);
        e->table.push_back(c->dev);
        for (int b = 0; b < c->dev.nk1; ++b) e->k1.push_back({ti, b});
        // substrate cells take their reactions after every cell's patch phase: a second launch
        for (int p = 0; p < c->dev.np; ++p) (c->is_sub ? k2_sub : e->k2).push_back({ti, p});
    }
    e->n2_sub = (int)k2_sub.size();
    e->k2.insert(e->k2.end(), k2_sub.begin(), k2_sub.end());
    e->k1a.clear();
    for (const WorkItem& w : e->k1)
        if (w.idx == 0) e->k1a.push_back(w);
    for (const WorkItem& w : e->k1)
        if (w.idx != 0) e->k1a.push_back(w);
    return WCFE_OK;
}

int table_index(wcfe_engine* e, int32_t id) {
    for (size_t i = 0; i < e->order.size(); ++i)
        if (e->order[i] == id) return (int)i;
    return -1;
}

int rec_flag(const wcfe_engine* e) { return e->prec == WCFE_PREC_MIXED ? VP_RECORD : 0; }

// vertex phase of the engine's arithmetic form (the mixed form has its own kernel)
void vphase(const wcfe_engine* e, const CellDev* cells, const WorkItem* work, int nwork, double dt, int flags, int grid,
            cudaStream_t st, const double* stage_in = nullptr, double* stage_out = nullptr) {
    if (e->prec == WCFE_PREC_MIXED)
        launch_vertex_mixed(cells, work, nwork, dt, flags, grid, e->vblock, st, stage_in, stage_out, e->vertex_kind);
    else launch_vertex_phase(cells, work, nwork, dt, flags, grid, e->vblock, st, stage_in, stage_out);
}

int grid_for(wcfe_engine* e, int nwork, int per_sm) {
    int g = e->num_sms * std::max(per_sm, 1);
    return std::max(1, std::min(nwork, g));
}

void invalidate_graph(wcfe_engine* e) {
    if (e->graph.exec) cudaGraphExecDestroy(e->graph.exec);
    e->graph.exec = nullptr;
}

// the main stream waits for the exchange path's group work (see wcfe_engine::xpending)
void xjoin(wcfe_engine* e) {
    if (!e || !e->xpending) return;
    for (int c = 0; c < wcfe_engine::kXMax; ++c) cudaStreamWaitEvent(e->stream, e->cdone[c], 0);
    e->xpending = false;
}

// The kinds of step in a run of explicit steps.  A mixed engine folds the vertex phase of
// step s + 1 into the patch phase of step s (each patch predicts its owned vertices once
// their update is done, and the cell's last patch forms the next area): the first step of
// a run launches the vertex phase and a fused patch phase, the middle steps one fused
// patch phase each, and the last step a plain patch phase, so that between runs the state
// is exactly that of the unfused steps.  The arithmetic is the same either way.
enum { STEP_FULL = 0, STEP_FIRST = 1, STEP_MID = 2, STEP_LAST = 3 };

// fused runs: the mixed form's plain patch kernels, no coupled substrate (whose patch phase
// must follow its cells' before their next prediction)
bool fused_ok(const wcfe_engine* e) {
    return e->prec == WCFE_PREC_MIXED && e->fused && e->patch_kernel != 0 && e->n2_sub == 0 && !e->element_ff;
}
int step_kind(const wcfe_engine* e, int s, int n) {
    if (n < 2 || !fused_ok(e)) return STEP_FULL;
    return s == 0 ? STEP_FIRST : (s == n - 1 ? STEP_LAST : STEP_MID);
}

// the patch phase of a step (STEP mode): the staged mixed kernel where it applies
void patch_step(wcfe_engine* e, const WorkItem* k2, int n2, double dt, double dt_real, double apt, double t_override,
                int vh_from_buf, cudaStream_t st = nullptr, int fused = 0) {
    if (!st) st = e->stream;
    if (e->prec == WCFE_PREC_MIXED) {
        if (e->patch_kernel == 0 && !e->element_ff &&
            launch_patch_staged(e->d_table, k2, n2, e->cap_ne, e->cap_nvp, e->cap_nh, e->cap_nc, dt, dt_real, apt,
                                t_override, vh_from_buf, e->num_sms, st))
            return;
        const int kind = e->element_ff ? 6 : (e->patch_kernel == 0 ? 1 : e->patch_kernel);
        const size_t smem = mixed_smem_bytes(e->patch_emax);
        const int okind = fused ? 5 : kind;   // the fused form is its own instantiation
        launch_patch_mixed(e->d_table, k2, n2, e->patch_emax, dt, dt_real, apt, t_override, vh_from_buf,
                           e->patch_threads, grid_for(e, n2, mixed_occupancy(e->patch_threads, smem, okind)), st, kind,
                           fused);
        return;
    }
    size_t smem = patch_smem_bytes(e->prec, PP_STEP, e->patch_emax);
    launch_patch(e->prec, PP_STEP, e->d_table, k2, n2, e->patch_emax, dt, dt_real, apt, t_override, vh_from_buf,
                 nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, e->patch_threads,
                 grid_for(e, n2, patch_occupancy(e->prec, e->patch_threads, smem)), st);
}

// one explicit step of the cells listed in (k1, k2) device lists; kind: STEP_* above
int enqueue_step(wcfe_engine* e, const WorkItem* k1, int n1, const WorkItem* k2, int n2, double dt,
                 int kind = STEP_FULL) {
    const double apt = std::numeric_limits<double>::quiet_NaN();  // per-cell thresholds from the table
    int g1 = grid_for(e, n1, vertex_occupancy(e->vblock));
    cudaEvent_t* tv = (e->timing && e->tev.size() >= 3) ? &e->tev[3 * (size_t)e->timed_steps] : nullptr;
    const bool vertex = kind == STEP_FULL || kind == STEP_FIRST;
    // the whole engine's list: the same items with every cell's block 0 first
    const WorkItem* k1v = (k1 == e->d_k1 && n1 == (int)e->k1.size() && e->k1a.size() == e->k1.size()) ? k1 + n1 : k1;
    if (tv) cudaEventRecord(tv[0], e->stream);
    if (vertex) vphase(e, e->d_table, k1v, n1, dt, VP_PREDICT | VP_UPDATE_FA | rec_flag(e), g1, e->stream);
    if (tv) cudaEventRecord(tv[1], e->stream);
    const int nsub = (k2 == e->d_k2 && n2 == (int)e->k2.size()) ? e->n2_sub : 0;
    patch_step(e, k2, n2 - nsub, dt, dt, apt, std::numeric_limits<double>::quiet_NaN(), 0, nullptr,
               (kind == STEP_FIRST || kind == STEP_MID) ? 1 : 0);
    if (nsub > 0) {   // substrate cells, after the reactions of their coupled cells
        patch_step(e, k2 + (n2 - nsub), nsub, dt, dt, apt, std::numeric_limits<double>::quiet_NaN(), 0);
        e->launches += 1;
    }
    if (tv) {
        cudaEventRecord(tv[2], e->stream);
        e->timed_steps++;
    }
    e->launches += vertex ? 2 : 1;
    CK(cudaGetLastError());
    return WCFE_OK;
}

// single-cell work lists for the drop-in entry points
int one_cell_lists(wcfe_engine* e, Cell* c, int ti, int* n1, int* n2) {
    std::vector<WorkItem> w;
    for (int b = 0; b < c->dev.nk1; ++b) w.push_back({ti, b});
    for (int p = 0; p < c->dev.np; ++p) w.push_back({ti, p});
    int r = ensure_dev(&e->d_one, &e->d_one_cap, w.size());
    if (r) return r;
    CK(cudaMemcpyAsync(e->d_one, w.data(), sizeof(WorkItem) * w.size(), cudaMemcpyHostToDevice, e->stream));
    *n1 = c->dev.nk1;
    *n2 = c->dev.np;
    return WCFE_OK;
}

int read_parity(wcfe_engine* e, Cell* c, int* par) {
    int32_t ctl[2];
    CK(cudaMemcpyAsync(ctl, c->dev.ctl, sizeof ctl, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *par = ctl[0] & 1;
    return WCFE_OK;
}

// host [n][3] <-> device double4 (strided 2-D copy, no kernel)
int put3(wcfe_engine* e, double4* d, const double* h, int n) {
    CK(cudaMemcpy2DAsync(d, sizeof(double4), h, 3 * sizeof(double), 3 * sizeof(double), n, cudaMemcpyHostToDevice, e->stream));
    return WCFE_OK;
}
int get3(wcfe_engine* e, double* h, const double4* d, int n) {
    CK(cudaMemcpy2DAsync(h, 3 * sizeof(double), d, sizeof(double4), 3 * sizeof(double), n, cudaMemcpyDeviceToHost, e->stream));
    return WCFE_OK;
}

// A mixed engine keeps its state as float-float pairs (hi = RN(x), lo = RN(x - hi))
// in the same slots, as structures of arrays over the cell's n vertices
// (wcfe_mixed.cu): pos, vel, fau, vhl as hi float4[n] then lo float4[n]; acc as the
// FP32 acceleration float4[n]; ea as hi float4[n] (xx yy zz xy), lo float4[n],
// then float4[n] (xz hi, yz hi, xz lo, yz lo); cA, cC as hi float[n] then lo float[n].
// Positions are triple-float (wcfe_ff.cuh): hi float4 (x.h, y.h, z.h, x.l) and lo float4
// (x.m, y.m, z.m, y.l), exact for any binary64 input (z is 0 in the planar mixed form).
// These convert on the host.
inline void split_ff(double x, float* hi, float* lo) {
    const float h = (float)x;
    *hi = h;
    *lo = (float)(x - (double)h);
}
inline void split_tf(double x, float* h, float* m, float* l) {
    *h = (float)x;
    const double r = x - (double)*h;
    *m = (float)r;
    *l = (float)(r - (double)*m);
}
int put_ff(wcfe_engine* e, void* d, const double* h, int n, int kind) {
    const size_t N = (size_t)n;
    std::vector<float> b;
    if (kind == 4) {                       // [n][3] positions (triple-float x, y; float-float z)
        b.assign(8 * N, 0.0f);
        for (size_t v = 0; v < N; ++v) {
            const double* q = h + 3 * v;
            split_tf(q[0], &b[4 * v + 0], &b[4 * (N + v) + 0], &b[4 * v + 3]);
            split_tf(q[1], &b[4 * v + 1], &b[4 * (N + v) + 1], &b[4 * (N + v) + 3]);
            split_ff(q[2], &b[4 * v + 2], &b[4 * (N + v) + 2]);
        }
    } else if (kind == 0 || kind == 1) {   // [n][3] vectors
        b.assign((kind == 1 ? 4 : 8) * N, 0.0f);
        for (size_t v = 0; v < N; ++v)
            for (int k = 0; k < 3; ++k) {
                if (kind == 1) b[4 * v + k] = (float)h[3 * v + k];
                else split_ff(h[3 * v + k], &b[4 * v + k], &b[4 * (N + v) + k]);
            }
    } else if (kind == 2) {                // [n][6] strain (xx yy zz xy xz yz)
        b.assign(12 * N, 0.0f);
        for (size_t v = 0; v < N; ++v) {
            const double* q = h + 6 * v;
            for (int k = 0; k < 4; ++k) split_ff(q[k], &b[4 * v + k], &b[4 * (N + v) + k]);
            split_ff(q[4], &b[4 * (2 * N + v) + 0], &b[4 * (2 * N + v) + 2]);
            split_ff(q[5], &b[4 * (2 * N + v) + 1], &b[4 * (2 * N + v) + 3]);
        }
    } else {                               // [n] scalars
        b.assign(2 * N, 0.0f);
        for (size_t v = 0; v < N; ++v) split_ff(h[v], &b[v], &b[N + v]);
    }
    CK(cudaMemcpyAsync(d, b.data(), sizeof(float) * b.size(), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}
int get_ff(wcfe_engine* e, double* h, const void* d, int n, int kind) {
    const size_t N = (size_t)n;
    const size_t per = (kind == 0 || kind == 4) ? 8 : kind == 1 ? 4 : kind == 2 ? 12 : 2;
    std::vector<float> b(per * N);
    CK(cudaMemcpyAsync(b.data(), d, sizeof(float) * b.size(), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    auto ffd = [](float hi, float lo) { return (double)hi + (double)lo; };
    for (size_t v = 0; v < N; ++v) {
        if (kind == 4) {   // (h + m) is exact in binary64; one rounding for + l
            h[3 * v] = ffd(b[4 * v], b[4 * (N + v)]) + (double)b[4 * v + 3];
            h[3 * v + 1] = ffd(b[4 * v + 1], b[4 * (N + v) + 1]) + (double)b[4 * (N + v) + 3];
            h[3 * v + 2] = ffd(b[4 * v + 2], b[4 * (N + v) + 2]);
        } else if (kind == 0) for (int k = 0; k < 3; ++k) h[3 * v + k] = ffd(b[4 * v + k], b[4 * (N + v) + k]);
        else if (kind == 1) for (int k = 0; k < 3; ++k) h[3 * v + k] = (double)b[4 * v + k];
        else if (kind == 2) {
            double* q = h + 6 * v;
            for (int k = 0; k < 4; ++k) q[k] = ffd(b[4 * v + k], b[4 * (N + v) + k]);
            q[4] = ffd(b[4 * (2 * N + v) + 0], b[4 * (2 * N + v) + 2]);
            q[5] = ffd(b[4 * (2 * N + v) + 1], b[4 * (2 * N + v) + 3]);
        } else h[v] = ffd(b[v], b[N + v]);
    }
    return WCFE_OK;
}
enum { FF_VEC = 0, FF_ACC = 1, FF_EA = 2, FF_SCALAR = 3, FF_POS = 4 };

// the mixed form assumes a planar membrane with counter-clockwise triangles (its element
// inputs drop z and its area comes from the boundary loop)
int check_planar_ccw(const double* x, int n, const std::vector<int32_t>& T) {
    for (int v = 0; v < n; ++v)
        if (x[3 * v + 2] != 0.0) return fail("the mixed form needs a planar membrane (z = 0)", WCFE_ERR_ARG);
    for (size_t t = 0; 3 * t < T.size(); ++t) {
        const double* a = x + 3 * T[3 * t];
        const double* b = x + 3 * T[3 * t + 1];
        const double* q = x + 3 * T[3 * t + 2];
        if ((b[0] - a[0]) * (q[1] - a[1]) - (b[1] - a[1]) * (q[0] - a[0]) <= 0)
            return fail("the mixed form needs counter-clockwise, non-degenerate triangles", WCFE_ERR_ARG);
    }
    return WCFE_OK;
}


}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {
namespace {
void release_newton_plan(wcfe_engine* e);   // the implicit step's kept workspace (below)
}  // namespace


void wcfe_params_default(wcfe_params* p, int32_t variant) {
    std::memset(p, 0, sizeof *p);
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

uint32_t wcfe_ap_draw(uint32_t seed, uint32_t stream, uint64_t call, uint32_t k) {
    return ap_draw(seed, stream, (unsigned long long)call, k);
}
void wcfe_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox4x32_10(ctr, key, out); }

const char* wcfe_last_error(void) { return g_last_error.c_str(); }

int wcfe_engine_create(int32_t device, int32_t precision, uint64_t hbm_budget_bytes, wcfe_engine** out) {
    if (!out || (precision != WCFE_PREC_FP64 && precision != WCFE_PREC_MIXED)) return fail("bad argument", WCFE_ERR_ARG);
    if (precision == WCFE_PREC_MIXED && !mixed_available()) return fail("mixed-precision kernels not built", WCFE_ERR_ARG);
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device) {
        cudaGetLastError();
        return fail("no CUDA device", WCFE_ERR_NODEVICE);
    }
    std::unique_ptr<wcfe_engine> e(new wcfe_engine());
    e->device = device;
    e->prec = precision;
    e->budget = hbm_budget_bytes;
    CK(cudaSetDevice(device));
    CK(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device));
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    int max_optin = 0;
    CK(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    CK(configure_kernels((size_t)max_optin));
    CK(configure_newton((size_t)max_optin, e->num_sms > 0 ? e->num_sms : 1));
    for (auto& ev : e->ev) CK(cudaEventCreate(&ev));
    CK(cudaStreamCreateWithFlags(&e->xstream, cudaStreamNonBlocking));
    // exchange group c's stream at a higher priority than group c + 1's (as far as the
    // device's levels go): the block scheduler then finishes the groups in order, so each
    // group's copy to the host runs while later groups still compute
    int prio_least = 0, prio_greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    for (int c = 0; c < wcfe_engine::kXMax; ++c) {
        const int prio = std::min(prio_least, prio_greatest + c);
        CK(cudaStreamCreateWithPriority(&e->cstream[c], cudaStreamNonBlocking, prio));
        CK(cudaEventCreateWithFlags(&e->xin[c], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&e->xout[c], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&e->cdone[c], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&e->xprev, cudaEventDisableTiming));
    if (precision == WCFE_PREC_MIXED) { e->patch_threads = 128; e->patch_emax = 512; e->vblock = 256; }
    else { e->patch_threads = 64; e->patch_emax = 96; e->vblock = 64; }  // FP64: more, smaller blocks
    *out = e.release();
    return WCFE_OK;
}

int wcfe_engine_destroy(wcfe_engine* e) {
    if (!e) return WCFE_ERR_ARG;
    cudaSetDevice(e->device);
    xjoin(e);
    cudaStreamSynchronize(e->stream);
    release_newton_plan(e);
    for (auto& kv : e->cells) free_cell(e, kv.second.get());
    e->cells.clear();
    invalidate_graph(e);
    cudaStreamSynchronize(e->stream);
    if (e->d_table) cudaFree(e->d_table);
    if (e->d_k1) cudaFree(e->d_k1);
    if (e->d_k2) cudaFree(e->d_k2);
    if (e->d_one) cudaFree(e->d_one);
    if (e->d_xchg) cudaFree(e->d_xchg);
    if (e->d_stage) cudaFree(e->d_stage);
    if (e->h_stage) cudaFreeHost(e->h_stage);
    for (int k = 0; k < 2; ++k) {
        if (e->h_tab[k]) cudaFreeHost(e->h_tab[k]);
        if (e->tab_ev[k]) cudaEventDestroy(e->tab_ev[k]);
    }
    for (auto& ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : e->tev) cudaEventDestroy(ev);
    for (int c = 0; c < wcfe_engine::kXMax; ++c) {
        if (e->cstream[c]) {
            cudaStreamSynchronize(e->cstream[c]);
            cudaStreamDestroy(e->cstream[c]);
        }
        for (cudaEvent_t ev : {e->xin[c], e->xout[c], e->cdone[c]})
            if (ev) cudaEventDestroy(ev);
    }
    if (e->xprev) cudaEventDestroy(e->xprev);
    if (e->xstream) {
        cudaStreamSynchronize(e->xstream);
        cudaStreamDestroy(e->xstream);
    }
    cudaStreamDestroy(e->stream);
    delete e;
    return WCFE_OK;
}

int wcfe_engine_precision(const wcfe_engine* e) { return e ? e->prec : -1; }
uint64_t wcfe_engine_free_bytes(const wcfe_engine* e) {
    if (!e || !e->budget) return 0;
    return e->budget > e->used ? e->budget - e->used : 0;
}
uint64_t wcfe_cell_bytes(int32_t nv, int32_t nt) {
    size_t off[32];
    int32_t nb = (int32_t)(4 * std::sqrt((double)std::max(nv, 1)) + 16);
    size_t s = state_layout(nv, nt, nb, 3 * nb, nk1_of(nv, nt, 64), true, off);
    size_t p7[7];
    size_t p = patch_layout(nv / 64 + 2, (size_t)(1.6 * nt) + 64, 3 * (size_t)nt, (size_t)(0.6 * nv) + 64, p7);
    return (uint64_t)(s + p + rho_bytes(nv));
}
int wcfe_engine_sync(wcfe_engine* e) {
    xjoin(e);
    if (!e) return WCFE_ERR_ARG;
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_create(wcfe_engine* e, int32_t nv, int32_t nt, const int32_t* tri, const int32_t* vt_ptr,
                     const int32_t* vt_idx, const uint8_t* is_bnd, const wcfe_params* params, int32_t* cell_out) {
    xjoin(e);
    if (!e || !tri || !params || !cell_out || nv <= 0 || nt <= 0) return fail("bad argument", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    std::unique_ptr<Cell> c(new Cell());
    std::string err = build_topology(c->topo, nv, nt, tri, vt_ptr, vt_idx, is_bnd);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    c->prm = *params;
    int r = upload_cell_topology(e, c.get());
    if (!r) r = upload_cell_patches(e, c.get());
    if (r) {
        free_cell(e, c.get());
        return r;
    }
    c->id = e->next_id++;
    *cell_out = c->id;
    e->cells[c->id] = std::move(c);
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_cell_destroy(wcfe_engine* e, int32_t id) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    // drop substrate couplings that involve this cell
    std::vector<int32_t> users;
    for (auto& kv : e->cells)
        if (kv.second->couple_sub == id) users.push_back(kv.first);
    for (int32_t u : users) wcfe_cell_couple_substrate(e, u, -1, 0.0);
    if (c->couple_sub >= 0) wcfe_cell_couple_substrate(e, id, -1, 0.0);
    free_cell(e, c);
    e->cells.erase(id);
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_cell_set_params(wcfe_engine* e, int32_t id, const wcfe_params* p) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !p) return fail("bad argument", WCFE_ERR_ARG);
    c->prm = *p;
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_cell_set_topology(wcfe_engine* e, int32_t id, int32_t nv, int32_t nt, const int32_t* tri,
                           const int32_t* vt_ptr, const int32_t* vt_idx, const uint8_t* is_bnd) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !tri) return fail("bad argument", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    Topology T;
    std::string err = build_topology(T, nv, nt, tri, vt_ptr, vt_idx, is_bnd);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    c->topo = std::move(T);
    int r = upload_cell_topology(e, c);
    if (!r) r = upload_cell_patches(e, c);
    if (c->rho_dev) {
        void* p = c->rho_dev;
        size_t b = c->rho_size;
        dev_free(e, p, b);
        c->rho_dev = nullptr;
    }
    if (c->mu_dev) {
        void* p = c->mu_dev;
        size_t b = c->mu_size;
        dev_free(e, p, b);
        c->mu_dev = nullptr;
    }
    e->version++;
    invalidate_graph(e);
    return r;
}

int wcfe_cell_remesh(wcfe_engine* e, int32_t id, int32_t n_split, const int32_t* split_ab, int32_t nv_new,
                     const int32_t* keep, int32_t nt_new, const int32_t* tri, const int32_t* vt_ptr,
                     const int32_t* vt_idx, const uint8_t* is_bnd, const double* x_new) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    if (n_split < 0 || (n_split > 0 && !split_ab) || nv_new <= 0 || !keep || nt_new <= 0 || !tri || !x_new)
        return fail("bad argument", WCFE_ERR_ARG);
    if (c->couple_sub >= 0 || c->is_sub) return fail("remeshing a coupled cell or substrate is not supported", WCFE_ERR_STATE);
    const int32_t n_old = c->topo.nv;
    const int64_t M = (int64_t)n_old + n_split;
    if (M > INT32_MAX) return fail("too many vertices", WCFE_ERR_ARG);
    // El Topo's change list: split k appends vertex n_old + k from two earlier vertices; its
    // level is one more than theirs (old vertices: level 0)
    std::vector<int32_t> level((size_t)M, 0);
    int32_t max_level = 0;
    for (int32_t k = 0; k < n_split; ++k) {
        const int32_t a = split_ab[2 * k], b = split_ab[2 * k + 1];
        if (a < 0 || b < 0 || a >= n_old + k || b >= n_old + k) return fail("split endpoint out of range", WCFE_ERR_ARG);
        level[(size_t)n_old + k] = 1 + std::max(level[a], level[b]);
        max_level = std::max(max_level, level[(size_t)n_old + k]);
    }
    for (int32_t j = 0; j < nv_new; ++j)   // defrag_mesh keeps the survivors in order
        if (keep[j] < 0 || keep[j] >= M || (j && keep[j] <= keep[j - 1])) return fail("bad vertex map", WCFE_ERR_ARG);
    Topology T;
    std::string err = build_topology(T, nv_new, nt_new, tri, vt_ptr, vt_idx, is_bnd);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    const int mixed = e->prec == WCFE_PREC_MIXED ? 1 : 0;
    int r;
    if (mixed && (r = check_planar_ccw(x_new, nv_new, T.tri))) return r;
    CK(cudaSetDevice(e->device));
    // scratch: records [M][18], header, splits grouped by level, the map, the positions
    std::vector<int32_t> ks;
    std::vector<int32_t> lstart(max_level + 2, 0);
    for (int32_t k = 0; k < n_split; ++k) lstart[level[(size_t)n_old + k] + 1]++;
    for (int32_t l = 1; l <= max_level + 1; ++l) lstart[l] += lstart[l - 1];
    ks.resize(n_split);
    {
        std::vector<int32_t> fill(lstart.begin(), lstart.end() - 1);
        for (int32_t k = 0; k < n_split; ++k) ks[fill[level[(size_t)n_old + k]]++] = k;
    }
    size_t o = 0;
    auto put = [&](size_t bytes) { const size_t at = o; o = align_up(o + bytes); return at; };
    const size_t o_ext = put(sizeof(double) * 18 * (size_t)M), o_hdr = put(sizeof(unsigned long long) * 4);
    const size_t o_ab = put(sizeof(int2) * (size_t)std::max(n_split, 1)), o_ks = put(sizeof(int32_t) * std::max(n_split, 1));
    const size_t o_keep = put(sizeof(int32_t) * nv_new), o_x = put(sizeof(double) * 3 * (size_t)nv_new);
    void* scratch = nullptr;
    if ((r = dev_alloc(e, &scratch, o))) return r;
    size_t scratch_bytes = o;
    char* sb = (char*)scratch;
    double* ext = (double*)(sb + o_ext);
    unsigned long long* hdr = (unsigned long long*)(sb + o_hdr);
    if (n_split) {
        CK(cudaMemcpyAsync(sb + o_ab, split_ab, sizeof(int2) * n_split, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(sb + o_ks, ks.data(), sizeof(int32_t) * n_split, cudaMemcpyHostToDevice, e->stream));
    }
    CK(cudaMemcpyAsync(sb + o_keep, keep, sizeof(int32_t) * nv_new, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(sb + o_x, x_new, sizeof(double) * 3 * nv_new, cudaMemcpyHostToDevice, e->stream));
    // old state -> records, then the splits level by level (stream order keeps the old block
    // alive until these have run: its release below is stream-ordered)
    launch_remesh_pack(c->dev, mixed, c->rho_dev, ext, hdr, e->stream);
    for (int32_t l = 1; l <= max_level; ++l)
        launch_remesh_split(ext, n_old, (const int*)(sb + o_ks) + lstart[l], lstart[l + 1] - lstart[l],
                            (const int2*)(sb + o_ab), e->stream);
    CK(cudaGetLastError());
    const bool had_rho = c->rho_dev != nullptr;
    if (had_rho) {
        void* p = c->rho_dev;
        size_t b = c->rho_size;
        dev_free(e, p, b);
        c->rho_dev = nullptr;
    }
    if (c->mu_dev) {   // per-element moduli do not survive a change of elements: back to params.mu
        void* p = c->mu_dev;
        size_t b = c->mu_size;
        dev_free(e, p, b);
        c->mu_dev = nullptr;
    }
    c->topo = std::move(T);
    if ((r = upload_cell_topology(e, c)) || (r = upload_cell_patches(e, c))) {
        dev_free(e, scratch, scratch_bytes);
        return r;
    }
    if (had_rho) {
        void* p = nullptr;
        if ((r = dev_alloc(e, &p, rho_bytes(nv_new)))) {
            dev_free(e, scratch, scratch_bytes);
            return r;
        }
        c->rho_dev = (double*)p;
        c->rho_size = rho_bytes(nv_new);
    }
    launch_remesh_unpack(c->dev, mixed, ext, (const int*)(sb + o_keep), (const double*)(sb + o_x), c->rho_dev, hdr,
                         e->stream);
    CK(cudaGetLastError());
    dev_free(e, scratch, scratch_bytes);
    CK(cudaStreamSynchronize(e->stream));
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_cell_set_substrate(wcfe_engine* e, int32_t id, int32_t nv, int32_t nt, const int32_t* tri, const double* Xs,
                            const double* xs) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    if (nt <= 0 || !tri) {
        c->sub_nt = 0;
        c->sub_nv = 0;
    } else {
        if (!Xs || nv <= 0) return fail("substrate positions missing", WCFE_ERR_ARG);
        for (int64_t k = 0; k < 3 * (int64_t)nt; ++k)
            if (tri[k] < 0 || tri[k] >= nv) return fail("substrate index out of range", WCFE_ERR_TOPOLOGY);
        c->sub_nv = nv;
        c->sub_nt = nt;
        c->sub_tri.assign(tri, tri + 3 * (size_t)nt);
        c->sub_X.assign(Xs, Xs + 3 * (size_t)nv);
        c->sub_x.assign(xs ? xs : Xs, (xs ? xs : Xs) + 3 * (size_t)nv);
        c->sub_moving = std::memcmp(c->sub_X.data(), c->sub_x.data(), sizeof(double) * 3 * nv) != 0;
    }
    int r = upload_substrate(e, c);
    e->version++;
    invalidate_graph(e);
    return r;
}

int wcfe_cell_set_state(wcfe_engine* e, int32_t id, const double* x, const double* V, const double* A, const double* ea,
                        const double* cA, const double* cC, const double* fau) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    int par;
    int r = read_parity(e, c, &par);
    if (r) return r;
    const int n = c->topo.nv;
    CellDev& d = c->dev;
    if (x && e->prec == WCFE_PREC_MIXED && (r = check_planar_ccw(x, n, c->topo.tri))) return r;
    if (e->prec == WCFE_PREC_MIXED) {
        if (x && (r = put_ff(e, d.pos[par], x, n, FF_POS))) return r;
        if (V && (r = put_ff(e, d.vel, V, n, FF_VEC))) return r;
        if (A && (r = put_ff(e, d.acc, A, n, FF_ACC))) return r;
        if (fau && (r = put_ff(e, d.fau, fau, n, FF_VEC))) return r;
        // both strain buffers: the mixed step carries xz, yz (zero rates in the plane) unchanged
        if (ea && ((r = put_ff(e, d.ea[par], ea, n, FF_EA)) || (r = put_ff(e, d.ea[par ^ 1], ea, n, FF_EA)))) return r;
        if (cA && (r = put_ff(e, d.cA, cA, n, FF_SCALAR))) return r;
        if (cC && (r = put_ff(e, d.cC, cC, n, FF_SCALAR))) return r;
        return WCFE_OK;
    }
    if (x && (r = put3(e, d.pos[par], x, n))) return r;
    if (V && (r = put3(e, d.vel, V, n))) return r;
    if (A && (r = put3(e, d.acc, A, n))) return r;
    if (fau && (r = put3(e, d.fau, fau, n))) return r;
    if (ea) CK(cudaMemcpyAsync(d.ea[par], ea, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, e->stream));
    if (cA) CK(cudaMemcpyAsync(d.cA, cA, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
    if (cC) CK(cudaMemcpyAsync(d.cC, cC, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_get_state(wcfe_engine* e, int32_t id, double* x, double* V, double* A, double* ea, double* cA,
                        double* cC, double* fau) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    int par;
    int r = read_parity(e, c, &par);
    if (r) return r;
    const int n = c->topo.nv;
    CellDev& d = c->dev;
    if (e->prec == WCFE_PREC_MIXED) {
        if (x && (r = get_ff(e, x, d.pos[par], n, FF_POS))) return r;
        if (V && (r = get_ff(e, V, d.vel, n, FF_VEC))) return r;
        if (A && (r = get_ff(e, A, d.acc, n, FF_ACC))) return r;
        if (fau && (r = get_ff(e, fau, d.fau, n, FF_VEC))) return r;
        if (ea && (r = get_ff(e, ea, d.ea[par], n, FF_EA))) return r;
        if (cA && (r = get_ff(e, cA, d.cA, n, FF_SCALAR))) return r;
        if (cC && (r = get_ff(e, cC, d.cC, n, FF_SCALAR))) return r;
        return WCFE_OK;
    }
    if (x && (r = get3(e, x, d.pos[par], n))) return r;
    if (V && (r = get3(e, V, d.vel, n))) return r;
    if (A && (r = get3(e, A, d.acc, n))) return r;
    if (fau && (r = get3(e, fau, d.fau, n))) return r;
    if (ea) CK(cudaMemcpyAsync(ea, d.ea[par], sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, e->stream));
    if (cA) CK(cudaMemcpyAsync(cA, d.cA, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    if (cC) CK(cudaMemcpyAsync(cC, d.cC, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_set_step_budget(wcfe_engine* e, int32_t id, int32_t steps) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || steps < 0) return fail("bad argument", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    CK(cudaMemcpyAsync(c->dev.ctl + 3, &steps, sizeof(int32_t), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_get_step_budget(wcfe_engine* e, int32_t id, int32_t* steps) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !steps) return fail("bad argument", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    CK(cudaMemcpyAsync(steps, c->dev.ctl + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_set_clock(wcfe_engine* e, int32_t id, double t, uint64_t calls) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    unsigned long long ap = calls;
    CK(cudaMemcpyAsync(c->dev.clk, &t, sizeof(double), cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(c->dev.ap, &ap, sizeof ap, cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_get_clock(wcfe_engine* e, int32_t id, double* t, uint64_t* calls) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    double tt;
    unsigned long long ap;
    CK(cudaMemcpyAsync(&tt, c->dev.clk, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(&ap, c->dev.ap, sizeof ap, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    if (t) *t = tt;
    if (calls) *calls = ap;
    return WCFE_OK;
}

int wcfe_cell_status(wcfe_engine* e, int32_t id, uint32_t* status) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !status) return fail("bad argument", WCFE_ERR_ARG);
    CK(cudaMemcpyAsync(status, c->dev.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_sizes(wcfe_engine* e, int32_t id, int32_t* nv, int32_t* nt, int32_t* nb, int32_t* np) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    if (nv) *nv = c->topo.nv;
    if (nt) *nt = c->topo.nt;
    if (nb) *nb = c->topo.nb;
    if (np) *np = c->patches.np;
    return WCFE_OK;
}

// ---- drop-in pieces -------------------------------------------------------
int wcfe_cell_predict(wcfe_engine* e, int32_t id, double dt, double* x_pred, double* V_hlf) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED)
        return fail("the per-function entry points run on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e);
    if (r) return r;
    int ti = table_index(e, id);
    const int n = c->topo.nv;
    double* st = dev_stage(e, sizeof(double) * 6 * n);
    if (!st) return fail("staging allocation failed", WCFE_ERR_NOMEM);
    launch_predict(e->d_table, ti, dt, x_pred ? st : nullptr, V_hlf ? st + 3 * n : nullptr, n, e->stream);
    e->launches++;
    CK(cudaGetLastError());
    if (x_pred) CK(cudaMemcpyAsync(x_pred, st, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (V_hlf) CK(cudaMemcpyAsync(V_hlf, st + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_update_fa(wcfe_engine* e, int32_t id, double dt_real, const double* X, const double* x_new,
                        const double* X_s, const double* x_s) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !x_new) return fail("bad argument", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED)
        return fail("the per-function entry points run on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    if ((X_s || x_s) && c->sub_nt > 0) {
        bool changedX = X_s && std::memcmp(X_s, c->sub_X.data(), sizeof(double) * 3 * c->sub_nv) != 0;
        if (X_s) c->sub_X.assign(X_s, X_s + 3 * (size_t)c->sub_nv);
        if (x_s) c->sub_x.assign(x_s, x_s + 3 * (size_t)c->sub_nv);
        bool moving = std::memcmp(c->sub_X.data(), c->sub_x.data(), sizeof(double) * 3 * c->sub_nv) != 0;
        if (changedX) {
            c->sub_moving = moving;
            int r = upload_substrate(e, c);
            if (r) return r;
        } else {
            int r = put3(e, (double4*)c->dev.sub.x, c->sub_x.data(), c->sub_nv);
            if (r) return r;
            if (moving != c->sub_moving) {
                c->sub_moving = moving;
                c->dev.sub.moving = moving ? 1 : 0;
            }
        }
        e->version++;
        invalidate_graph(e);
    }
    int r = sync_tables(e);
    if (r) return r;
    int par;
    if ((r = read_parity(e, c, &par))) return r;
    const int n = c->topo.nv;
    if (X && (r = put3(e, c->dev.pos[par], X, n))) return r;
    if ((r = put3(e, c->dev.pos[par ^ 1], x_new, n))) return r;
    int ti = table_index(e, id), n1, n2;
    if ((r = one_cell_lists(e, c, ti, &n1, &n2))) return r;
    vphase(e, e->d_table, e->d_one, n1, dt_real, VP_UPDATE_FA | rec_flag(e), grid_for(e, n1, vertex_occupancy(e->vblock)),
           e->stream);
    e->launches++;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_update_forces(wcfe_engine* e, int32_t id, double dt, double dt_real, double t_tot) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED)
        return fail("the per-function entry points run on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e);
    if (r) return r;
    int ti = table_index(e, id), n1, n2;
    if ((r = one_cell_lists(e, c, ti, &n1, &n2))) return r;
    // area and centroid of the current positions (calculateAreaTot, UL:531), then the patch phase
    vphase(e, e->d_table, e->d_one, n1, dt_real, rec_flag(e), grid_for(e, n1, vertex_occupancy(e->vblock)), e->stream);
    size_t smem = patch_smem_bytes(e->prec, PP_STEP, e->patch_emax);
    launch_patch(e->prec, PP_STEP, e->d_table, e->d_one + n1, n2, e->patch_emax, dt, dt_real, ap_threshold(c->prm, dt_real),
                 t_tot, 1, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, e->patch_threads,
                 grid_for(e, n2, patch_occupancy(e->prec, e->patch_threads, smem)), e->stream);
    e->launches += 2;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_eval_residual(wcfe_engine* e, int32_t id, const double* X, const double* x_new, double dt_real,
                            const double centroid[3], double t_tot, double* Res, double* Res_ea, double* MM,
                            double* Res_Adif, double* Res_Cdif) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !X || !x_new || !centroid) return fail("bad argument", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED)
        return fail("the per-function entry points run on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e);
    if (r) return r;
    int par;
    if ((r = read_parity(e, c, &par))) return r;
    const int n = c->topo.nv;
    if ((r = put3(e, c->dev.pos[par], X, n))) return r;
    if ((r = put3(e, c->dev.pos[par ^ 1], x_new, n))) return r;
    double* st = dev_stage(e, sizeof(double) * (13 * (size_t)n + 4));
    if (!st) return fail("staging allocation failed", WCFE_ERR_NOMEM);
    double* dR = st;
    double* dE = dR + 3 * n;
    double* dM = dE + 6 * n;
    double* dA = dM + n;
    double* dC = dA + n;
    double* dcen = dC + n;
    CK(cudaMemcpyAsync(dcen, centroid, 3 * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    int ti = table_index(e, id), n1, n2;
    if ((r = one_cell_lists(e, c, ti, &n1, &n2))) return r;
    // partials for area (unused by the residual itself but keeps the kernel's prologue well defined)
    launch_vertex_phase(e->d_table, e->d_one, n1, dt_real, 0, grid_for(e, n1, vertex_occupancy(e->vblock)), e->vblock,
                        e->stream);
    size_t smem = patch_smem_bytes(e->prec, PP_RESIDUAL, e->patch_emax);
    launch_patch(e->prec, PP_RESIDUAL, e->d_table, e->d_one + n1, n2, e->patch_emax, dt_real, dt_real, 0.0, t_tot, 0, dcen,
                 dR, dE, dM, dA, dC, e->patch_threads, grid_for(e, n2, patch_occupancy(e->prec, e->patch_threads, smem)),
                 e->stream);
    e->launches += 2;
    CK(cudaGetLastError());
    if (Res) CK(cudaMemcpyAsync(Res, dR, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (Res_ea) CK(cudaMemcpyAsync(Res_ea, dE, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, e->stream));
    if (MM) CK(cudaMemcpyAsync(MM, dM, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    if (Res_Adif) CK(cudaMemcpyAsync(Res_Adif, dA, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    if (Res_Cdif) CK(cudaMemcpyAsync(Res_Cdif, dC, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

int wcfe_cell_eval_forces(wcfe_engine* e, int32_t id, const double* x, double dt_real, double* F_FA, double* F_AP,
                          double* F_bend, double* F_area, double area4[4]) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !x) return fail("bad argument", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED)
        return fail("the per-function entry points run on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e);
    if (r) return r;
    int par;
    if ((r = read_parity(e, c, &par))) return r;
    const int n = c->topo.nv;
    // the element pass reads X too: use x for both so the residual part is defined
    if ((r = put3(e, c->dev.pos[par], x, n))) return r;
    if ((r = put3(e, c->dev.pos[par ^ 1], x, n))) return r;
    double* st = dev_stage(e, sizeof(double) * 12 * (size_t)n);
    if (!st) return fail("staging allocation failed", WCFE_ERR_NOMEM);
    int ti = table_index(e, id), n1, n2;
    if ((r = one_cell_lists(e, c, ti, &n1, &n2))) return r;
    launch_vertex_phase(e->d_table, e->d_one, n1, dt_real, 0, grid_for(e, n1, vertex_occupancy(e->vblock)), e->vblock,
                        e->stream);
    size_t smem = patch_smem_bytes(e->prec, PP_FORCES, e->patch_emax);
    launch_patch(e->prec, PP_FORCES, e->d_table, e->d_one + n1, n2, e->patch_emax, dt_real, dt_real,
                 ap_threshold(c->prm, dt_real), std::numeric_limits<double>::quiet_NaN(), 0, nullptr, st, st + 3 * n,
                 st + 6 * n, st + 9 * n, nullptr, e->patch_threads,
                 grid_for(e, n2, patch_occupancy(e->prec, e->patch_threads, smem)), e->stream);
    e->launches += 2;
    CK(cudaGetLastError());
    if (F_FA) CK(cudaMemcpyAsync(F_FA, st, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (F_AP) CK(cudaMemcpyAsync(F_AP, st + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (F_bend) CK(cudaMemcpyAsync(F_bend, st + 6 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (F_area) CK(cudaMemcpyAsync(F_area, st + 9 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (area4) {
        std::vector<double> part(4 * (size_t)c->dev.nk1);
        CK(cudaMemcpyAsync(part.data(), c->dev.k1_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        double s[4] = {0, 0, 0, 0};
        for (int b = 0; b < c->dev.nk1; ++b)
            for (int q = 0; q < 4; ++q) s[q] += part[4 * b + q];
        area4[0] = s[0];
        for (int q = 1; q < 4; ++q) area4[q] = s[q] / s[0];
    }
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

// ---- batched stepping -------------------------------------------------------
int wcfe_engine_step(wcfe_engine* e, int32_t nsteps, double dt) {
    xjoin(e);
    if (!e || nsteps < 0 || !(dt > 0)) return fail("bad argument", WCFE_ERR_ARG);
    if (e->cells.empty() || nsteps == 0) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e, dt);
    if (r) return r;
    const int n1 = (int)e->k1.size(), n2 = (int)e->k2.size();
    if (e->use_graphs && !e->timing) {
        // a fused run replays its middle steps from the graph; the first and last launch directly
        const bool fz = step_kind(e, 0, nsteps) != STEP_FULL;
        const int gkind = fz ? STEP_MID : STEP_FULL;
        const int ngraph = fz ? nsteps - 2 : nsteps;
        if (fz && (r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, STEP_FIRST))) return r;
        const int chunk = std::min(ngraph, 8);
        const int per_step = gkind == STEP_MID ? 1 : 2;
        if (chunk > 0 && (!e->graph.exec || e->graph.dt != dt || e->graph.version != e->version ||
                          e->graph.steps != chunk || e->graph.kind != gkind)) {
            invalidate_graph(e);
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
            for (int s = 0; s < chunk; ++s) {
                r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, gkind);
                if (r) {
                    cudaStreamEndCapture(e->stream, &g);
                    return r;
                }
            }
            e->launches -= (uint64_t)per_step * chunk;  // counted at replay
            CK(cudaStreamEndCapture(e->stream, &g));
            CK(cudaGraphInstantiate(&e->graph.exec, g, 0));
            cudaGraphDestroy(g);
            e->graph.dt = dt;
            e->graph.version = e->version;
            e->graph.steps = chunk;
            e->graph.kind = gkind;
        }
        int done = 0;
        while (chunk > 0 && done + chunk <= ngraph) {
            CK(cudaGraphLaunch(e->graph.exec, e->stream));
            e->launches += (uint64_t)per_step * chunk;
            done += chunk;
        }
        for (; done < ngraph; ++done)
            if ((r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, gkind))) return r;
        if (fz && (r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, STEP_LAST))) return r;
        return WCFE_OK;
    }
    if (e->timing) {
        // events for every step, recorded on the engine stream without host synchronisation;
        // read back by wcfe_engine_last_timing / wcfe_engine_step_times
        while (e->tev.size() < 3 * (size_t)nsteps) {
            cudaEvent_t ev;
            CK(cudaEventCreate(&ev));
            e->tev.push_back(ev);
        }
        e->timed_steps = 0;
    }
    for (int s = 0; s < nsteps; ++s)
        if ((r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, step_kind(e, s, nsteps)))) return r;
    if (e->timing) {
        CK(cudaEventSynchronize(e->tev[3 * (size_t)e->timed_steps - 1]));
        e->ms_v = e->ms_p = 0;
        e->step_ms.assign(e->timed_steps, 0.f);
        for (int s = 0; s < e->timed_steps; ++s) {
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, e->tev[3 * s], e->tev[3 * s + 1]);
            cudaEventElapsedTime(&b, e->tev[3 * s + 1], e->tev[3 * s + 2]);
            e->ms_v += a;
            e->ms_p += b;
            e->step_ms[s] = a + b;
        }
        cudaEventElapsedTime(&e->ms_span, e->tev[0], e->tev[3 * (size_t)e->timed_steps - 1]);
    }
    return WCFE_OK;
}

int wcfe_engine_step_cells(wcfe_engine* e, const int32_t* ids, int32_t ncells, int32_t nsteps, double dt) {
    xjoin(e);
    if (!e || !ids || ncells <= 0 || nsteps < 0 || !(dt > 0)) return fail("bad argument", WCFE_ERR_ARG);
    if (e && std::any_of(e->cells.begin(), e->cells.end(), [](const auto& kv) { return kv.second->is_sub; }))
        return fail("coupled substrates step only through wcfe_engine_step", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e, dt);
    if (r) return r;
    std::vector<WorkItem> w1, w2;
    for (int i = 0; i < ncells; ++i) {
        Cell* c = find(e, ids[i]);
        if (!c) return fail("unknown cell", WCFE_ERR_ARG);
        int ti = table_index(e, ids[i]);
        for (int b = 0; b < c->dev.nk1; ++b) w1.push_back({ti, b});
        for (int p = 0; p < c->dev.np; ++p) w2.push_back({ti, p});
    }
    std::vector<WorkItem> w(w1);
    w.insert(w.end(), w2.begin(), w2.end());
    if ((r = ensure_dev(&e->d_one, &e->d_one_cap, w.size()))) return r;
    CK(cudaMemcpyAsync(e->d_one, w.data(), sizeof(WorkItem) * w.size(), cudaMemcpyHostToDevice, e->stream));
    for (int s = 0; s < nsteps; ++s)
        if ((r = enqueue_step(e, e->d_one, (int)w1.size(), e->d_one + w1.size(), (int)w2.size(), dt))) return r;
    return WCFE_OK;
}

int wcfe_engine_set_graphs(wcfe_engine* e, int32_t enable) {
    xjoin(e);
    if (!e) return WCFE_ERR_ARG;
    e->use_graphs = enable != 0;
    if (!e->use_graphs) invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_set_shape(wcfe_engine* e, int32_t threads, int32_t emax) {
    xjoin(e);
    if (!e) return WCFE_ERR_ARG;
    if (threads == 0) threads = e->patch_threads;
    if (emax == 0) emax = e->patch_emax;
    if (threads % 32 || threads < 32 || threads > 512 || emax < 32 || emax > 4096) return fail("bad shape", WCFE_ERR_ARG);
    if (e->prec == WCFE_PREC_MIXED && threads > 128) return fail("mixed patch kernels run at most 128 threads", WCFE_ERR_ARG);
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device);
    if (patch_smem_bytes(e->prec, PP_RESIDUAL, emax) + 1024 > (size_t)max_optin) return fail("shape exceeds shared memory", WCFE_ERR_LIMIT);
    CK(cudaStreamSynchronize(e->stream));
    e->patch_threads = threads;
    if (emax != e->patch_emax) {
        e->patch_emax = emax;
        for (auto& kv : e->cells) {
            int r = upload_cell_patches(e, kv.second.get());
            if (r) return r;
        }
        e->version++;
    }
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_set_lu(wcfe_engine* e, int32_t block, int32_t kind) {
    xjoin(e);
    if (!e || !lu_block_ok(block, kind)) return fail("bad argument", WCFE_ERR_ARG);
    e->lu_nb = block;
    e->lu_kind = kind;
    return WCFE_OK;
}

int wcfe_engine_set_lu_reuse(wcfe_engine* e, int32_t reuse) {
    xjoin(e);
    if (!e || reuse < 0 || reuse > 1) return fail("bad argument", WCFE_ERR_ARG);
    e->lu_reuse = reuse;
    return WCFE_OK;
}

int wcfe_engine_set_patch_kernel(wcfe_engine* e, int32_t kind) {
    xjoin(e);
    if (!e || kind < 0 || kind > 4) return fail("bad argument", WCFE_ERR_ARG);
    if (kind >= 2 && e->patch_threads != 128) return fail("register-capped patch kernels run 128 threads", WCFE_ERR_ARG);
    e->patch_kernel = kind;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_set_element_precision(wcfe_engine* e, int32_t mode) {
    xjoin(e);
    if (!e || mode < 0 || mode > 1) return fail("bad argument", WCFE_ERR_ARG);
    if (mode == 1 && e->prec != WCFE_PREC_MIXED) return fail("the float-float element is the mixed form's", WCFE_ERR_ARG);
    e->element_ff = mode == 1;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_get_element_precision(const wcfe_engine* e, int32_t* mode) {
    if (!e || !mode) return fail("bad argument", WCFE_ERR_ARG);
    *mode = e->element_ff ? 1 : 0;
    return WCFE_OK;
}

int wcfe_engine_set_fused(wcfe_engine* e, int32_t enable) {
    xjoin(e);
    if (!e || enable < 0 || enable > 1) return fail("bad argument", WCFE_ERR_ARG);
    e->fused = enable != 0;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_get_fused(const wcfe_engine* e) { return e ? (fused_ok(e) ? 1 : 0) : -1; }

int wcfe_engine_set_vertex_kernel(wcfe_engine* e, int32_t kind) {
    xjoin(e);
    if (!e || kind < 0 || kind > 3) return fail("bad argument", WCFE_ERR_ARG);
    e->vertex_kind = kind;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_engine_get_kernels(const wcfe_engine* e, int32_t* patch_kind, int32_t* vertex_kind) {
    if (!e) return WCFE_ERR_ARG;
    if (patch_kind) *patch_kind = e->patch_kernel;
    if (vertex_kind) *vertex_kind = e->vertex_kind;
    return WCFE_OK;
}

int wcfe_engine_get_shape(const wcfe_engine* e, int32_t* threads, int32_t* emax) {
    if (!e) return WCFE_ERR_ARG;
    if (threads) *threads = e->patch_threads;
    if (emax) *emax = e->patch_emax;
    return WCFE_OK;
}

int wcfe_engine_set_timing(wcfe_engine* e, int32_t enable) {
    xjoin(e);
    if (!e) return WCFE_ERR_ARG;
    e->timing = enable != 0;
    return WCFE_OK;
}

int64_t wcfe_engine_step_times(wcfe_engine* e, float* out, int64_t cap, float* span_ms) {
    if (!e) return -1;
    for (int64_t i = 0; out && i < cap && i < (int64_t)e->step_ms.size(); ++i) out[i] = e->step_ms[i];
    if (span_ms) *span_ms = e->ms_span;
    return (int64_t)e->step_ms.size();
}

int wcfe_engine_last_timing(wcfe_engine* e, float* ms_v, float* ms_p) {
    xjoin(e);
    if (!e) return WCFE_ERR_ARG;
    if (ms_v) *ms_v = e->ms_v;
    if (ms_p) *ms_p = e->ms_p;
    return WCFE_OK;
}

uint64_t wcfe_engine_launches(const wcfe_engine* e) { return e ? e->launches : 0; }
void* wcfe_engine_stream(const wcfe_engine* e) { return e ? (void*)e->stream : nullptr; }

int wcfe_debug_topology(int32_t nv, int32_t nt, const int32_t* tri, const int32_t* vt_ptr, const int32_t* vt_idx,
                        const uint8_t* is_bnd, int32_t emax, int32_t* nb_out, int32_t* bnd_rank, int32_t* bnd_cptr,
                        int32_t* bnd_cand, int32_t cand_cap, int32_t* np_out, int32_t* patch, int32_t patch_cap,
                        int32_t* patch_elems, int32_t elems_cap, uint16_t* vc_code) {
    Topology T;
    std::string err = build_topology(T, nv, nt, tri, vt_ptr, vt_idx, is_bnd);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    Patches P;
    err = build_patches(P, T, emax);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    if ((int64_t)T.bnd_cand.size() > cand_cap || (int64_t)P.patch.size() > patch_cap ||
        (int64_t)P.elems.size() > elems_cap)
        return fail("output capacity too small", WCFE_ERR_LIMIT);
    if (nb_out) *nb_out = T.nb;
    if (bnd_rank) std::memcpy(bnd_rank, T.bnd_rank.data(), sizeof(int32_t) * nv);
    if (bnd_cptr) std::memcpy(bnd_cptr, T.bnd_cptr.data(), sizeof(int32_t) * T.bnd_cptr.size());
    if (bnd_cand && !T.bnd_cand.empty()) std::memcpy(bnd_cand, T.bnd_cand.data(), sizeof(int32_t) * T.bnd_cand.size());
    if (np_out) *np_out = P.np;
    if (patch) std::memcpy(patch, P.patch.data(), sizeof(int32_t) * P.patch.size());
    if (patch_elems) std::memcpy(patch_elems, P.elems.data(), sizeof(int32_t) * P.elems.size());
    if (vc_code) std::memcpy(vc_code, P.vc_code.data(), sizeof(uint16_t) * P.vc_code.size());
    return WCFE_OK;
}

int wcfe_debug_patch_staging(int32_t nv, int32_t nt, const int32_t* tri, int32_t emax, int32_t* np_out, int32_t* xinfo,
                             int32_t xinfo_cap, int32_t* halo, int32_t halo_cap, uint16_t* loc, int32_t loc_cap,
                             int32_t* maxima_out) {
    Topology T;
    std::string err = build_topology(T, nv, nt, tri, nullptr, nullptr, nullptr);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    Patches P;
    err = build_patches(P, T, emax);
    if (!err.empty()) return fail(err, WCFE_ERR_TOPOLOGY);
    if ((int64_t)P.xinfo.size() > xinfo_cap || (int64_t)P.halo.size() > halo_cap || (int64_t)P.loc.size() > loc_cap)
        return fail("output capacity too small", WCFE_ERR_LIMIT);
    if (np_out) *np_out = P.np;
    if (xinfo) std::memcpy(xinfo, P.xinfo.data(), sizeof(int32_t) * P.xinfo.size());
    if (halo && !P.halo.empty()) std::memcpy(halo, P.halo.data(), sizeof(int32_t) * P.halo.size());
    if (loc) std::memcpy(loc, P.loc.data(), sizeof(uint16_t) * P.loc.size());
    if (maxima_out) {
        maxima_out[0] = P.max_ne;
        maxima_out[1] = P.max_nvp;
        maxima_out[2] = P.max_nh;
        maxima_out[3] = P.max_nc;
    }
    return WCFE_OK;
}

int64_t wcfe_engine_total_vertices(wcfe_engine* e) {
    if (!e) return -1;
    if (sync_tables(e)) return -1;
    return e->total_nv;
}

namespace {
// The exchange split into up to xchunks groups of consecutive cells (table order, which
// is also the order of the work lists and of the packed exchange array), balanced by
// vertex count; rebuilt only when the tables or the group count change.
const std::vector<XChunk>& exchange_chunks(wcfe_engine* e) {
    if (e->xch_version == e->table_version && e->xch_count == e->xchunks) return e->xch;
    std::vector<XChunk>& out = e->xch;
    out.clear();
    const int ncell = (int)e->table.size();
    const int nch = std::max(1, std::min(e->xchunks, ncell));
    size_t k1 = 0, k2 = 0, v = 0;
    int cell = 0;
    for (int c = 0; c < nch && cell < ncell; ++c) {
        XChunk x{(int)k1, (int)k1, (int)k2, (int)k2, v, v};
        const size_t target = (size_t)e->total_nv * (c + 1) / nch;
        while (cell < ncell && (x.v_hi < target || x.v_hi == x.v_lo || c == nch - 1)) {
            x.v_hi += (size_t)e->table[cell].nv;
            while (k1 < e->k1.size() && e->k1[k1].cell == cell) ++k1;
            while (k2 < e->k2.size() && e->k2[k2].cell == cell) ++k2;
            ++cell;
        }
        x.k1_hi = (int)k1;
        x.k2_hi = (int)k2;
        v = x.v_hi;
        out.push_back(x);
    }
    e->xch_version = e->table_version;
    e->xch_count = e->xchunks;
    return out;
}

// Start of an exchange call: the tables (re-uploaded on the main stream once every group
// stream has finished with them, if they changed) and whether the group streams are
// already ordered after everything the main stream holds.  They are when the last work
// on this engine was an exchange call; otherwise each group stream, and the copy stream,
// waits for the main stream.
int exchange_begin(wcfe_engine* e, double dt, bool* ordered) {
    const bool stale = (dt > 0 && dt != e->table_dt) || e->table_version != e->version;
    if (stale) xjoin(e);
    int r = sync_tables(e, dt);
    if (r) return r;
    if ((r = ensure_dev(&e->d_xchg, &e->d_xchg_cap, 3 * (size_t)e->total_nv))) return r;
    *ordered = e->xpending;
    if (!e->xpending) {
        CK(cudaEventRecord(e->xprev, e->stream));
        CK(cudaStreamWaitEvent(e->xstream, e->xprev, 0));
        for (int c = 0; c < wcfe_engine::kXMax; ++c) CK(cudaStreamWaitEvent(e->cstream[c], e->xprev, 0));
    }
    return WCFE_OK;
}
}  // namespace

int wcfe_engine_predict(wcfe_engine* e, double dt, double* x_pred) {
    if (e && std::any_of(e->cells.begin(), e->cells.end(), [](const auto& kv) { return kv.second->is_sub; }))
        return fail("coupled substrates step only through wcfe_engine_step", WCFE_ERR_STATE);
    if (!e || !x_pred || !(dt > 0)) return fail("bad argument", WCFE_ERR_ARG);
    if (e->cells.empty()) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    bool ordered = false;
    int r = exchange_begin(e, dt, &ordered);
    if (r) return r;
    // group by group on the group's own stream (after that group's update): the predicted
    // positions of a group copy back while the other groups still update or predict
    const std::vector<XChunk>& ch = exchange_chunks(e);
    for (size_t c = 0; c < ch.size(); ++c) {
        const XChunk& x = ch[c];
        const int n1 = x.k1_hi - x.k1_lo;
        if (n1 > 0)
            vphase(e, e->d_table, e->d_k1 + x.k1_lo, n1, dt, VP_PREDICT | VP_EXPORT | VP_NOAREA,
                   grid_for(e, n1, vertex_occupancy(e->vblock)), e->cstream[c], nullptr, e->d_xchg);
        e->launches++;
        CK(cudaEventRecord(e->xout[c], e->cstream[c]));
        CK(cudaEventRecord(e->cdone[c], e->cstream[c]));
        CK(cudaStreamWaitEvent(e->xstream, e->xout[c], 0));
        if (x.v_hi > x.v_lo)
            CK(cudaMemcpyAsync(x_pred + 3 * x.v_lo, e->d_xchg + 3 * x.v_lo, sizeof(double) * 3 * (x.v_hi - x.v_lo),
                               cudaMemcpyDeviceToHost, e->xstream));
    }
    e->xpending = true;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->xstream));
    return WCFE_OK;
}

int wcfe_engine_update(wcfe_engine* e, double dt, double dt_real, const double* x_new) {
    if (e && std::any_of(e->cells.begin(), e->cells.end(), [](const auto& kv) { return kv.second->is_sub; }))
        return fail("coupled substrates step only through wcfe_engine_step", WCFE_ERR_STATE);
    if (!e || !x_new || !(dt > 0) || !(dt_real > 0)) return fail("bad argument", WCFE_ERR_ARG);
    if (e->cells.empty()) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    bool ordered = false;
    int r = exchange_begin(e, dt_real, &ordered);
    if (r) return r;
    const std::vector<XChunk>& ch = exchange_chunks(e);
    // a group's copy overwrites its part of the staging array only after that group's
    // earlier work has read it
    if (ordered)
        for (size_t c = 0; c < ch.size(); ++c) CK(cudaStreamWaitEvent(e->xstream, e->cdone[c], 0));
    // each group's phases start on its own stream as soon as its positions are in; the copy
    // and the phases of a group are issued together, so the first group's work is queued
    // before the host issues the later groups' copies
    for (size_t c = 0; c < ch.size(); ++c) {
        const XChunk& x = ch[c];
        if (x.v_hi > x.v_lo)
            CK(cudaMemcpyAsync(e->d_xchg + 3 * x.v_lo, x_new + 3 * x.v_lo, sizeof(double) * 3 * (x.v_hi - x.v_lo),
                               cudaMemcpyHostToDevice, e->xstream));
        CK(cudaEventRecord(e->xin[c], e->xstream));
        cudaStream_t st = e->cstream[c];
        CK(cudaStreamWaitEvent(st, e->xin[c], 0));
        const int n1 = x.k1_hi - x.k1_lo, n2 = x.k2_hi - x.k2_lo;
        if (n1 > 0)
            vphase(e, e->d_table, e->d_k1 + x.k1_lo, n1, dt_real, VP_IMPORT | VP_UPDATE_FA | rec_flag(e),
                   grid_for(e, n1, vertex_occupancy(e->vblock)), st, e->d_xchg, nullptr);
        if (n2 > 0)
            patch_step(e, e->d_k2 + x.k2_lo, n2, dt, dt_real, std::numeric_limits<double>::quiet_NaN(),
                       std::numeric_limits<double>::quiet_NaN(), 1, st);
        CK(cudaEventRecord(e->cdone[c], st));
        e->launches += 2;
    }
    e->xpending = true;
    CK(cudaGetLastError());
    return WCFE_OK;
}

int wcfe_engine_set_exchange_groups(wcfe_engine* e, int32_t groups) {
    if (!e || groups < 1 || groups > wcfe_engine::kXMax) return fail("bad argument", WCFE_ERR_ARG);
    xjoin(e);
    e->xchunks = groups;
    return WCFE_OK;
}

// ---------------------------------------------------------------------------- implicit (Newton) step
namespace {
struct NewtonPlan {
    void* block = nullptr;
    size_t bytes = 0;
    std::vector<NewtonCell> cells;   // host copy
    NewtonCell* d_cells = nullptr;
    int* d_ident = nullptr;          // slot s <-> table index s
    unsigned int* d_tickets = nullptr;
    double* norms = nullptr;         // [nslots][8]
    LuMaps* d_maps = nullptr;        // [nslots] TMA descriptors of J and Ut
    int* d_prefix = nullptr;         // per-launch tile prefix sums of the LU's trailing updates
    int* d_sweep = nullptr;          // the triangular sweeps' block counter and abort word
    int sweep_epoch = 0;             // the last epoch the cells' sweep flags were given
    cudaEvent_t sev[2] = {nullptr, nullptr};   // around each triangular solve (statistics)
    cudaStream_t side = nullptr;                // the LU's second stream (row-panel transposes)
    cudaEvent_t lev[2] = {nullptr, nullptr};    // ordering between the two LU streams
    double *res = nullptr, *rea = nullptr, *mm = nullptr, *f4 = nullptr, *fext = nullptr;
    int max_n = 0;
};

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// one device block for every cell of the table: packed residual and force arrays, per cell
// J, element tangents and vectors
int newton_plan(wcfe_engine* e, NewtonPlan& P) {
    const int ns = (int)e->order.size();
    const size_t NV = (size_t)e->total_nv;
    size_t o = 0;
    auto put = [&](size_t bytes) { const size_t at = o; o = al256(o + bytes); return at; };
    const size_t o_res = put(sizeof(double) * 3 * NV), o_rea = put(sizeof(double) * 6 * NV), o_mm = put(sizeof(double) * NV);
    const size_t o_f4 = put(sizeof(double) * 12 * NV), o_fext = put(sizeof(double) * 3 * NV);
    const size_t o_norm = put(sizeof(double) * 8 * ns), o_nc = put(sizeof(NewtonCell) * ns);
    const size_t o_id = put(sizeof(int) * ns), o_tk = put(sizeof(unsigned int) * ns);
    const size_t o_maps = put(sizeof(LuMaps) * ns);
    struct Off { size_t J, Ut, Dinv, At, Ke, diag, G, dx, d, r, z, zt, flags; int n, ld; };
    std::vector<Off> off(ns);
    P.max_n = 0;
    for (int sl = 0; sl < ns; ++sl) {
        const Cell* c = e->cells.at(e->order[sl]).get();
        const int n = c->topo.nv, m = 2 * n, ld = (m + 3) & ~3;
        Off& f = off[sl];
        f.n = n;
        f.ld = ld;
        f.J = put(sizeof(float) * (size_t)m * ld);
        f.Ut = put(sizeof(float) * (size_t)m * e->lu_nb);   // Ut row length: the outer block width
        f.Dinv = put(sizeof(float) * 2 * 64 * 64 * (size_t)((m + 63) / 64));
        f.zt = put(sizeof(float) * m);
        f.At = put(sizeof(float) * 64 * (size_t)m);
        f.Ke = put(sizeof(float) * 36 * (size_t)c->topo.nt);
        f.diag = put(sizeof(double) * n);
        f.G = put(sizeof(double) * m);
        f.dx = put(sizeof(double) * m);
        f.d = put(sizeof(double) * m);
        f.r = put(sizeof(double) * m);
        f.z = put(sizeof(float) * m);
        f.flags = put(sizeof(int) * (size_t)((m + 63) / 64));
        P.max_n = std::max(P.max_n, n);
    }
    const size_t o_pref = put(sizeof(int) * lu_prefix_capacity(ns, 2 * P.max_n));
    const size_t o_sweep = put(sizeof(int) * 2);
    int r = dev_alloc(e, &P.block, o);
    if (r) return r;
    P.bytes = o;
    char* b = (char*)P.block;
    CK(cudaMemsetAsync(b, 0, o, e->stream));
    P.res = (double*)(b + o_res);
    P.rea = (double*)(b + o_rea);
    P.mm = (double*)(b + o_mm);
    P.f4 = (double*)(b + o_f4);
    P.fext = (double*)(b + o_fext);
    P.norms = (double*)(b + o_norm);
    P.d_cells = (NewtonCell*)(b + o_nc);
    P.d_ident = (int*)(b + o_id);
    P.d_tickets = (unsigned int*)(b + o_tk);
    P.d_maps = (LuMaps*)(b + o_maps);
    P.d_prefix = (int*)(b + o_pref);
    P.d_sweep = (int*)(b + o_sweep);
    P.sweep_epoch = 0;   // the block is zeroed: every flag is below the first epoch
    P.cells.resize(ns);
    std::vector<int> ident(ns);
    for (int sl = 0; sl < ns; ++sl) {
        const Cell* c = e->cells.at(e->order[sl]).get();
        const size_t h = (size_t)c->dev.hoff;
        const Off& f = off[sl];
        NewtonCell& N = P.cells[sl];
        N.J = (float*)(b + f.J);
        N.Ut = (float*)(b + f.Ut);
        N.utld = e->lu_nb;
        N.pad2 = 0;
        N.Dinv = (float*)(b + f.Dinv);
        N.zt = (float*)(b + f.zt);
        N.At = (float*)(b + f.At);
        N.Ke = (float*)(b + f.Ke);
        N.diag = (double*)(b + f.diag);
        N.G = (double*)(b + f.G);
        N.dx = (double*)(b + f.dx);
        N.d = (double*)(b + f.d);
        N.r = (double*)(b + f.r);
        N.z = (float*)(b + f.z);
        N.flags = (int*)(b + f.flags);
        N.Fext = P.fext + 3 * h;
        N.Res = P.res + 3 * h;
        N.MM = P.mm + h;
        N.norms = P.norms + 8 * (size_t)sl;
        N.n = f.n;
        N.ld = f.ld;
        N.active = 1;
        N.pad = 0;
        ident[sl] = sl;
    }
    std::vector<LuMaps> maps(ns);
    if (encode_lu_maps(P.cells.data(), ns, maps.data())) return fail("tensor map encoding failed", WCFE_ERR_CUDA);
    CK(cudaMemcpyAsync(P.d_maps, maps.data(), sizeof(LuMaps) * ns, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(P.d_ident, ident.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(P.d_cells, P.cells.data(), sizeof(NewtonCell) * ns, cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (auto& ev : P.sev) CK(cudaEventCreate(&ev));
    for (auto& ev : P.lev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&P.side, cudaStreamNonBlocking));
    return WCFE_OK;
}

void newton_free(wcfe_engine* e, NewtonPlan& P) {
    for (auto& ev : P.sev)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : P.lev)
        if (ev) cudaEventDestroy(ev);
    if (P.side) {
        cudaStreamSynchronize(P.side);
        cudaStreamDestroy(P.side);
    }
    if (P.block) {
        cudaStreamSynchronize(e->stream);
        dev_free(e, P.block, P.bytes);
    }
}

void release_newton_plan(wcfe_engine* e) {
    if (!e->newton_plan) return;
    NewtonPlan* P = static_cast<NewtonPlan*>(e->newton_plan);
    newton_free(e, *P);
    delete P;
    e->newton_plan = nullptr;
}

// the engine's implicit-step workspace: kept between calls, rebuilt when the cells or the
// LU's outer block changed (a workspace for 512 cells of up to 4,000 vertices is tens of
// GB: allocating and clearing it per call took longer than a factorisation)
int kept_newton_plan(wcfe_engine* e, NewtonPlan** out) {
    if (e->newton_plan && (e->newton_version != e->version || e->newton_nb != e->lu_nb)) release_newton_plan(e);
    if (!e->newton_plan) {
        NewtonPlan* P = new NewtonPlan;
        int r = newton_plan(e, *P);
        if (r) {
            newton_free(e, *P);
            delete P;
            return r;
        }
        e->newton_plan = P;
        e->newton_version = e->version;
        e->newton_nb = e->lu_nb;
    }
    *out = static_cast<NewtonPlan*>(e->newton_plan);
    return WCFE_OK;
}

int newton_upload_active(wcfe_engine* e, NewtonPlan& P) {
    CK(cudaMemcpyAsync(P.d_cells, P.cells.data(), sizeof(NewtonCell) * P.cells.size(), cudaMemcpyHostToDevice,
                       e->stream));
    return WCFE_OK;
}

int newton_read_norms(wcfe_engine* e, NewtonPlan& P, std::vector<double>& h) {
    h.resize(8 * P.cells.size());
    CK(cudaMemcpyAsync(h.data(), P.norms, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return WCFE_OK;
}

// the FP64 membrane residual, lumped mass and strain residual at the iterate (packed arrays)
void newton_membrane(wcfe_engine* e, NewtonPlan& P, double dt) {
    const int n2 = (int)e->k2.size();
    const size_t smem = patch_smem_bytes(WCFE_PREC_FP64, PP_RESIDUAL, e->patch_emax);
    launch_patch(WCFE_PREC_FP64, PP_RESIDUAL, e->d_table, e->d_k2, n2, e->patch_emax, dt, dt, 0.0,
                 std::numeric_limits<double>::quiet_NaN(), 0, nullptr, P.res, P.rea, P.mm, nullptr, nullptr,
                 e->patch_threads, grid_for(e, n2, patch_occupancy(WCFE_PREC_FP64, e->patch_threads, smem)), e->stream, 1);
}

int newton_step(wcfe_engine* e, NewtonPlan& P, double dt, double rtol, int max_newton, wcfe_newton_stats* st) {
    const int ns = (int)P.cells.size();
    const int n1 = (int)e->k1.size(), n2 = (int)e->k2.size();
    const size_t NV = (size_t)e->total_nv;
    std::vector<double> hn;
    // A1 + A5: predicted positions, bond kinetics, area and centroid of the predicted positions
    vphase(e, e->d_table, e->d_k1, n1, dt, VP_PREDICT | VP_UPDATE_FA, grid_for(e, n1, vertex_occupancy(e->vblock)),
           e->stream);
    // external forces at the predicted positions
    {
        const size_t smem = patch_smem_bytes(WCFE_PREC_FP64, PP_FORCES, e->patch_emax);
        launch_patch(WCFE_PREC_FP64, PP_FORCES, e->d_table, e->d_k2, n2, e->patch_emax, dt, dt,
                     std::numeric_limits<double>::quiet_NaN(), std::numeric_limits<double>::quiet_NaN(), 0, nullptr,
                     P.f4, P.f4 + 3 * NV, P.f4 + 6 * NV, P.f4 + 9 * NV, nullptr, e->patch_threads,
                     grid_for(e, n2, patch_occupancy(WCFE_PREC_FP64, e->patch_threads, smem)), e->stream, 1);
        launch_sum4(P.f4, P.f4 + 3 * NV, P.f4 + 6 * NV, P.f4 + 9 * NV, P.fext, 3 * NV, e->stream);
    }
    for (auto& N : P.cells) N.active = 1;
    std::vector<double> gprev(ns, INFINITY);
    int r = newton_upload_active(e, P);
    if (r) return r;
    launch_newton_apply(e->d_table, P.d_cells, P.d_ident, ns, P.max_n, 1, e->stream);   // d = x_pred - X
    e->launches += 3;
    for (int it = 0;; ++it) {
        newton_membrane(e, P, dt);
        // |G| and the force scale (entries 0, 1) are rebuilt; entries 4, 5 hold the last update
        launch_norms_clear(P.norms, ns, 0, 4, e->stream);
        launch_newton_residual(e->d_table, P.d_cells, P.d_ident, ns, P.max_n, dt, e->stream);
        e->launches += 2;
        if ((r = newton_read_norms(e, P, hn))) return r;
        int nact = 0;
        for (int sl = 0; sl < ns; ++sl) {
            const double g = hn[8 * sl], f = std::max(hn[8 * sl + 1], 1e-300);
            const bool bad = !std::isfinite(g) || hn[8 * sl + 3] != 0.0;
            // converged: the residual at rtol of the force scale, or the iteration has reached the
            // residual's rounding floor, about |dRes/dx| ulp(x) (the positions are FP64): the last
            // correction was at the rounding level of the displacement, or Newton, which otherwise
            // converges quadratically here, stopped reducing |G| (below 1e-6 of the scale)
            const bool floor = it > 0 && (hn[8 * sl + 4] <= 1e-13 * hn[8 * sl + 5] ||
                                          (it > 1 && g > 0.25 * gprev[sl] && g <= 1e-6 * f));
            const bool conv = g <= rtol * f || floor;
            if (floor && !(g <= rtol * f) && st && P.cells[sl].active) st->floor_exits += 1;
            gprev[sl] = g;
            P.cells[sl].active = (!bad && !conv && it < max_newton) ? 1 : 0;
            nact += P.cells[sl].active;
            if (!P.cells[sl].active) {   // final for this step
                if (st) {
                    st->max_rel_residual = std::max(st->max_rel_residual, std::isfinite(g) ? g / f : INFINITY);
                    if (!conv) st->unconverged += 1;
                }
                if (bad) {   // non-finite residual or zero pivot: flag the cell (status bit 16)
                    Cell* c = e->cells.at(e->order[sl]).get();
                    uint32_t s0 = 0;
                    CK(cudaMemcpyAsync(&s0, c->dev.status, sizeof s0, cudaMemcpyDeviceToHost, e->stream));
                    CK(cudaStreamSynchronize(e->stream));
                    s0 |= 16u;
                    CK(cudaMemcpyAsync(c->dev.status, &s0, sizeof s0, cudaMemcpyHostToDevice, e->stream));
                }
            }
        }
        if (!nact) break;
        if ((r = newton_upload_active(e, P))) return r;
        if (st) st->newton_iters += 1;
        // tangent; the dense LU on the first iteration of the step (or every iteration without
        // reuse).  Later iterations keep the factors: the FP64 refinement against the current
        // sparse tangent still gives the Newton correction to 1e-10, in a pass or two more.
        const bool factor = it == 0 || !e->lu_reuse;
        if (factor) launch_dense_clear(P.d_cells, ns, P.max_n, e->stream);
        launch_newton_tangent(e->d_table, P.d_cells, P.d_ident, e->d_k2, n2, e->patch_emax, dt, factor ? 1 : 0,
                              e->stream);
        if (factor) {
        if (st) CK(cudaEventRecord(e->ev[0], e->stream));
        if (const char* k = launch_newton_lu(P.d_cells, P.cells.data(), ns, 2 * P.max_n, P.d_maps, P.d_prefix,
                                             e->lu_nb, e->lu_kind, e->stream, P.side, P.lev))
            return fail(std::string("launch failed: ") + k + lu_attr_note(), WCFE_ERR_CUDA);
        if (st) {
            CK(cudaEventRecord(e->ev[1], e->stream));
            for (const auto& N : P.cells)
                if (N.active) st->lu_gflop += (2.0 / 3.0) * std::pow(2.0 * N.n, 3) * 1e-9;
        }
        }
        // J dx = -G, refined in FP64
        launch_newton_clear(P.d_cells, ns, P.max_n, e->stream);
        launch_newton_refine(e->d_table, P.d_cells, P.d_ident, e->d_k2, n2, 0, e->stream);
        int q = 0;
        double final_ratio = 0.0;
        for (; q < 16; ++q) {
            if (st) CK(cudaEventRecord(P.sev[0], e->stream));
            launch_newton_solve(P.d_cells, ns, P.max_n, P.d_sweep, &P.sweep_epoch, e->stream);
            if (st) CK(cudaEventRecord(P.sev[1], e->stream));
            launch_norms_clear(P.norms, ns, 2, 1, e->stream);   // |r| only (G's norm is kept on the host)
            launch_newton_refine(e->d_table, P.d_cells, P.d_ident, e->d_k2, n2, 1, e->stream);
            launch_newton_accumulate(P.d_cells, ns, P.max_n, e->stream);
            e->launches += 3;
            std::vector<double> hr;
            if ((r = newton_read_norms(e, P, hr))) return r;
            if (st) {
                float sv = 0.0f;
                CK(cudaEventElapsedTime(&sv, P.sev[0], P.sev[1]));   // the stream was synchronised
                st->solve_ms += sv;
            }
            bool done = true;
            final_ratio = 0.0;
            for (int sl = 0; sl < ns; ++sl) {
                if (!P.cells[sl].active) continue;
                const double ratio = hr[8 * sl + 2] / std::max(hn[8 * sl], 1e-300);
                if (!(ratio <= 1e-10)) done = false;
                final_ratio = std::max(final_ratio, ratio);
            }
            if (done) break;
        }
        if (st) {
            float lu = 0.0f;
            if (factor) CK(cudaEventElapsedTime(&lu, e->ev[0], e->ev[1]));   // both passed: the stream was synchronised
            st->lu_ms += lu;
            st->max_refine_iters = std::max(st->max_refine_iters, q + 1);
            st->max_refine_rel_residual = std::max(st->max_refine_rel_residual, final_ratio);
        }
        launch_norms_clear(P.norms, ns, 4, 2, e->stream);
        launch_newton_apply(e->d_table, P.d_cells, P.d_ident, ns, P.max_n, 0, e->stream);
        e->launches += 4 + 3 * ((2 * P.max_n + 63) / 64);
        CK(cudaGetLastError());
    }
    // finish at the converged x: strain residual, V, A, ea; advance parity, clock, AP counter
    newton_membrane(e, P, dt);
    launch_newton_finish(e->d_table, P.d_cells, P.d_ident, ns, P.max_n, P.rea, dt, P.d_tickets, e->stream);
    e->launches += 2;
    CK(cudaGetLastError());
    return WCFE_OK;
}
}  // namespace

int wcfe_engine_step_implicit(wcfe_engine* e, int32_t nsteps, double dt, double newton_rtol, int32_t max_newton,
                              wcfe_newton_stats* stats) {
    xjoin(e);
    if (!e || nsteps < 0 || !(dt > 0) || !(newton_rtol > 0) || max_newton < 1) return fail("bad argument", WCFE_ERR_ARG);
    if (e->prec != WCFE_PREC_FP64)
        return fail("the implicit step runs on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    if (e && std::any_of(e->cells.begin(), e->cells.end(), [](const auto& kv) { return kv.second->is_sub; }))
        return fail("coupled substrates step only through wcfe_engine_step", WCFE_ERR_STATE);
    if (std::any_of(e->cells.begin(), e->cells.end(), [](const auto& kv) { return kv.second->prm.protrude_v != 0.0; }))
        return fail("the implicit step has no protrusion driver (params.protrude_v must be 0)", WCFE_ERR_ARG);
    if (stats) std::memset(stats, 0, sizeof *stats);
    if (e->cells.empty() || nsteps == 0) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e, dt);
    if (r) return r;
    NewtonPlan* P = nullptr;
    if ((r = kept_newton_plan(e, &P))) return r;
    for (int s = 0; s < nsteps && !r; ++s) r = newton_step(e, *P, dt, newton_rtol, max_newton, stats);
    if (!r) {
        cudaError_t ce = cudaStreamSynchronize(e->stream);
        if (ce != cudaSuccess) r = fail(std::string("CUDA: ") + cudaGetErrorString(ce), WCFE_ERR_CUDA);
    }
    if (r) release_newton_plan(e);   // rebuilt on the next call
    return r;
}

int wcfe_cell_newton_tangent(wcfe_engine* e, int32_t id, double dt, const double* x, float* J_out, double* diag_out) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !x || !J_out || !(dt > 0)) return fail("bad argument", WCFE_ERR_ARG);
    if (e->prec != WCFE_PREC_FP64)
        return fail("the implicit step runs on an FP64 engine (WCFE_PREC_FP64)", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    int r = sync_tables(e, dt);
    if (r) return r;
    int par;
    if ((r = read_parity(e, c, &par))) return r;
    const int n = c->topo.nv;
    if ((r = put3(e, c->dev.pos[par ^ 1], x, n))) return r;
    NewtonPlan P;
    if ((r = newton_plan(e, P))) return r;
    const int ti = table_index(e, id);
    int n1, n2;
    if ((r = one_cell_lists(e, c, ti, &n1, &n2)) == 0) {
        // area and centroid of x, then the lumped mass, then J
        launch_vertex_phase(e->d_table, e->d_one, n1, dt, 0, grid_for(e, n1, vertex_occupancy(e->vblock)), e->vblock,
                            e->stream);
        const size_t smem = patch_smem_bytes(WCFE_PREC_FP64, PP_RESIDUAL, e->patch_emax);
        launch_patch(WCFE_PREC_FP64, PP_RESIDUAL, e->d_table, e->d_one + n1, n2, e->patch_emax, dt, dt, 0.0,
                     std::numeric_limits<double>::quiet_NaN(), 0, nullptr, P.res, P.rea, P.mm, nullptr, nullptr,
                     e->patch_threads, grid_for(e, n2, patch_occupancy(WCFE_PREC_FP64, e->patch_threads, smem)),
                     e->stream, 1);
        launch_newton_tangent(e->d_table, P.d_cells, P.d_ident, e->d_one + n1, n2, e->patch_emax, dt, 1, e->stream);
        const NewtonCell& N = P.cells[ti];
        CK(cudaMemcpy2DAsync(J_out, sizeof(float) * 2 * n, N.J, sizeof(float) * N.ld, sizeof(float) * 2 * n, 2 * n,
                             cudaMemcpyDeviceToHost, e->stream));
        if (diag_out) CK(cudaMemcpyAsync(diag_out, N.diag, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        e->launches += 3;
    }
    newton_free(e, P);
    return r;
}

int wcfe_debug_lu_schedule(int32_t m, int32_t block, int32_t* ops, int32_t cap, int32_t* nops) {
    if (m <= 0 || !nops || !lu_block_ok(block, 0) || cap < 0 || (cap > 0 && !ops))
        return fail("bad argument", WCFE_ERR_ARG);
    const std::vector<LuOp> sched = lu_schedule(m, block);
    *nops = (int32_t)sched.size();
    if (!ops) return WCFE_OK;
    if ((int64_t)sched.size() * 14 > (int64_t)cap) return fail("ops buffer too small", WCFE_ERR_LIMIT);
    for (const LuOp& o : sched) {
        const LuUpdateArgs& a = o.a;
        const int32_t rec[14] = {o.type,    o.k0,      a.nreg,    a.ka,      a.kb,      a.K,       a.rlo[0],
                                 a.rhi[0],  a.clo[0],  a.chi[0],  a.rlo[1],  a.rhi[1],  a.clo[1],  a.chi[1]};
        std::memcpy(ops, rec, sizeof rec);
        ops += 14;
    }
    return WCFE_OK;
}

int wcfe_debug_lu_solve(int32_t m, const float* A, const double* b, float* x) {
    return wcfe_debug_lu_solve_with(m, A, b, x, 512, 0);
}

namespace {
int debug_lu_solve_impl(int32_t m, const float* A, const double* b, float* x, int32_t block, int32_t kind,
                        int withhold, long long wait_limit);
}  // namespace

int wcfe_debug_lu_solve_with(int32_t m, const float* A, const double* b, float* x, int32_t block, int32_t kind) {
    return debug_lu_solve_impl(m, A, b, x, block, kind, -1, 0);
}

int wcfe_debug_trsv_withheld(int32_t m, const float* A, const double* b, float* x, int32_t withhold,
                             int64_t wait_clocks) {
    if (withhold < 0 || wait_clocks <= 0) return fail("bad argument", WCFE_ERR_ARG);
    return debug_lu_solve_impl(m, A, b, x, 1024, 0, withhold, wait_clocks);
}

namespace {
int debug_lu_solve_impl(int32_t m, const float* A, const double* b, float* x, int32_t block, int32_t kind,
                        int withhold, long long wait_limit) {
    if (m <= 0 || (m & 1) || !A || !b || !x) return fail("bad argument", WCFE_ERR_ARG);
    if (!lu_block_ok(block, kind)) return fail("bad argument", WCFE_ERR_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail("no CUDA device", WCFE_ERR_NODEVICE);
    }
    int max_optin = 0, sms = 0;
    CK(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    CK(configure_newton((size_t)max_optin, sms));
    const int ld = (m + 3) & ~3;
    const size_t npref = lu_prefix_capacity(1, m);
    const size_t ndinv = 2 * 64 * 64 * (size_t)((m + 63) / 64);
    const size_t bytes = sizeof(float) * (size_t)m * ld + sizeof(float) * (size_t)m * block + sizeof(double) * m +
                         2 * sizeof(float) * m + sizeof(float) * ndinv + sizeof(float) * 64 * (size_t)m +
                         sizeof(double) * 8 + sizeof(NewtonCell) + sizeof(LuMaps) + sizeof(int) * npref +
                         sizeof(int) * ((size_t)(m + 63) / 64 + 2) + 13 * 256;
    char* blk = nullptr;
    CK(cudaMalloc(&blk, bytes));
    size_t o = 0;
    auto take = [&](size_t n) { char* p = blk + o; o = (o + n + 255) & ~(size_t)255; return p; };
    NewtonCell N{};
    N.J = (float*)take(sizeof(float) * (size_t)m * ld);
    N.Ut = (float*)take(sizeof(float) * (size_t)m * block);
    N.utld = block;
    N.r = (double*)take(sizeof(double) * m);
    N.z = (float*)take(sizeof(float) * m);
    N.zt = (float*)take(sizeof(float) * m);
    N.Dinv = (float*)take(sizeof(float) * ndinv);
    N.At = (float*)take(sizeof(float) * 64 * (size_t)m);
    N.norms = (double*)take(sizeof(double) * 8);
    N.flags = (int*)take(sizeof(int) * (size_t)((m + 63) / 64));
    int* d_sweep = (int*)take(sizeof(int) * 2);
    int epoch = 0;
    N.n = m / 2;
    N.ld = ld;
    N.active = 1;
    NewtonCell* d_nc = (NewtonCell*)take(sizeof(NewtonCell));
    LuMaps* d_maps = (LuMaps*)take(sizeof(LuMaps));
    int* d_pref = (int*)take(sizeof(int) * npref);
    LuMaps maps{};
    cudaError_t ce = encode_lu_maps(&N, 1, &maps) ? cudaErrorInvalidValue : cudaSuccess;
    if (ce == cudaSuccess) ce = cudaMemset(blk, 0, bytes);
    if (ce == cudaSuccess)
        ce = cudaMemcpy2D(N.J, sizeof(float) * ld, A, sizeof(float) * m, sizeof(float) * m, m, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(N.r, b, sizeof(double) * m, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_maps, &maps, sizeof maps, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_nc, &N, sizeof N, cudaMemcpyHostToDevice);
    const char* failed = nullptr;
    if (ce == cudaSuccess) {
        failed = launch_newton_lu(d_nc, &N, 1, m, d_maps, d_pref, block, kind, 0);
        launch_newton_solve(d_nc, 1, m / 2, d_sweep, &epoch, 0, withhold, wait_limit);
        if (!failed && cudaGetLastError() != cudaSuccess) failed = "triangular solves";
        ce = cudaDeviceSynchronize();
    }
    if (failed) {
        cudaFree(blk);
        return fail(std::string("launch failed: ") + failed + lu_attr_note(), WCFE_ERR_CUDA);
    }
    double flag = 0;
    if (ce == cudaSuccess) ce = cudaMemcpy(x, N.z, sizeof(float) * m, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(&flag, N.norms + 3, sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(blk);
    if (ce != cudaSuccess) return fail(std::string("CUDA: ") + cudaGetErrorString(ce), WCFE_ERR_CUDA);
    if (flag == 2.0) return fail("tensor-core update timed out", WCFE_ERR_CUDA);
    if (flag == 3.0) return fail("triangular sweep timed out", WCFE_ERR_CUDA);
    if (flag != 0.0) return fail("zero or non-finite pivot", WCFE_ERR_STATE);
    return WCFE_OK;
}
}  // namespace

int wcfe_cell_set_element_mu(wcfe_engine* e, int32_t id, const double* mu) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    const int nt = c->topo.nt;
    if (!mu) {
        if (c->mu_dev) {
            void* p = c->mu_dev;
            size_t b = c->mu_size;
            dev_free(e, p, b);
            c->mu_dev = nullptr;
        }
    } else {
        for (int t = 0; t < nt; ++t)
            if (!(mu[t] > 0) || !std::isfinite(mu[t])) return fail("shear moduli must be positive", WCFE_ERR_ARG);
        if (!c->mu_dev) {
            void* p = nullptr;
            int r = dev_alloc(e, &p, rho_bytes(nt));
            if (r) return r;
            c->mu_dev = (double*)p;
            c->mu_size = rho_bytes(nt);
        }
        if (e->prec == WCFE_PREC_MIXED) {
            std::vector<float> f(nt);
            for (int t = 0; t < nt; ++t) f[t] = (float)mu[t];
            CK(cudaMemcpyAsync(c->mu_dev, f.data(), sizeof(float) * nt, cudaMemcpyHostToDevice, e->stream));
        } else {
            CK(cudaMemcpyAsync(c->mu_dev, mu, sizeof(double) * nt, cudaMemcpyHostToDevice, e->stream));
        }
        CK(cudaStreamSynchronize(e->stream));
    }
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int wcfe_cell_couple_substrate(wcfe_engine* e, int32_t id, int32_t sub_id, double grid_margin) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    if (e->prec != WCFE_PREC_FP64) return fail("substrate coupling runs on an FP64 engine", WCFE_ERR_STATE);
    CK(cudaSetDevice(e->device));
    CK(cudaStreamSynchronize(e->stream));
    // undo a previous coupling of this cell
    if (c->couple_sub >= 0) {
        const int32_t old = c->couple_sub;
        c->couple_sub = -1;
        dev_free(e, c->cgrid_block, c->cgrid_bytes);
        std::memset(&c->dev.sub, 0, sizeof(SubDev));
        c->dev.has_sub = 0;
        bool still = false;
        for (auto& kv : e->cells) still = still || kv.second->couple_sub == old;
        auto it = e->cells.find(old);
        if (!still && it != e->cells.end()) {
            it->second->is_sub = false;
            dev_free(e, it->second->fext_block, it->second->fext_bytes);
        }
    }
    e->version++;
    invalidate_graph(e);
    if (sub_id < 0) return WCFE_OK;
    Cell* s = find(e, sub_id);
    if (!s || s == c) return fail("bad substrate cell", WCFE_ERR_ARG);
    if (c->is_sub || s->couple_sub >= 0) return fail("a substrate cell cannot be coupled to a substrate", WCFE_ERR_ARG);
    if (!(grid_margin >= 0)) return fail("bad grid margin", WCFE_ERR_ARG);
    // point-location grid over the substrate's current positions
    const int ns = s->topo.nv, nts = s->topo.nt;
    std::vector<double> xs(3 * (size_t)ns);
    int r = wcfe_cell_get_state(e, sub_id, xs.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (r) return r;
    build_subgrid(c->cgrid, ns, nts, s->topo.tri.data(), xs.data(), grid_margin);
    const SubGrid& G = c->cgrid;
    const size_t b0 = align_up(sizeof(int32_t) * G.cell_ptr.size());
    const size_t bytes = b0 + align_up(sizeof(int32_t) * std::max<size_t>(G.cell_tri.size(), 1));
    if ((r = dev_alloc(e, &c->cgrid_block, bytes))) return r;
    c->cgrid_bytes = bytes;
    char* b = (char*)c->cgrid_block;
    CK(cudaMemcpyAsync(b, G.cell_ptr.data(), sizeof(int32_t) * G.cell_ptr.size(), cudaMemcpyHostToDevice, e->stream));
    if (!G.cell_tri.empty())
        CK(cudaMemcpyAsync(b + b0, G.cell_tri.data(), sizeof(int32_t) * G.cell_tri.size(), cudaMemcpyHostToDevice,
                           e->stream));
    if (!s->fext_block) {
        if ((r = dev_alloc(e, &s->fext_block, sizeof(unsigned long long) * 4 * (size_t)ns))) return r;
        s->fext_bytes = sizeof(unsigned long long) * 4 * (size_t)ns;
        CK(cudaMemsetAsync(s->fext_block, 0, s->fext_bytes, e->stream));
    }
    CK(cudaStreamSynchronize(e->stream));
    SubDev& sd = c->dev.sub;
    std::memset(&sd, 0, sizeof sd);
    sd.nv = ns;
    sd.nt = nts;
    sd.tri = s->dev.tri;
    sd.cell_ptr = (const int32_t*)b;
    sd.cell_tri = (const int32_t*)(b + b0);
    sd.ox = G.ox;
    sd.oy = G.oy;
    sd.inv_h = G.inv_h;
    sd.gx = G.gx;
    sd.gy = G.gy;
    sd.moving = 1;
    c->dev.has_sub = 1;
    c->couple_sub = sub_id;
    s->is_sub = true;
    e->version++;
    return WCFE_OK;
}

int wcfe_cell_set_integrins(wcfe_engine* e, int32_t id, const double* rho) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    CK(cudaSetDevice(e->device));
    const int n = c->topo.nv;
    if (!rho) {
        if (c->rho_dev) {
            void* p = c->rho_dev;
            size_t b = c->rho_size;
            dev_free(e, p, b);
            c->rho_dev = nullptr;
        }
    } else {
        if (!c->rho_dev) {
            void* p = nullptr;
            int r = dev_alloc(e, &p, rho_bytes(n));
            if (r) return r;
            c->rho_dev = (double*)p;
            c->rho_size = rho_bytes(n);
        }
        if (e->prec == WCFE_PREC_MIXED) {   // FP32 densities
            std::vector<float> f(n);
            for (int v = 0; v < n; ++v) f[v] = (float)rho[v];
            CK(cudaMemcpyAsync(c->rho_dev, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice, e->stream));
        } else {
            CK(cudaMemcpyAsync(c->rho_dev, rho, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
        }
        CK(cudaStreamSynchronize(e->stream));
    }
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

// Autotuner: time every candidate (threads, emax) on the live cells.  The state
// is saved and restored around the trials so tuning does not advance the cells.
int wcfe_engine_autotune(wcfe_engine* e, double dt, int32_t reps) {
    xjoin(e);
    if (!e || !(dt > 0) || reps < 1) return fail("bad argument", WCFE_ERR_ARG);
    if (e->cells.empty()) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    // save all state blocks
    std::vector<std::pair<Cell*, void*>> saved;
    for (auto& kv : e->cells) {
        Cell* c = kv.second.get();
        void* copy = nullptr;
        CK(cudaMalloc(&copy, c->state_bytes));
        CK(cudaMemcpyAsync(copy, c->state_block, c->state_bytes, cudaMemcpyDeviceToDevice, e->stream));
        saved.push_back({c, copy});
    }
    const int threads_c[] = {32, 64, 128, 256};
    const int emax_c[] = {48, 64, 96, 128, 192, 256, 384, 512, 768};
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device);
    float best = 1e30f;
    int bt = e->patch_threads, be = e->patch_emax, bk = e->patch_kernel;
    bool was_timing = e->timing;
    e->timing = true;
    // mixed engines also try the staged patch kernel (its block shape is fixed; it uses emax)
    // and the plain kernel with register caps for 6, 7 and 8 CTAs of 128 threads per SM
    std::vector<int> kinds = {1};
    if (e->prec == WCFE_PREC_MIXED && !e->element_ff) kinds = {1, 2, 3, 4, 0};
    for (int kind : kinds) {
        e->patch_kernel = kind;
        for (int em : emax_c) {
            if (patch_smem_bytes(e->prec, PP_RESIDUAL, em) + 1024 > (size_t)max_optin) continue;
            for (int th : threads_c) {
                if (kind == 0 && th != threads_c[0]) continue;
                if (kind >= 2 && th != 128) continue;
                int r = wcfe_engine_set_shape(e, kind == 0 ? e->patch_threads : th, em);
                if (r) continue;
                wcfe_engine_step(e, 1, dt);  // warm
                r = wcfe_engine_step(e, reps, dt);
                if (r) continue;
                float t = e->ms_v + e->ms_p;
                if (t < best) { best = t; bt = e->patch_threads; be = em; bk = kind; }
                for (auto& s : saved)
                    CK(cudaMemcpyAsync(s.first->state_block, s.second, s.first->state_bytes, cudaMemcpyDeviceToDevice,
                                       e->stream));
            }
        }
    }
    e->patch_kernel = bk;
    int r = wcfe_engine_set_shape(e, bt, be);
    if (!r && e->prec == WCFE_PREC_MIXED) {   // the vertex phase's register cap, at the chosen patch shape
        float bestv = 1e30f;
        int bv = 0;
        for (int vk = 0; vk < 4; ++vk) {
            e->vertex_kind = vk;
            wcfe_engine_step(e, 1, dt);
            if (wcfe_engine_step(e, reps, dt)) continue;
            if (e->ms_v < bestv) { bestv = e->ms_v; bv = vk; }
            for (auto& s : saved)
                CK(cudaMemcpyAsync(s.first->state_block, s.second, s.first->state_bytes, cudaMemcpyDeviceToDevice,
                                   e->stream));
        }
        e->vertex_kind = bv;
    }
    e->timing = was_timing;
    for (auto& s : saved) {
        cudaMemcpyAsync(s.first->state_block, s.second, s.first->state_bytes, cudaMemcpyDeviceToDevice, e->stream);
    }
    CK(cudaStreamSynchronize(e->stream));
    for (auto& s : saved) cudaFree(s.second);
    e->tuned = true;
    return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------- frame output (wcfe_vtk.cu)
namespace wcfe {
int set_error(const char* msg, int code) {
    g_last_error = msg;
    return code;
}

int engine_device(wcfe_engine* e) { return e->device; }

int engine_frame_source(wcfe_engine* e, int32_t id, FrameSource* out) {
    xjoin(e);
    Cell* c = e ? find(e, id) : nullptr;
    if (!c || !out) return fail("unknown cell", WCFE_ERR_ARG);
    out->dev = c->dev;
    out->mixed = e->prec == WCFE_PREC_MIXED ? 1 : 0;
    out->nv = c->topo.nv;
    out->nt = c->topo.nt;
    out->tri = c->topo.tri;
    out->prm = c->prm;
    out->stream = e->stream;
    out->device = e->device;
    return WCFE_OK;
}
}  // namespace wcfe

// ---------------------------------------------------------------------------- serving (wcfe_server.cu)
namespace wcfe {
namespace {
std::string planar_ccw_error(const double* x, int n, const std::vector<int32_t>& T) {
    for (int v = 0; v < n; ++v)
        if (x[3 * v + 2] != 0.0) return "the mixed form needs a planar membrane (z = 0)";
    for (size_t t = 0; 3 * t < T.size(); ++t) {
        const double* a = x + 3 * T[3 * t];
        const double* b = x + 3 * T[3 * t + 1];
        const double* q = x + 3 * T[3 * t + 2];
        if ((b[0] - a[0]) * (q[1] - a[1]) - (b[1] - a[1]) * (q[0] - a[0]) <= 0)
            return "the mixed form needs counter-clockwise, non-degenerate triangles";
    }
    return "";
}

// the tables into the device buffers without a host synchronisation: device buffers grow in
// stream order, the host images go through one of two pinned buffers (reused once the copy
// made from it two refreshes ago has run)
int sync_tables_async(wcfe_engine* e, double dt) {
    if (dt > 0 && dt != e->table_dt) {
        e->table_dt = dt;
        e->version++;
        invalidate_graph(e);
    }
    if (e->table_version == e->version) return WCFE_OK;
    for (auto& kv : e->cells)
        if (kv.second->couple_sub >= 0 || kv.second->is_sub)
            return fail("a serving engine holds no coupled substrates", WCFE_ERR_STATE);
    int r = build_tables(e);
    if (r) return r;
    auto grow = [&](auto** p, size_t* cap, size_t n, size_t elem) -> int {
        if (n <= *cap) return WCFE_OK;
        const size_t c = std::max<size_t>(n, 2 * *cap);
        void* q = nullptr;
        if (cudaMallocAsync(&q, elem * c, e->stream) != cudaSuccess) {
            cudaGetLastError();
            return fail("cudaMallocAsync of a work list failed", WCFE_ERR_NOMEM);
        }
        if (*p) cudaFreeAsync(*p, e->stream);
        *p = static_cast<std::remove_reference_t<decltype(**p)>*>(q);
        *cap = c;
        return WCFE_OK;
    };
    if ((r = grow(&e->d_table, &e->d_table_cap, std::max<size_t>(e->table.size(), 1), sizeof(CellDev)))) return r;
    if ((r = grow(&e->d_k1, &e->d_k1_cap, std::max<size_t>(2 * e->k1.size(), 1), sizeof(WorkItem)))) return r;
    if ((r = grow(&e->d_k2, &e->d_k2_cap, std::max<size_t>(e->k2.size(), 1), sizeof(WorkItem)))) return r;
    const size_t b0 = sizeof(CellDev) * e->table.size(), b1 = 2 * sizeof(WorkItem) * e->k1.size(),
                 b2 = sizeof(WorkItem) * e->k2.size();
    const int k = e->tab_buf;
    e->tab_buf ^= 1;
    if (!e->tab_ev[k]) CK(cudaEventCreateWithFlags(&e->tab_ev[k], cudaEventDisableTiming));
    else CK(cudaEventSynchronize(e->tab_ev[k]));
    if (b0 + b1 + b2 > e->h_tab_cap[k]) {
        if (e->h_tab[k]) cudaFreeHost(e->h_tab[k]);
        e->h_tab[k] = nullptr;
        e->h_tab_cap[k] = 0;
        const size_t cap = 2 * (b0 + b1 + b2) + 4096;
        CK(cudaMallocHost(&e->h_tab[k], cap));
        e->h_tab_cap[k] = cap;
    }
    char* h = static_cast<char*>(e->h_tab[k]);
    std::memcpy(h, e->table.data(), b0);
    std::memcpy(h + b0, e->k1.data(), b1 / 2);
    std::memcpy(h + b0 + b1 / 2, e->k1a.data(), b1 / 2);
    std::memcpy(h + b0 + b1, e->k2.data(), b2);
    if (b0) CK(cudaMemcpyAsync(e->d_table, h, b0, cudaMemcpyHostToDevice, e->stream));
    if (b1) CK(cudaMemcpyAsync(e->d_k1, h + b0, b1, cudaMemcpyHostToDevice, e->stream));
    if (b2) CK(cudaMemcpyAsync(e->d_k2, h + b0 + b1, b2, cudaMemcpyHostToDevice, e->stream));
    CK(cudaEventRecord(e->tab_ev[k], e->stream));
    e->table_version = e->version;
    return WCFE_OK;
}
}  // namespace

std::string serving_prepare(const wcfe_engine* e, PreparedCell& pc, int32_t nv, int32_t nt, const int32_t* tri,
                            const double* x, const wcfe_params& prm, int32_t steps) {
    pc.mixed = e->prec == WCFE_PREC_MIXED;
    pc.prm = prm;
    pc.steps = steps;
    std::string err = build_topology(pc.topo, nv, nt, tri, nullptr, nullptr, nullptr);
    if (!err.empty()) return err;
    if (pc.mixed && !(err = planar_ccw_error(x, nv, pc.topo.tri)).empty()) return err;
    const Topology& T = pc.topo;
    if ((int64_t)T.bnd_out.size() > std::max<int64_t>(2 * (int64_t)T.nb, 1)) return "non-manifold boundary";
    err = build_patches(pc.patches, T, e->patch_emax);
    if (!err.empty()) return err;
    const Patches& P = pc.patches;
    pc.nk1 = nk1_of(T.nv, T.nt, e->vblock);
    pc.state_bytes = state_layout(T.nv, T.nt, T.nb, (int32_t)(T.bnd_cand.size() / 2), pc.nk1, pc.mixed, pc.soff);
    pc.patch_bytes = patch_layout(P.np, P.elems.size(), P.vc_code.size(), P.halo.size(), pc.poff);
    tri4_of(T, pc.tri4);
    bnd_vert_of(T, pc.bnd_vert);
    patch_tri_of(P, T, pc.patch_tri);
    ca_init_of(T.nv, pc.mixed, pc.ca);
    // positions: binary64 double4, or the mixed form's triple-float planes (hi float4 then lo float4)
    pc.pos.assign(4 * (size_t)nv, 0.0);
    if (!pc.mixed) {
        for (int v = 0; v < nv; ++v)
            for (int k = 0; k < 3; ++k) pc.pos[4 * (size_t)v + k] = x[3 * (size_t)v + k];
    } else {
        float* f = reinterpret_cast<float*>(pc.pos.data());
        const size_t N = (size_t)nv;
        for (size_t v = 0; v < N; ++v) {
            split_tf(x[3 * v], &f[4 * v + 0], &f[4 * (N + v) + 0], &f[4 * v + 3]);
            split_tf(x[3 * v + 1], &f[4 * v + 1], &f[4 * (N + v) + 1], &f[4 * (N + v) + 3]);
            split_ff(x[3 * v + 2], &f[4 * v + 2], &f[4 * (N + v) + 2]);
        }
    }
    return "";
}

int serving_admit(wcfe_engine* e, PreparedCell& pc, cudaStream_t st, cudaMemPool_t pool, int32_t* id) {
    CK(cudaSetDevice(e->device));
    std::unique_ptr<Cell> c(new Cell());
    c->topo = std::move(pc.topo);
    c->patches = std::move(pc.patches);
    c->prm = pc.prm;
    void* sb = nullptr;
    void* pb = nullptr;
    if (cudaMallocFromPoolAsync(&sb, pc.state_bytes, pool, st) != cudaSuccess ||
        cudaMallocFromPoolAsync(&pb, pc.patch_bytes, pool, st) != cudaSuccess) {
        cudaGetLastError();
        if (sb) cudaFreeAsync(sb, st);
        return fail("cudaMallocFromPoolAsync failed", WCFE_ERR_NOMEM);
    }
    c->state_block = sb;
    c->state_bytes = pc.state_bytes;
    c->patch_block = pb;
    c->patch_bytes = pc.patch_bytes;
    CK(cudaMemsetAsync(sb, 0, pc.state_bytes, st));
    CK(cudaMemsetAsync(pb, 0, pc.patch_bytes, st));
    bind_state(c.get(), (char*)sb, pc.soff, pc.nk1, e->vblock, pc.mixed);
    bind_patches(c.get(), (char*)pb, pc.poff);
    int r = upload_state_arrays(c.get(), st, pc.tri4, pc.bnd_vert, pc.ca);
    if (!r) r = upload_patch_arrays(c.get(), st, pc.patch_tri);
    if (!r && cudaMemcpyAsync(c->dev.pos[0], pc.pos.data(), sizeof(double) * pc.pos.size(), cudaMemcpyHostToDevice,
                              st) != cudaSuccess)
        r = fail("cudaMemcpyAsync of the start positions failed", WCFE_ERR_CUDA);
    if (!r && cudaMemcpyAsync(c->dev.ctl + 3, &pc.steps, sizeof(int32_t), cudaMemcpyHostToDevice, st) != cudaSuccess)
        r = fail("cudaMemcpyAsync of the step budget failed", WCFE_ERR_CUDA);
    if (r) {
        cudaFreeAsync(sb, st);
        cudaFreeAsync(pb, st);
        return r;
    }
    e->used += pc.state_bytes + pc.patch_bytes;
    c->id = e->next_id++;
    *id = c->id;
    e->cells[c->id] = std::move(c);
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

int serving_step(wcfe_engine* e, int32_t nsteps, double dt) {
    if (e->cells.empty() || nsteps <= 0) return WCFE_OK;
    CK(cudaSetDevice(e->device));
    int r = sync_tables_async(e, dt);
    if (r) return r;
    const int n1 = (int)e->k1.size(), n2 = (int)e->k2.size();
    for (int s = 0; s < nsteps; ++s)
        if ((r = enqueue_step(e, e->d_k1, n1, e->d_k2, n2, dt, step_kind(e, s, nsteps)))) return r;
    return WCFE_OK;
}

size_t serving_raw_bytes(int32_t nv) { return sizeof(double4) * (size_t)nv; }

int serving_retire(wcfe_engine* e, int32_t id, int parity, void* pinned_dst, size_t cap, size_t* bytes) {
    Cell* c = find(e, id);
    if (!c) return fail("unknown cell", WCFE_ERR_ARG);
    const size_t nb = serving_raw_bytes(c->topo.nv);
    if (nb > cap) return fail("result buffer too small", WCFE_ERR_ARG);
    CK(cudaMemcpyAsync(pinned_dst, c->dev.pos[parity & 1], nb, cudaMemcpyDeviceToHost, e->stream));
    *bytes = nb;
    free_cell(e, c);   // cudaFreeAsync on the engine stream: after the copy
    e->cells.erase(id);
    e->version++;
    invalidate_graph(e);
    return WCFE_OK;
}

void serving_decode_positions(const wcfe_engine* e, const void* raw, int32_t nv, double* x) {
    const size_t N = (size_t)nv;
    if (e->prec != WCFE_PREC_MIXED) {
        const double* d = static_cast<const double*>(raw);
        for (size_t v = 0; v < N; ++v)
            for (int k = 0; k < 3; ++k) x[3 * v + k] = d[4 * v + k];
        return;
    }
    const float* b = static_cast<const float*>(raw);   // hi float4 plane, then lo float4 plane
    for (size_t v = 0; v < N; ++v) {
        x[3 * v] = ((double)b[4 * v] + (double)b[4 * (N + v)]) + (double)b[4 * v + 3];
        x[3 * v + 1] = ((double)b[4 * v + 1] + (double)b[4 * (N + v) + 1]) + (double)b[4 * (N + v) + 3];
        x[3 * v + 2] = (double)b[4 * v + 2] + (double)b[4 * (N + v) + 2];
    }
}

cudaStream_t engine_stream(const wcfe_engine* e) { return e->stream; }
uint64_t engine_budget(const wcfe_engine* e) { return e->budget; }
uint64_t engine_used(const wcfe_engine* e) { return e->used; }
}  // namespace wcfe
