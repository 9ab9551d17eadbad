/*
 * wcfe.h — C ABI of the GB300 (sm_103a) per-step mechanics engine for the
 * wholeCellFE 2-D cell-adhesion model.
 *
 * Everything crosses this boundary as plain pointers and sizes.  Host arrays
 * use the reference's own memory order so a caller can pass the storage of a
 * std::vector<Vec3d> (3 contiguous doubles per vertex) without repacking:
 *
 *   positions / velocities / accelerations / bond vectors : double[n][3]
 *   Euler-Almansi strain (Voigt xx, yy, zz, xy, xz, yz)     : double[n][6]
 *   concentrations c_A, c_C                                  : double[n]
 *   triangles                                                : int32[t][3]
 *   vertex -> triangle map (CSR, in the mesh's own order)    : int32[n+1], int32[3t]
 *
 * Every entry point returns an int status (WCFE_OK == 0).  No C++ exception
 * crosses the ABI.  An engine works on one device with its own CUDA streams (one
 * main stream; the exchange path adds a copy stream and group streams that every
 * other call waits for); calls on one engine are not re-entrant (the reference is
 * single threaded too).
 *
 * Reference interfaces replaced (file:line inside dredremontes/wholeCellFE,
 * variant directory wholeCellFE_kMD unless stated):
 *   driverVelocities_Explicit      cellBP/UL_growth_explicit.cpp:103-124 (+ predict cellBP/main.cpp:227-231)
 *   updateFA (full)                cellBP/UL_growth_explicit.cpp:2026-2174 (k1: wholeCellFE_k1/cellBP/UL_growth_explicit.cpp:2005-2090)
 *   updateForces_Explicit (cell)   cellBP/UL_growth_explicit.cpp:508-630
 *   updateForces_Explicit (subs)   cellBP/UL_growth_explicit.cpp:429-504
 *   calculateRes / evalElementRe   cellBP/UL_growth_explicit.cpp:632-928 (subs 931-1176)
 *   calculateForce_FA              cellBP/UL_growth_explicit.cpp:1198-1303
 *   calculateForce_FA_subs         cellBP/UL_growth_explicit.cpp:1305-1475
 *   calculateForce_AP              cellBP/UL_growth_explicit.cpp:1477-1568
 *   calculateBendingForce2D        cellBP/UL_growth_explicit.cpp:1571-1660
 *   calculateAreaTot               cellBP/UL_growth_explicit.cpp:1662-1688
 *   calculateAreaConstraintForce   cellBP/UL_growth_explicit.cpp:1691-1784
 * The reference declares these ad hoc in cellBP/main.cpp:69-87 and has no header.
 */
#ifndef WCFE_H
#define WCFE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WCFE_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    WCFE_OK = 0,
    WCFE_ERR_ARG = 1,        /* bad argument (null pointer, size, unknown id) */
    WCFE_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    WCFE_ERR_NOMEM = 3,      /* device allocation failed */
    WCFE_ERR_TOPOLOGY = 4,   /* mesh cannot be processed (e.g. a one-ring too large for a patch) */
    WCFE_ERR_STATE = 5,      /* a cell's state holds NaN/Inf after a step (see wcfe_cell_status) */
    WCFE_ERR_BUDGET = 6,     /* request does not fit the engine's HBM budget */
    WCFE_ERR_LIMIT = 8,      /* size beyond a documented maximum */
    WCFE_ERR_NODEVICE = 9    /* no CUDA device visible */
};

/* ---- integrin force laws ------------------------------------------------ */
enum {
    WCFE_LAW_LINEAR = 0,     /* f = k D (L0 = 0: wholeCellFE_k1 / wholeCellFE_k31); with a rest length
                                L0 > 0 the bond is slack below it: f = k max(D - L0, 0) */
    WCFE_LAW_MD_TABLE = 1,   /* piecewise-linear MD fit; wholeCellFE_kMD UL:1203-1214 */
    WCFE_LAW_POLY = 2        /* tangent stiffness k0 (1 + (e/x0)^2): f = k0 (e + e^3/(3 x0^2)) for
                                e = D - L0 > 0, slack (0) below */
};

/* ---- arithmetic forms --------------------------------------------------- */
enum {
    WCFE_PREC_FP64 = 0,      /* element assembly and update in FP64 (the plain form) */
    WCFE_PREC_MIXED = 1      /* element assembly and forces in FP32 (increment form); the state and
                                the update in extended FP32 formats: positions triple-float (about
                                72 bits, exact for binary64 input), velocity, strain, bond state
                                float-float (about 48 bits); planar cells (z = 0) only */
};

/* Reference variants for wcfe_params_default. */
enum { WCFE_VARIANT_KMD = 0, WCFE_VARIANT_K1 = 1, WCFE_VARIANT_K31 = 2 };

/*
 * Per-cell physical constants.  The reference hard-codes every one of these in
 * UL_growth_explicit.cpp; wcfe_params_default fills the reference values.
 * Units: um, pN, s (stress pN/um^2 = Pa).
 */
typedef struct wcfe_params {
    /* membrane (evalElementRe, UL:710-928) */
    double mu;            /* shear modulus, 1000 (cell, UL:724) */
    double thick;         /* thickness, 1 (UL:768) */
    double thetag_dot;    /* growth rate, 0 (UL:714) */
    double kappa;         /* active-stress anisotropy, 0.5 (UL:872) */
    double tact_rate;     /* active stress ramp 200 Pa/s ... (UL:744-757) */
    double tact_t1;       /* ... until t = 2 s ... */
    double tact_max;      /* ... then 400 Pa */
    double D_A, D_C;      /* diffusion coefficients 1, 1e-10 (UL:920-921); only the diagnostic residual uses them */
    /* integrins (calculateForce_FA UL:1198-1303, updateFA UL:2026-2174) */
    int32_t force_law;    /* WCFE_LAW_* */
    int32_t linear_norm2d;/* 1: Bell force of the linear law uses the in-plane norm (k1 UL:2077) */
    double k_lin;         /* linear stiffness, pN/um (1000 = 1 pN/nm) */
    double rest_len;      /* spring rest length, um (0 in the reference); a bond shorter than it
                             carries no force (tension only), so that a fresh bond of zero length,
                             whose direction is rounding noise, pushes nothing */
    double poly_k0;       /* WCFE_LAW_POLY stiffness at zero extension, pN/um */
    double poly_x0;       /* WCFE_LAW_POLY stiffening length, um */
    double rho_i_max;     /* integrin density 100 /um^2 (UL:1218) */
    double k_on, ka, kb, Fa, Fb;   /* Bell model 1, 0.004, 10, 15, 15 (UL:2139-2143) */
    /* boundary (UL:1477-1784) */
    double k_bend;        /* 20 (UL:1653) */
    double k_area;        /* 1 (UL:1776) */
    double area0;         /* 10*10*3.1416 (UL:1777) */
    double ap_rate;       /* actin polymerisation rate 10 1/s (UL:1549) */
    double ap_force;      /* 5 pN per event (UL:1560) */
    double ap_density;    /* 100: events counted for ii < ap_density*L/2 (UL:1551) */
    int32_t ap_enable;    /* 1: apply calculateForce_AP */
    uint32_t seed;        /* key word 0 of the counter-based AP stream */
    uint32_t stream;      /* key word 1: a per-cell stream id chosen by the caller */
    /* integrator (updateForces_Explicit UL:567-628) */
    double drag;          /* 0.001 */
    double damp;          /* 0.001 */
    double rho;           /* 1 */
    /* radial protrusion driver (no counterpart in the reference's default driver; the
     * reference's velocity drivers, e.g. driverVelocities_Uniaxial UL:125-168, prescribe the
     * half-step velocity of selected nodes the same way): when protrude_v != 0, every
     * boundary vertex gets V_hlf = protrude_v (X - c) / |X - c| in the plane, c =
     * (protrude_cx, protrude_cy), instead of V + dt/2 A; 0 in the reference variants */
    double protrude_v;    /* um/s (10 nm per step at dt = 5e-5 s: 200) */
    double protrude_cx, protrude_cy;
} wcfe_params;

void wcfe_params_default(wcfe_params* p, int32_t variant);

/* Message of the last failing call on this thread ("" if none). */
const char* wcfe_last_error(void);

/*
 * Counter-based stream shared by the GPU path and the oracle for the actin
 * push of calculateForce_AP (UL:1546), which the reference draws from libc
 * rand() after srand(time(NULL)) (UL:1481).  The k-th boundary vertex (in
 * vertex index order) at AP call `call` of stream (seed, stream) draws the
 * 31-bit value philox4x32_10(key = {seed, stream},
 * counter = {k, call & 0xffffffff, call >> 32, 0}).x >> 1, used as
 * Pr = r / (RAND_MAX + 1.0) with RAND_MAX = 2^31 - 1.
 */
uint32_t wcfe_ap_draw(uint32_t seed, uint32_t stream, uint64_t call, uint32_t k);
/* Raw Philox4x32-10 block (Salmon et al., SC'11), exposed for known-answer tests. */
void wcfe_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- engine --------------------------------------------------------------- */
typedef struct wcfe_engine wcfe_engine;

/* hbm_budget_bytes == 0: no budget (allocate on demand). */
int wcfe_engine_create(int32_t device, int32_t precision, uint64_t hbm_budget_bytes, wcfe_engine** out);
int wcfe_engine_destroy(wcfe_engine* eng);
int wcfe_engine_precision(const wcfe_engine* eng);
/* Bytes of the budget still free for new cells (0 when there is no budget). */
uint64_t wcfe_engine_free_bytes(const wcfe_engine* eng);
/* Device bytes a cell of this size would take (state, topology, work lists). */
uint64_t wcfe_cell_bytes(int32_t n_vert, int32_t n_tri);
int wcfe_engine_sync(wcfe_engine* eng);

/* ---- cells -------------------------------------------------------------- */
/*
 * Create a cell from its triangle mesh.  vt_ptr/vt_idx give the vertex ->
 * triangle map in the mesh's own order (NonDestructiveTriMesh::
 * m_vertex_to_triangle_map); pass NULL to build it in ascending triangle order
 * (what read_ecomsol's add_triangle sequence gives).  is_bnd may be NULL: then
 * a vertex is on the boundary when one of its edges has an odd triangle count
 * (NonDestructiveTriMesh::rebuild_auxiliary_structures).
 * The state starts at zero with c_A = 100 (cellBP/main.cpp:674-677).
 */
int wcfe_cell_create(wcfe_engine* eng, int32_t n_vert, int32_t n_tri, const int32_t* tri,
                     const int32_t* vt_ptr, const int32_t* vt_idx, const uint8_t* is_bnd,
                     const wcfe_params* params, int32_t* cell_out);
int wcfe_cell_destroy(wcfe_engine* eng, int32_t cell);
int wcfe_cell_set_params(wcfe_engine* eng, int32_t cell, const wcfe_params* params);
/* Replace the topology after El Topo remeshing; the state must be set again afterwards. */
int wcfe_cell_set_topology(wcfe_engine* eng, int32_t cell, int32_t n_vert, int32_t n_tri, const int32_t* tri,
                           const int32_t* vt_ptr, const int32_t* vt_idx, const uint8_t* is_bnd);
/* Substrate mesh of the cell, at its previous (X_s) and current (x_s) positions.
 * n_tri == 0 / tri == NULL: a flat rigid plane (the substrate displacement is 0). */
int wcfe_cell_set_substrate(wcfe_engine* eng, int32_t cell, int32_t n_vert, int32_t n_tri,
                            const int32_t* tri, const double* X_s, const double* x_s);
/* Any pointer may be NULL (that array is left unchanged / not returned). */
int wcfe_cell_set_state(wcfe_engine* eng, int32_t cell, const double* x, const double* V, const double* A,
                        const double* ea, const double* c_A, const double* c_C, const double* fa_u);
int wcfe_cell_get_state(wcfe_engine* eng, int32_t cell, double* x, double* V, double* A, double* ea,
                        double* c_A, double* c_C, double* fa_u);
/* Simulation time used for the active-stress ramp and the AP call counter. */
int wcfe_cell_set_clock(wcfe_engine* eng, int32_t cell, double t_cur, uint64_t ap_calls);
/* Step budget of a cell (no counterpart in the reference; the serving loop's stop rule):
 * 0 = unlimited (the default), n > 0 = the cell runs n more steps and then stays put,
 * skipped by every later step, whatever the number of steps queued; the device counts it
 * down, and get returns -1 once it ran out. */
int wcfe_cell_set_step_budget(wcfe_engine* eng, int32_t cell, int32_t steps);
int wcfe_cell_get_step_budget(wcfe_engine* eng, int32_t cell, int32_t* steps);
int wcfe_cell_get_clock(wcfe_engine* eng, int32_t cell, double* t_cur, uint64_t* ap_calls);
/* Bit 0: NaN/Inf in the state after the last step. */
int wcfe_cell_status(wcfe_engine* eng, int32_t cell, uint32_t* status);
int wcfe_cell_sizes(wcfe_engine* eng, int32_t cell, int32_t* n_vert, int32_t* n_tri, int32_t* n_bnd, int32_t* n_patch);

/* ---- drop-in step pieces (one cell; the order of cellBP/main.cpp:224-363) -- */
/* driverVelocities_Explicit + new_positions: V_hlf = V + dt/2 A (z = 0), x_pred = x + dt V_hlf.
 * Outputs to host arrays (either may be NULL); V_hlf also stays on the device. */
int wcfe_cell_predict(wcfe_engine* eng, int32_t cell, double dt, double* x_pred, double* V_hlf);
/* updateFA: X (NULL = device positions) are the positions before El Topo's
 * integrate, x_new after it; X_s/x_s the substrate's (NULL = as set). */
int wcfe_cell_update_fa(wcfe_engine* eng, int32_t cell, double dt_real, const double* X, const double* x_new,
                        const double* X_s, const double* x_s);
/* updateForces_Explicit (cell overload): residual, integrin, AP, drag, bending and
 * area forces, then A, ea and V.  Positions x_new become the current positions. */
int wcfe_cell_update_forces(wcfe_engine* eng, int32_t cell, double dt, double dt_real, double t_tot);

/* ---- diagnostic mirrors of the reference's force functions ------------- */
/* calculateRes (cell overload): outputs double[n][3], [n][6], [n], [n], [n] (any may be NULL).
 * X and x_new are host positions; centroid and time as in the reference call. */
int wcfe_cell_eval_residual(wcfe_engine* eng, int32_t cell, const double* X, const double* x_new,
                            double dt_real, const double centroid[3], double t_tot,
                            double* Res, double* Res_ea, double* MM, double* Res_Adif, double* Res_Cdif);
/* calculateAreaTot + calculateForce_FA + calculateForce_AP + calculateBendingForce2D +
 * calculateAreaConstraintForce at host positions x (outputs double[n][3], area4 = {A, cx, cy, cz}). */
int wcfe_cell_eval_forces(wcfe_engine* eng, int32_t cell, const double* x, double dt_real,
                          double* F_FA, double* F_AP, double* F_bend, double* F_area, double area4[4]);

/* Mixed engines: which patch-phase kernel a step uses.  0: the staged kernel (a
 * producer warp copies each patch's records and owned-vertex state into shared
 * memory one patch ahead with bulk asynchronous copies) wherever its shared-memory
 * plan fits, else the plain kernel; 1 (default): the plain kernel; 2, 3, 4: the plain
 * kernel compiled for at least 6, 7, 8 resident CTAs of 128 threads per SM (registers
 * capped; 128 patch threads only).  Results are identical; wcfe_engine_autotune times
 * them all.  No counterpart in the reference. */
int wcfe_engine_set_patch_kernel(wcfe_engine* e, int32_t kind);
/* Mixed engines: the vertex-phase kernel compiled for 5 (kind 0, default), 4 (kind 1), 6
 * (kind 2) or 8 (kind 3) resident blocks of 256 threads per SM (48, 64, 40 or 32
 * registers); results are identical; wcfe_engine_autotune times them all. */
int wcfe_engine_set_vertex_kernel(wcfe_engine* e, int32_t kind);
/* The patch and vertex kernel kinds in use (after wcfe_engine_autotune: its choice). */
int wcfe_engine_get_kernels(const wcfe_engine* e, int32_t* patch_kind, int32_t* vertex_kind);
/* Mixed engines: fused runs of steps (enable 1; default 0).  A wcfe_engine_step of
 * n >= 2 steps then folds the vertex phase of each next step into the patch phase of the
 * step before (each patch predicts its owned vertices from the velocity, acceleration and
 * strain it has just formed, still in registers; the cell's last patch forms the next
 * area): n + 1 launches instead of 2n and about 18 % fewer HBM bytes per step.  The last
 * step of a run is unfused, so the state between calls, and every result, is
 * bit-identical to enable 0.  On GB300 it is slower (0.50 against 0.35 ms per step on
 * the 256-cell workload): the vertex work then runs at the patch kernel's 20 resident
 * warps per SM instead of the vertex kernel's 40, and both phases are latency-bound, not
 * bandwidth-bound.  It applies where a plain patch kernel (kinds 1-4) is selected, in
 * engines without a coupled substrate (the fused form is one kernel, for 5 CTAs of 128
 * threads per SM); wcfe_engine_get_fused returns 1 where a run of steps is fused, else 0
 * (-1: no engine).  No counterpart in the reference (a batching schedule). */
int wcfe_engine_set_fused(wcfe_engine* e, int32_t enable);
int wcfe_engine_get_fused(const wcfe_engine* e);
/* Mixed engines: the arithmetic of the element assembly.  0 (default): FP32 (the
 * increment form of the mixed form); 1: every intermediate of the element in
 * float-float (about 48 bits) from the same FP32 vertex records, the per-corner outputs
 * rounded to FP32 once.  Mode 1 removes the FP32 element's own rounding floor (on a
 * 20,000-vertex cell over 500 steps the displacement error against the FP64 form falls
 * from about 1.1e-6 to about 1e-7) and runs the patch phase at 2 CTAs per SM; it is not
 * fused (wcfe_engine_set_fused) and not staged (patch kernel kind 0).  FP64 engines
 * accept 0 only.  get: *mode receives the current value. */
int wcfe_engine_set_element_precision(wcfe_engine* e, int32_t mode);
int wcfe_engine_get_element_precision(const wcfe_engine* e, int32_t* mode);

/* Couple cell `cell` to a deformable substrate simulated by the same FP64 engine:
 * `substrate` is another cell of the engine holding the substrate mesh and state
 * (A10; its params.mu is the substrate modulus, 1e6 in the reference, UL:726; its
 * other params give damp and rho; it has no active stress, integrins, boundary
 * terms or drag).  Each wcfe_engine_step then runs, per step: the cell's bond
 * kinetics on the substrate's step-start positions and predicted displacement
 * (updateFA UL:2026-2174), the bond reactions onto every substrate triangle
 * containing each anchor at the substrate's predicted positions
 * (calculateForce_FA_subs UL:1305-1475, accumulated in 2^-40 fixed point so the
 * sum is order-independent), and the substrate's update with them
 * (updateForces_Explicit, substrate overload UL:429-504).  Point location uses a
 * grid over the substrate's current positions; triangles that later move by more
 * than grid_margin may be missed (couple again to rebuild).  substrate < 0
 * uncouples.  The other stepping entry points refuse engines with coupled
 * substrates.  Status bit 32: a reaction beyond the fixed-point range. */
int wcfe_cell_couple_substrate(wcfe_engine* e, int32_t cell, int32_t substrate, double grid_margin);

/* Per-element shear modulus mu of the membrane [n_tri] (NULL restores params.mu for
 * every element).  An extension without counterpart in the reference, which has one
 * mu per material (UL:721-728); dropped when the topology changes. */
int wcfe_cell_set_element_mu(wcfe_engine* e, int32_t id, const double* mu);

/* ---- synthetic stepping of every live cell (no El Topo) ----------------- */
/* nsteps full explicit steps of every live cell: predict, updateFA, updateForces.
 * All cells advance in one launch per phase; runs asynchronously on the engine stream. */
int wcfe_engine_step(wcfe_engine* eng, int32_t nsteps, double dt);
/* Same, restricted to the listed cells. */
int wcfe_engine_step_cells(wcfe_engine* eng, const int32_t* cells, int32_t ncells, int32_t nsteps, double dt);
/* Batched drop-in exchange for cells coupled to a host-side integrator (El Topo):
 * positions of every live cell packed [sum n][3] in ascending cell-id order.
 * wcfe_engine_predict: driverVelocities_Explicit + predict of every cell, predicted
 *   positions copied to x_pred (returns when the copy is done);
 * wcfe_engine_update: the integrated positions x_new (dt_real = the step El Topo took)
 *   drive updateFA and updateForces_Explicit of every cell in one launch per phase;
 *   x_new is read asynchronously: keep it unchanged until the next synchronising call. */
int64_t wcfe_engine_total_vertices(wcfe_engine* eng);
int wcfe_engine_predict(wcfe_engine* eng, double dt, double* x_pred);
int wcfe_engine_update(wcfe_engine* eng, double dt, double dt_real, const double* x_new);
/* The exchange path splits the cells into `groups` (1 to 8, default 8) of about equal
 * vertex count, each stepped on its own stream, the streams at descending priorities so
 * that the groups finish in order: one group's predict and copy to the host overlap the
 * later groups' update.  Results do not depend on the grouping. */
int wcfe_engine_set_exchange_groups(wcfe_engine* eng, int32_t groups);
/* Per-vertex integrin density (#/um^2) replacing rho_i_max (UL:1218); NULL restores the
 * uniform density.  A zero entry is a vertex without integrins. */
int wcfe_cell_set_integrins(wcfe_engine* eng, int32_t cell, const double* rho);
/* Capture steps into CUDA graphs (1) or launch eagerly (0, default). */
int wcfe_engine_set_graphs(wcfe_engine* eng, int32_t enable);
/* Kernel shapes: threads per CTA of the patch kernel (a multiple of 32; at most 512, at
 * most 128 for a mixed engine), max elements per patch (32-4096).
 * 0 = keep the current value (wcfe_engine_autotune chooses both). */
int wcfe_engine_set_shape(wcfe_engine* eng, int32_t patch_threads, int32_t patch_elems);
int wcfe_engine_get_shape(const wcfe_engine* eng, int32_t* patch_threads, int32_t* patch_elems);
/* Time every candidate shape on the live cells (reps steps each) and keep the fastest. */
int wcfe_engine_autotune(wcfe_engine* eng, double dt, int32_t reps);
/* Device timing of the last wcfe_engine_step (ms per kernel phase, summed over steps). */
int wcfe_engine_last_timing(wcfe_engine* eng, float* ms_vertex, float* ms_patch);
/* Per-step device time (ms, events on the engine stream) of the last timed wcfe_engine_step;
 * *span_ms receives the time from the first step's start to the last step's end. Returns the count. */
int64_t wcfe_engine_step_times(wcfe_engine* eng, float* out, int64_t cap, float* span_ms);
/* Enable per-phase CUDA-event timing inside wcfe_engine_step (off by default); a timed
 * call launches eagerly (no graph) and records three events per step without host sync. */
int wcfe_engine_set_timing(wcfe_engine* eng, int32_t enable);
/* Number of kernels this engine launched since creation. */
uint64_t wcfe_engine_launches(const wcfe_engine* eng);
/* The engine's main CUDA stream (a cudaStream_t), so that a caller can order its own work
 * or record timing events against the engine's steps. */
void* wcfe_engine_stream(const wcfe_engine* eng);

/* ---- serving: continuous batching of whole cell simulations -------------- */
typedef struct wcfe_server wcfe_server;
/* A request: one cell mesh + initial state + number of steps. Arrays are copied at submit. */
typedef struct wcfe_request {
    int32_t n_vert, n_tri;
    const int32_t* tri;
    const double* x;          /* [n][3] initial positions */
    const wcfe_params* params;
    int32_t n_steps;
    const int32_t* sub_tri;   /* optional substrate mesh (NULL = plane) */
    const double* sub_X;
    int32_t sub_n_vert, sub_n_tri;
} wcfe_request;

int wcfe_server_create(wcfe_engine* eng, double dt, wcfe_server** out);
int wcfe_server_destroy(wcfe_server* srv);
/* Queue a request; *req_id receives its id (monotonic from 0). */
int wcfe_server_submit(wcfe_server* srv, const wcfe_request* req, int64_t* req_id);
/* One serving iteration: admit queued requests (prepared on the server's host worker
 * threads, in arrival order) while the engine's HBM budget has room, enqueue K steps of
 * every resident cell (K chosen so that an iteration takes about the target GPU time,
 * wcfe_server_set_iteration_ms; each cell stops on the device after exactly its
 * n_steps), and queue the results of the cells that finish.  At most two iterations are
 * in flight: the call waits for the one before the last.  *n_active reports the resident
 * cells, *n_queued the requests not yet admitted plus the iterations still in flight. */
int wcfe_server_iterate(wcfe_server* srv, int32_t* n_active, int32_t* n_queued);
/* Target GPU time of one serving iteration (default 8 ms). */
int wcfe_server_set_iteration_ms(wcfe_server* srv, double ms);
/* Cell-steps enqueued by the server so far. */
uint64_t wcfe_server_cell_steps(const wcfe_server* srv);
/* Fetch a finished request's final positions (double[n][3]) and latency stats.
 * Returns WCFE_ERR_ARG while it is still running. */
int wcfe_server_result(wcfe_server* srv, int64_t req_id, double* x_out, double* seconds_in_system);
/* Per-step latency samples (seconds) collected so far, one per step: the device time
 * of each completed iteration divided by its steps; returns the count. */
int64_t wcfe_server_step_times(wcfe_server* srv, double* out, int64_t cap);

/* Rates of the pipes on the current device, for roofline denominators (no counterpart in
 * the reference): TF32 tcgen05 MMAs (M 128, N 256, operands resident in shared memory,
 * one CTA per SM), and FP64 and FP32 FMA chains, in TFLOP/s.  A negative TF32 rate means
 * its bounded wait gave up.  Takes a few hundred milliseconds. */
int wcfe_debug_pipe_rates(double* tf32_tflops, double* fp64_tflops, double* fp32_tflops);

/* ---- allocation-free area reduction ------------------------------------- */
/* No counterpart in the reference: the same total area and area-weighted
 * centroid as calculateAreaTot (computed inside every engine step), as a
 * single call that allocates no device memory, for host codes that reserve
 * all their device memory up front or must not synchronise on cudaMalloc /
 * cudaFree mid-loop.  Inputs and output are the caller's device memory:
 * x double[n][3], tri int32[t][3], area4 double[4] = {A, cx, cy, cz}.  The
 * scratch is a 128 KiB file-scope device array that every GPU loading the
 * library keeps until exit; t <= 4,194,304 (else WCFE_ERR_LIMIT).  The first
 * call on a device resolves the array's address (do it before any stream
 * capture) and keeps it for the life of the process, so the entry point must
 * not be called on a device again after a cudaDeviceReset of it.  Calls
 * overlapping on the GPU race on the shared array.  An index outside [0, n)
 * yields NaN.  A CUDA error already pending on the calling thread is left in
 * place and the call returns WCFE_ERR_CUDA without launching.  stream: a
 * cudaStream_t, or NULL. */
int wcfe_area_tot_noalloc(const double* x_dev, int32_t n_vert, const int32_t* tri_dev, int32_t n_tri,
                          double* area4_dev, void* stream);

/* ---- implicit (Newton) step: no counterpart in the reference -------------
 * Backward Euler of the explicit step's equations of motion (UL:592-628) with the
 * membrane implicit and the adhesion and boundary forces (A4, A6-A8) taken at the
 * predicted positions (A1, after the bond kinetics A5):
 *   G(x) = m (x - X)/dt^2 - m V/dt + (drag + damp m)(x - X)/dt - F_ext + Res(X, x, ea) = 0
 * in the plane (2N unknowns; planar cells).  Per Newton iteration: G in FP64, the
 * dense 2N x 2N tangent from FP32 element tangents, its LU factorisation (trailing
 * updates on the tensor cores, TF32), and the solve refined in FP64 until its
 * residual is 1e-10 of |G|.  Converged when |G|inf <= newton_rtol * (the largest
 * term G sums), or at the residual's rounding floor, |dRes/dx| ulp(x) with FP64
 * positions: the last correction below 1e-13 of the displacement, or no further
 * reduction of |G| (more than 1/4 of the previous) once below 1e-6 of the scale.
 * After the step V = (x - X)/dt, A = (V - V_old)/dt, ea += Res_ea/MM.  FP64 engines
 * only.  Dense factors take 4 (2N)^2 bytes per cell on the device; this workspace is kept
 * (and counted against the HBM budget) from one call to the next until the cells or the
 * LU's outer block change, or the engine is destroyed. */
typedef struct wcfe_newton_stats {
    int32_t newton_iters;              /* Newton updates summed over steps (all cells together) */
    int32_t max_refine_iters;          /* largest number of refinement passes of one linear solve */
    int32_t unconverged;               /* cell-steps that hit max_newton without converging */
    int32_t floor_exits;               /* cell-steps that stopped at the residual's rounding floor above rtol */
    double max_rel_residual;           /* largest final |G|inf / force scale */
    double max_refine_rel_residual;    /* largest final |J dx + G|inf / |G|inf of a linear solve */
    double lu_ms;                      /* device time of the dense factorisations (CUDA events) */
    double lu_gflop;                   /* their work, 2/3 (2N)^3 per factored cell, in GFLOP */
    double solve_ms;                   /* device time of the triangular solves with the factors */
} wcfe_newton_stats;

int wcfe_engine_step_implicit(wcfe_engine* e, int32_t nsteps, double dt, double newton_rtol, int32_t max_newton,
                              wcfe_newton_stats* stats);

/* The implicit step's dense LU.  block: the outer block width, a multiple of 64 from 64
 * to 1024 (default 1024): the trailing matrix takes one update per outer block with
 * K = block, which reads and writes it once per block.  kind 0 (default):
 * trailing updates on the tcgen05 tensor cores (TMA-fed, TF32, accumulators in TMEM);
 * kind 1: the mma.sync TF32 updates (block must be 64).  FP64 engines; results agree
 * to TF32 rounding, and the refinement takes every solve to the same tolerance. */
int wcfe_engine_set_lu(wcfe_engine* e, int32_t block, int32_t kind);
/* reuse 1 (default): one dense factorisation per implicit step, kept by its later Newton
 * iterations (the refinement against the current tangent restores the exact correction);
 * 0: a fresh factorisation every Newton iteration. */
int wcfe_engine_set_lu_reuse(wcfe_engine* e, int32_t reuse);

/* Factor the dense m x m matrix A (row-major, FP32, m even) with the implicit step's
 * LU (no pivoting; TF32 tensor-core trailing updates) and solve A x = b once
 * (unrefined).  Device 0; for tests of the factorisation itself. */
int wcfe_debug_lu_solve(int32_t m, const float* A, const double* b, float* x);
/* The tensor-core LU's schedule for a matrix of order m and outer block `block` (host
 * logic, no device): *nops steps, each 14 int32 in ops (when ops is not NULL and cap, in
 * int32, holds them): type (0 diagonal 64 x 64 factor and its inverses at k0, 1 that
 * step's panels, 2 region update), k0, nreg, ka, kb, K, then (rlo, rhi, clo, chi) of two
 * regions (-1 = m): C[rlo:rhi, clo:chi] -= J[rlo:rhi, ka:ka+K] U[ka:ka+K, clo:chi]. */
int wcfe_debug_lu_schedule(int32_t m, int32_t block, int32_t* ops, int32_t cap, int32_t* nops);
/* The same with the LU variant of wcfe_engine_set_lu. */
int wcfe_debug_lu_solve_with(int32_t m, const float* A, const double* b, float* x, int32_t block, int32_t kind);
/* The failure path of the triangular solves, for tests: as wcfe_debug_lu_solve, but the
 * solution of 64-row block `withhold` is never published to the blocks that wait for it,
 * whose waits give up after wait_clocks SM clocks.  Returns WCFE_ERR_CUDA ("triangular
 * sweep timed out") when a wait ran out; the context stays usable. */
int wcfe_debug_trsv_withheld(int32_t m, const float* A, const double* b, float* x, int32_t withhold,
                             int64_t wait_clocks);

/* The dense tangent J (2N x 2N, row-major, FP32) of cell `id` at positions x [n][3]
 * with the cell's state as step start, and the mass/damping diagonal [n]. */
int wcfe_cell_newton_tangent(wcfe_engine* e, int32_t id, double dt, const double* x, float* J_out, double* diag_out);

/* ---- El Topo co-residency ---------------------------------------------------
 * After the host's remeshing (improve_mesh, defrag_mesh; cellBP/main.cpp:191-192),
 * rebuild cell `id` with its state carried on the device, as El Topo carries it:
 * split k (El Topo's VERTEX_ADD events, in order; eltopo3d/edgesplitter.cpp:564-577)
 * appends vertex n_old + k with every state field 0.5 (s[a] + s[b]), split_ab[2k] = a,
 * split_ab[2k + 1] = b in the same numbering (old vertices or earlier splits);
 * collapses and flips leave the survivors' states as they are; keep [nv_new] is the
 * defrag map (eltopo3d/surftrack.cpp:487-593): new vertex j is vertex keep[j] of that
 * numbering, ascending.  tri, vt_ptr, vt_idx, is_bnd: the new connectivity as for
 * wcfe_cell_set_topology; x_new [nv_new][3]: the remeshed positions.  The clock, the AP
 * counter and the integrin densities (copied and averaged like the state) carry over;
 * per-element moduli return to params.mu.  Not for coupled cells or substrates. */
int wcfe_cell_remesh(wcfe_engine* e, int32_t id, int32_t n_split, const int32_t* split_ab, int32_t nv_new,
                     const int32_t* keep, int32_t nt_new, const int32_t* tri, const int32_t* vt_ptr,
                     const int32_t* vt_idx, const uint8_t* is_bnd, const double* x_new);

/* ---- VTK frames (cellBP/iomesh.cpp:690-1047), byte for byte ------------------
 * Replaces the reference's write_vtk calls (cellBP/main.cpp:447-454, :721-723) without
 * stalling the stepping stream: a write packs the cell's current state on the engine's
 * stream (one gather kernel, either precision), copies it to pinned host memory on the
 * frame writer's own stream, and a host writer thread formats and writes the file.
 * slots: staging buffers in flight (a write waits for a free one); threads: writer
 * threads.  format 0: positions and triangles (iomesh.cpp:690); 1: strain measure
 * sqrt(det((I - 2 ea)^-1)) and bond vectors, fixed notation (:730, the substrate's
 * frames); 2: c_A, the strain measure, c_C, the integrin force and the bond vectors
 * (:844, the cell's frames; the force follows the cell's law: for WCFE_LAW_MD_TABLE
 * (kMD) the MD table, or kint |u| when kint >= 0; else |k_lin u| in the plane (k1,
 * k31)).  time: the header's time; NaN takes the cell's clock. */
typedef struct wcfe_frames wcfe_frames;
int wcfe_frames_create(wcfe_engine* e, int32_t slots, int32_t threads, wcfe_frames** out);
int wcfe_frames_write(wcfe_frames* f, int32_t cell, int32_t format, double time, double kint, const char* path);
/* wait until every queued frame is written; the first write error since the last flush */
int wcfe_frames_flush(wcfe_frames* f);
int wcfe_frames_destroy(wcfe_frames* f);
/* Host only: the text of a frame from host arrays (x, fau [n][3], cA, cC [n], ea [n][6]);
 * law and k_fa give the force column of format 2 as above.  Copies at most cap bytes
 * to out; *len is the full length. */
int wcfe_vtk_format(int32_t format, int32_t n, int32_t nt, const int32_t* tri, const double* x, const double* cA,
                    const double* cC, const double* fau, const double* ea, double time, double kint, int32_t law,
                    double k_fa, char* out, int64_t cap, int64_t* len);

/* ---- host-only inspection of the connectivity preprocessing (no device) --- */
/* Boundary ranks and neighbour candidates (the scan of UL:1500-1531), patches and
 * one-ring slot codes, exactly as the engine builds them.  Capacities in int32 units. */
int wcfe_debug_topology(int32_t n_vert, int32_t n_tri, const int32_t* tri, const int32_t* vt_ptr,
                        const int32_t* vt_idx, const uint8_t* is_bnd, int32_t patch_elems_max, int32_t* nb_out,
                        int32_t* bnd_rank, int32_t* bnd_cptr, int32_t* bnd_cand, int32_t cand_cap, int32_t* np_out,
                        int32_t* patch, int32_t patch_cap, int32_t* patch_elems, int32_t elems_cap,
                        uint16_t* vc_code);

/* The staging description the mixed form's patch kernel copies per patch: for
 * each patch (h0, nh, c0, nc) = its halo list (vertices of its elements outside
 * its owned range, ascending) and its one-ring code range; the corners of every
 * element slot as patch-local vertex indices (owned v -> v - v0, halo k -> nvp + k,
 * 4 uint16 per slot, each patch's rows padded to an even count); maxima_out[4] =
 * largest (ne, nvp, nh, nc) over the patches.  No counterpart in the reference. */
int wcfe_debug_patch_staging(int32_t n_vert, int32_t n_tri, const int32_t* tri, int32_t patch_elems_max,
                             int32_t* np_out, int32_t* xinfo, int32_t xinfo_cap, int32_t* halo, int32_t halo_cap,
                             uint16_t* loc, int32_t loc_cap, int32_t* maxima_out);

#ifdef __cplusplus
}
#endif
#endif /* WCFE_H */
