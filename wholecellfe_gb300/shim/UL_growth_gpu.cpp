// UL_growth_gpu.cpp — drop-in replacement for cellBP/UL_growth_explicit.cpp in the
// reference's cellBP build (cellBP/Makefile:27, SRC): the four mechanics calls that
// cellBP/main.cpp makes (main.cpp:224 driverVelocities_Explicit, :356 updateFA, :362-363
// updateForces_Explicit, declared at main.cpp:72-87) run on the GPU through the C ABI of
// libwcfe.so (include/wcfe.h).  The cell's state stays on the device between calls and is
// copied back into the driver's vectors after each call, so El Topo and the VTK writers
// see what they see with the CPU path.
//
// Build: compile inside cellBP against the reference's headers (vec.h,
// nondestructivetrimesh.h, Eigen) in place of UL_growth_explicit.cpp and link with
// -lwcfe -lcudart.  WCFE_SHIM_VARIANT selects the parameters of the reference variant
// (WCFE_VARIANT_KMD by default, or WCFE_VARIANT_K1 / WCFE_VARIANT_K31).
//
// Connectivity.  init_simulation (main.cpp:547) calls wcfe_gpu_attach(mesh, positions)
// once the meshes are read.  Before every predict the shim compares El Topo's triangle
// list with the one on the device:
//  - same vertices, other triangles (edge flips): wcfe_cell_remesh with no splits and the
//    identity map, so the state is carried on the device;
//  - a different vertex count (splits, collapses, defrag): the new connectivity is uploaded
//    and the state is taken from the driver's vectors, which El Topo has interpolated
//    (V and A at once, c_A, c_C, fa_u in updateFA, the strain in updateForces_Explicit).
// A driver that records El Topo's change history can call wcfe_cell_remesh itself
// instead (cellbp_gpu_extras.cpp, sync_after_remesh), which carries every field on the
// device.
#include <Eigen/Dense>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "nondestructivetrimesh.h"
#include "vec.h"
#include "wcfe.h"

#ifndef WCFE_SHIM_VARIANT
#define WCFE_SHIM_VARIANT WCFE_VARIANT_KMD
#endif

wcfe_engine* g_eng = nullptr;
int32_t g_cell = -1;
static const NonDestructiveTriMesh* g_mesh = nullptr;   // the cell mesh of the last call
static std::vector<int32_t> g_tri;                       // the triangles on the device
static bool g_pending_fa = false, g_pending_ea = false;  // host state to upload after a re-upload

static void check(int rc, const char* what) {
    if (rc) std::fprintf(stderr, "wcfe: %s failed (%d): %s\n", what, rc, wcfe_last_error());
}

static void triangles_of(const NonDestructiveTriMesh& m, std::vector<int32_t>& tri) {
    tri.resize(3 * m.num_triangles());
    for (size_t t = 0; t < m.num_triangles(); ++t)
        for (int a = 0; a < 3; ++a) tri[3 * t + a] = (int32_t)m.get_triangle(t)[a];
}

static void connectivity_of(const NonDestructiveTriMesh& m, size_t nv, std::vector<int32_t>& ptr,
                            std::vector<int32_t>& idx, std::vector<uint8_t>& bnd) {
    ptr.assign(nv + 1, 0);
    idx.clear();
    bnd.assign(nv, 0);
    for (size_t v = 0; v < nv; ++v) {
        ptr[v] = (int32_t)idx.size();
        for (size_t t : m.m_vertex_to_triangle_map[v]) idx.push_back((int32_t)t);
        bnd[v] = m.m_is_boundary_vertex[v];
    }
    ptr[nv] = (int32_t)idx.size();
}

// Create the device cell from the driver's mesh and positions (init_simulation).
void wcfe_gpu_attach(const NonDestructiveTriMesh& m, const std::vector<Vec3d>& x) {
    if (!g_eng) check(wcfe_engine_create(0, WCFE_PREC_FP64, 0, &g_eng), "wcfe_engine_create");
    std::vector<int32_t> ptr, idx;
    std::vector<uint8_t> bnd;
    triangles_of(m, g_tri);
    connectivity_of(m, x.size(), ptr, idx, bnd);
    wcfe_params p;
    wcfe_params_default(&p, WCFE_SHIM_VARIANT);
    if (g_cell >= 0) wcfe_cell_destroy(g_eng, g_cell);
    check(wcfe_cell_create(g_eng, (int32_t)x.size(), (int32_t)m.num_triangles(), g_tri.data(), ptr.data(), idx.data(),
                           bnd.data(), &p, &g_cell),
          "wcfe_cell_create");
    check(wcfe_cell_set_state(g_eng, g_cell, &x[0][0], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr),
          "wcfe_cell_set_state");
    g_mesh = &m;
}

// Bring the device connectivity in line with El Topo's mesh (see the file comment).
static void sync_topology(const std::vector<Vec3d>& X, const std::vector<Vec3d>& V, const std::vector<Vec3d>& A) {
    if (!g_mesh) return;
    std::vector<int32_t> tri;
    triangles_of(*g_mesh, tri);
    int32_t nv = 0, nt = 0, nb = 0, np = 0;
    wcfe_cell_sizes(g_eng, g_cell, &nv, &nt, &nb, &np);
    if ((size_t)nv == X.size() && tri == g_tri) return;
    std::vector<int32_t> ptr, idx;
    std::vector<uint8_t> bnd;
    connectivity_of(*g_mesh, X.size(), ptr, idx, bnd);
    if ((size_t)nv == X.size()) {   // flips: the state stays on the device
        std::vector<int32_t> keep(nv);
        for (int32_t v = 0; v < nv; ++v) keep[v] = v;
        check(wcfe_cell_remesh(g_eng, g_cell, 0, nullptr, nv, keep.data(), (int32_t)g_mesh->num_triangles(), tri.data(),
                               ptr.data(), idx.data(), bnd.data(), &X[0][0]),
              "wcfe_cell_remesh");
    } else {                         // splits / collapses: the driver's interpolated state
        check(wcfe_cell_set_topology(g_eng, g_cell, (int32_t)X.size(), (int32_t)g_mesh->num_triangles(), tri.data(),
                                     ptr.data(), idx.data(), bnd.data()),
              "wcfe_cell_set_topology");
        check(wcfe_cell_set_state(g_eng, g_cell, &X[0][0], &V[0][0], &A[0][0], nullptr, nullptr, nullptr, nullptr),
              "wcfe_cell_set_state");
        g_pending_fa = g_pending_ea = true;
    }
    g_tri.swap(tri);
}

void driverVelocities_Explicit(const std::vector<Vec3d>& X_t, std::vector<Vec3d>& V_t, std::vector<Vec3d>& V_t_hlf,
                               std::vector<Vec3d>& A_t, double dt) {
    sync_topology(X_t, V_t, A_t);
    std::vector<Vec3d> xp(X_t.size());
    check(wcfe_cell_predict(g_eng, g_cell, dt, &xp[0][0], &V_t_hlf[0][0]), "wcfe_cell_predict");   // main.cpp:227-231
}

void updateFA(std::vector<double>& c_A, std::vector<double>& c_C, std::vector<Vec3d>& fa_u, double dt_real,
              const std::vector<Vec3d>& X_cell, const std::vector<Vec3d>& x_cell, const NonDestructiveTriMesh& mesh_cell,
              const std::vector<Vec3d>& X_subs, const std::vector<Vec3d>& x_subs, const NonDestructiveTriMesh& mesh_subs,
              double kint) {
    g_mesh = &mesh_cell;
    if (g_pending_fa) {
        check(wcfe_cell_set_state(g_eng, g_cell, nullptr, nullptr, nullptr, nullptr, c_A.data(), c_C.data(), &fa_u[0][0]),
              "wcfe_cell_set_state");
        g_pending_fa = false;
    }
    check(wcfe_cell_update_fa(g_eng, g_cell, dt_real, &X_cell[0][0], &x_cell[0][0], &X_subs[0][0], &x_subs[0][0]),
          "wcfe_cell_update_fa");
    check(wcfe_cell_get_state(g_eng, g_cell, nullptr, nullptr, nullptr, nullptr, c_A.data(), c_C.data(), &fa_u[0][0]),
          "wcfe_cell_get_state");
}

void updateForces_Explicit(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Vec3d>& V_t,
                           std::vector<Vec3d>& V_t_hlf, std::vector<Vec3d>& A_t, std::vector<Eigen::VectorXd>& ea_t,
                           std::vector<double>& c_A, std::vector<double>& c_B, std::vector<double>& c_C,
                           std::vector<Vec3d>& fa_u, double dt, double dt_real, const NonDestructiveTriMesh& mesh,
                           double t_tot) {
    g_mesh = &mesh;
    std::vector<double> ea(6 * ea_t.size());
    if (g_pending_ea) {
        for (size_t v = 0; v < ea_t.size(); ++v)
            for (int q = 0; q < 6; ++q) ea[6 * v + q] = ea_t[v](q);
        check(wcfe_cell_set_state(g_eng, g_cell, nullptr, nullptr, nullptr, ea.data(), nullptr, nullptr, nullptr),
              "wcfe_cell_set_state");
        g_pending_ea = false;
    }
    check(wcfe_cell_update_forces(g_eng, g_cell, dt, dt_real, t_tot), "wcfe_cell_update_forces");
    check(wcfe_cell_get_state(g_eng, g_cell, nullptr, &V_t[0][0], &A_t[0][0], ea.data(), nullptr, nullptr, nullptr),
          "wcfe_cell_get_state");
    for (size_t v = 0; v < ea_t.size(); ++v)
        for (int q = 0; q < 6; ++q) ea_t[v](q) = ea[6 * v + q];
}

// main.cpp:363 also advances the substrate.  With the rigid substrate of main.cpp:299
// nothing reads its outputs, so this overload has nothing to do; a deformable substrate
// is a coupled cell of the engine instead (cellbp_gpu_extras.cpp).
void updateForces_Explicit(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Vec3d>& V_t,
                           std::vector<Vec3d>& V_t_hlf, std::vector<Vec3d>& A_t, std::vector<Eigen::VectorXd>& ea_t,
                           double dt, double dt_real, const NonDestructiveTriMesh& mesh, double t_tot,
                           std::vector<Vec3d>& fa_u, const std::vector<double>& c_C, const std::vector<Vec3d>& x_cell,
                           const NonDestructiveTriMesh& mesh_cell) {}
