// ref_harness.cpp — C entry points around the reference's own mechanics
// functions, compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/libwcfe_ref_<variant>.so.  TEST INFRASTRUCTURE ONLY: it exists
// to pin the C restatement (oracle/wcfe_oracle.c) and to produce the golden
// fixtures under tests/golden/.
//
// The reference declares its functions only inside cellBP/main.cpp:69-87, so
// the declarations below repeat those signatures.  Nothing here changes the
// reference's arithmetic: every entry point converts plain arrays into the
// reference's containers (std::vector<Vec3d>, std::vector<Eigen::VectorXd>,
// NonDestructiveTriMesh), calls the reference function, and converts back.
#include <Eigen/Dense>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <vector>

#include "iomesh.h"
#include "nondestructivetrimesh.h"
#include "vec.h"

// ---- reference functions (signatures as in cellBP/main.cpp:69-87 and UL) ----
void driverVelocities_Explicit(const std::vector<Vec3d>& X_t, std::vector<Vec3d>& V_t, std::vector<Vec3d>& V_t_hlf,
                               std::vector<Vec3d>& A_t, double dt);
void updateFA(std::vector<double>& c_A, std::vector<double>& c_C, std::vector<Vec3d>& fa_u, double dt_real,
              const std::vector<Vec3d>& X_t_cell, const std::vector<Vec3d>& x_t_cell, const NonDestructiveTriMesh& mesh_cell,
              const std::vector<Vec3d>& X_t_subs, const std::vector<Vec3d>& x_t_subs, const NonDestructiveTriMesh& mesh_subs,
              double kint);
void updateForces_Explicit(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Vec3d>& V_t,
                           std::vector<Vec3d>& V_t_hlf, std::vector<Vec3d>& A_t, std::vector<Eigen::VectorXd>& ea_t,
                           std::vector<double>& c_A, std::vector<double>& c_B, std::vector<double>& c_C,
                           std::vector<Vec3d>& fa_u, double dt, double dt_real, const NonDestructiveTriMesh& mesh,
                           double t_tot);
void updateForces_Explicit(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Vec3d>& V_t,
                           std::vector<Vec3d>& V_t_hlf, std::vector<Vec3d>& A_t, std::vector<Eigen::VectorXd>& ea_t,
                           double dt, double dt_real, const NonDestructiveTriMesh& mesh, double t_tot,
                           std::vector<Vec3d>& fa_u, const std::vector<double>& c_C, const std::vector<Vec3d>& x_cell,
                           const NonDestructiveTriMesh& mesh_cell);
void calculateRes(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Eigen::VectorXd>& ea_t,
                  const std::vector<double>& c_A, const std::vector<double>& c_C, const NonDestructiveTriMesh& mesh,
                  double dt_real, Eigen::VectorXd& Res, Eigen::VectorXd& Res_ea, Eigen::VectorXd& MM,
                  Eigen::VectorXd& Res_Adif, Eigen::VectorXd& Res_Cdif, int mat, Eigen::Vector3d& centroid, double time);
void calculateRes(const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t, std::vector<Eigen::VectorXd>& ea_t,
                  const NonDestructiveTriMesh& mesh, double dt_real, Eigen::VectorXd& Res, Eigen::VectorXd& Res_ea,
                  Eigen::VectorXd& MM, int mat, double time);
void calculateForce_FA(Eigen::VectorXd& F_constraint, const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t,
                       const std::vector<double>& c_C, std::vector<Vec3d>& fa_u, const NonDestructiveTriMesh& mesh,
                       double kint);
void calculateForce_FA_subs(Eigen::VectorXd& F_constraint, const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t,
                            const NonDestructiveTriMesh& mesh, const std::vector<double>& c_C,
                            const std::vector<Vec3d>& x_cell, std::vector<Vec3d>& fa_u,
                            const NonDestructiveTriMesh& mesh_cell, double kint);
void calculateForce_AP(Eigen::VectorXd& F_constraint, const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t,
                       const std::vector<double>& c_A, const NonDestructiveTriMesh& mesh, double dt_real);
void calculateBendingForce2D(Eigen::VectorXd& F_bending, const std::vector<Vec3d>& X_t, const std::vector<Vec3d>& x_t,
                             const NonDestructiveTriMesh& mesh);
Eigen::Vector4d calculateAreaTot(const std::vector<Vec3d>& x_t, const NonDestructiveTriMesh& mesh);
void calculateAreaConstraintForce(Eigen::VectorXd& F_areaConstraint, const std::vector<Vec3d>& X_t,
                                  const std::vector<Vec3d>& x_t, const NonDestructiveTriMesh& mesh, double tot_area);

// ---- counter-based rand()/srand() stand-ins (oracle/ref_rng.c) ----
extern "C" void ref_rng_set(uint32_t seed, uint32_t stream, uint64_t next_call);
extern "C" uint64_t ref_rng_calls(void);

namespace {
struct Quiet {  // the reference prints progress on std::cout from inside the hot loop
    std::streambuf* old;
    Quiet() : old(std::cout.rdbuf(nullptr)) {}
    ~Quiet() { std::cout.rdbuf(old); }
};
std::vector<Vec3d> v3(const double* a, int n) {
    std::vector<Vec3d> v(n);
    for (int i = 0; i < n; ++i) v[i] = Vec3d(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return v;
}
void out3(const std::vector<Vec3d>& v, double* a) {
    for (size_t i = 0; i < v.size(); ++i)
        for (int c = 0; c < 3; ++c) a[3 * i + c] = v[i][c];
}
std::vector<Eigen::VectorXd> v6(const double* a, int n) {
    std::vector<Eigen::VectorXd> v(n, Eigen::VectorXd(6));
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < 6; ++q) v[i](q) = a[6 * i + q];
    return v;
}
void out6(const std::vector<Eigen::VectorXd>& v, double* a) {
    for (size_t i = 0; i < v.size(); ++i)
        for (int q = 0; q < 6; ++q) a[6 * i + q] = v[i](q);
}
std::vector<double> vd(const double* a, int n) { return a ? std::vector<double>(a, a + n) : std::vector<double>(n, 0.0); }
void outv(const Eigen::VectorXd& v, double* a) {
    if (a) std::memcpy(a, v.data(), sizeof(double) * v.size());
}
}  // namespace

extern "C" {

// Build a mesh the way read_ecomsol does (iomesh.cpp:536-553): one add_triangle per triangle.
void* ref_mesh_new(int32_t nv, int32_t nt, const int32_t* tri) {
    NonDestructiveTriMesh* m = new NonDestructiveTriMesh();
    m->set_num_vertices(nv);
    for (int t = 0; t < nt; ++t) m->add_triangle(Vec3st(tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]));
    return m;
}
void ref_mesh_free(void* m) { delete static_cast<NonDestructiveTriMesh*>(m); }
// Vertex -> triangle map (CSR) and boundary flags as the mesh holds them.
int32_t ref_mesh_map(void* mp, int32_t* vt_ptr, int32_t* vt_idx, uint8_t* bnd) {
    NonDestructiveTriMesh* m = static_cast<NonDestructiveTriMesh*>(mp);
    int32_t nv = (int32_t)m->m_vertex_to_triangle_map.size(), k = 0;
    for (int32_t v = 0; v < nv; ++v) {
        if (vt_ptr) vt_ptr[v] = k;
        for (size_t t : m->m_vertex_to_triangle_map[v]) {
            if (vt_idx) vt_idx[k] = (int32_t)t;
            ++k;
        }
        if (bnd) bnd[v] = m->m_is_boundary_vertex[v] ? 1 : 0;
    }
    if (vt_ptr) vt_ptr[nv] = k;
    return k;
}

void ref_predict(int32_t n, const double* x, double* V, const double* A, double dt, double* Vh, double* xpred) {
    Quiet q;
    auto X = v3(x, n), Vv = v3(V, n), Av = v3(A, n), Vhv = std::vector<Vec3d>(n);
    driverVelocities_Explicit(X, Vv, Vhv, Av, dt);
    out3(Vhv, Vh);
    for (int i = 0; i < n; ++i) {
        Vec3d p = X[i] + dt * Vhv[i];  // cellBP/main.cpp:227-231
        for (int c = 0; c < 3; ++c) xpred[3 * i + c] = p[c];
    }
}

void ref_area_tot(void* mp, int32_t n, const double* x, double* out4) {
    Quiet q;
    Eigen::Vector4d a = calculateAreaTot(v3(x, n), *static_cast<NonDestructiveTriMesh*>(mp));
    for (int k = 0; k < 4; ++k) out4[k] = a(k);
}

void ref_calc_res(void* mp, int32_t n, const double* X, const double* x, const double* ea, const double* cA,
                  const double* cC, double dt_real, int32_t mat, const double* centroid, double time, double* Res,
                  double* Res_ea, double* MM, double* ResA, double* ResC) {
    Quiet q;
    auto Xv = v3(X, n), xv = v3(x, n);
    auto eav = v6(ea, n);
    Eigen::VectorXd R(3 * n), Re(6 * n), M(n), RA(n), RC(n);
    const NonDestructiveTriMesh& m = *static_cast<NonDestructiveTriMesh*>(mp);
    if (mat == 1) {
        auto a = vd(cA, n), c = vd(cC, n);
        Eigen::Vector3d cen(centroid[0], centroid[1], centroid[2]);
        calculateRes(Xv, xv, eav, a, c, m, dt_real, R, Re, M, RA, RC, 1, cen, time);
        outv(RA, ResA);
        outv(RC, ResC);
    } else {
        calculateRes(Xv, xv, eav, m, dt_real, R, Re, M, mat, time);
    }
    outv(R, Res);
    outv(Re, Res_ea);
    outv(M, MM);
}

void ref_force_fa(void* mp, int32_t n, const double* X, const double* x, const double* cC, const double* fau,
                  double kint, double* F) {
    Quiet q;
    auto f = v3(fau, n);
    Eigen::VectorXd Fv(3 * n);
    Fv.setZero();
    calculateForce_FA(Fv, v3(X, n), v3(x, n), vd(cC, n), f, *static_cast<NonDestructiveTriMesh*>(mp), kint);
    outv(Fv, F);
}

void ref_force_ap(void* mp, int32_t n, const double* X, const double* x, const double* cA, double dt_real,
                  uint32_t seed, uint32_t stream, uint64_t call, double* F) {
    Quiet q;
    ref_rng_set(seed, stream, call);
    Eigen::VectorXd Fv(3 * n);
    Fv.setZero();
    calculateForce_AP(Fv, v3(X, n), v3(x, n), vd(cA, n), *static_cast<NonDestructiveTriMesh*>(mp), dt_real);
    outv(Fv, F);
}

void ref_force_bending(void* mp, int32_t n, const double* X, const double* x, double* F) {
    Quiet q;
    Eigen::VectorXd Fv(3 * n);
    Fv.setZero();
    calculateBendingForce2D(Fv, v3(X, n), v3(x, n), *static_cast<NonDestructiveTriMesh*>(mp));
    outv(Fv, F);
}

void ref_force_area(void* mp, int32_t n, const double* X, const double* x, double tot_area, double* F) {
    Quiet q;
    Eigen::VectorXd Fv(3 * n);
    Fv.setZero();
    calculateAreaConstraintForce(Fv, v3(X, n), v3(x, n), *static_cast<NonDestructiveTriMesh*>(mp), tot_area);
    outv(Fv, F);
}

void ref_update_fa(void* mcell, int32_t n, double* cA, double* cC, double* fau, double dt_real, const double* X,
                   const double* x, void* msub, int32_t ns, const double* Xs, const double* xs, double kint) {
    Quiet q;
    auto a = vd(cA, n), c = vd(cC, n);
    auto f = v3(fau, n);
    updateFA(a, c, f, dt_real, v3(X, n), v3(x, n), *static_cast<NonDestructiveTriMesh*>(mcell), v3(Xs, ns), v3(xs, ns),
             *static_cast<NonDestructiveTriMesh*>(msub), kint);
    std::memcpy(cA, a.data(), sizeof(double) * n);
    std::memcpy(cC, c.data(), sizeof(double) * n);
    out3(f, fau);
}

void ref_update_forces(void* mp, int32_t n, const double* X, const double* x, double* V, const double* Vh, double* A,
                       double* ea, double* cA, double* cC, double* fau, double dt, double dt_real, double t_tot,
                       uint32_t seed, uint32_t stream, uint64_t call) {
    Quiet q;
    ref_rng_set(seed, stream, call);
    auto Vv = v3(V, n), Vhv = v3(Vh, n), Av = v3(A, n), f = v3(fau, n);
    auto eav = v6(ea, n);
    auto a = vd(cA, n), b = std::vector<double>(n, 0.0), c = vd(cC, n);
    updateForces_Explicit(v3(X, n), v3(x, n), Vv, Vhv, Av, eav, a, b, c, f, dt, dt_real,
                          *static_cast<NonDestructiveTriMesh*>(mp), t_tot);
    out3(Vv, V);
    out3(Av, A);
    out6(eav, ea);
}

void ref_update_forces_subs(void* msub, int32_t ns, const double* Xs, const double* xs, double* Vs, const double* Vhs,
                            double* As, double* eas, double dt, double dt_real, double t_tot, double* fau,
                            const double* cC, void* mcell, int32_t n, const double* xcell) {
    Quiet q;
    auto Vv = v3(Vs, ns), Vhv = v3(Vhs, ns), Av = v3(As, ns), f = v3(fau, n);
    auto eav = v6(eas, ns);
    updateForces_Explicit(v3(Xs, ns), v3(xs, ns), Vv, Vhv, Av, eav, dt, dt_real,
                          *static_cast<NonDestructiveTriMesh*>(msub), t_tot, f, vd(cC, n), v3(xcell, n),
                          *static_cast<NonDestructiveTriMesh*>(mcell));
    out3(Vv, Vs);
    out3(Av, As);
    out6(eav, eas);
}

void ref_force_fa_subs(void* msub, int32_t ns, const double* Xs, const double* xs, const double* cC, void* mcell,
                       int32_t n, const double* xcell, const double* fau, double kint, double* F) {
    Quiet q;
    auto f = v3(fau, n);
    Eigen::VectorXd Fv(3 * ns);
    Fv.setZero();
    calculateForce_FA_subs(Fv, v3(Xs, ns), v3(xs, ns), *static_cast<NonDestructiveTriMesh*>(msub), vd(cC, n),
                           v3(xcell, n), f, *static_cast<NonDestructiveTriMesh*>(mcell), kint);
    outv(Fv, F);
}

// Full explicit steps in the order of advance_sim (cellBP/main.cpp:168-408) with El Topo's
// integrate taking the full step (actual_dt = dt) and a substrate that does not move
// (main.cpp:299).  kint is what main.cpp passes to updateFA (k1: 1000, k31: 31000, kMD: -1).
void ref_steps(void* mcell, int32_t n, double* x, double* V, double* A, double* ea, double* cA, double* cC,
               double* fau, void* msub, int32_t ns, const double* Xs, double kint, double dt, int32_t nsteps,
               double* t_cur, uint32_t seed, uint32_t stream, uint64_t* call) {
    Quiet q;
    const NonDestructiveTriMesh& mc = *static_cast<NonDestructiveTriMesh*>(mcell);
    const NonDestructiveTriMesh& msb = *static_cast<NonDestructiveTriMesh*>(msub);
    auto xv = v3(x, n), Vv = v3(V, n), Av = v3(A, n), f = v3(fau, n);
    auto eav = v6(ea, n);
    auto a = vd(cA, n), b = std::vector<double>(n, 0.0), c = vd(cC, n);
    auto Xsv = v3(Xs, ns);
    ref_rng_set(seed, stream, *call);
    double t = *t_cur;
    for (int s = 0; s < nsteps; ++s) {
        std::vector<Vec3d> Vh(n), xn(n);
        driverVelocities_Explicit(xv, Vv, Vh, Av, dt);
        for (int i = 0; i < n; ++i) xn[i] = xv[i] + dt * Vh[i];
        updateFA(a, c, f, dt, xv, xn, mc, Xsv, Xsv, msb, kint);
        updateForces_Explicit(xv, xn, Vv, Vh, Av, eav, a, b, c, f, dt, dt, mc, t);
        xv = xn;
        t += dt;  // sim->m_curr_t += accum_dt (main.cpp:407)
    }
    *t_cur = t;
    *call = ref_rng_calls();
    out3(xv, x);
    out3(Vv, V);
    out3(Av, A);
    out6(eav, ea);
    out3(f, fau);
    std::memcpy(cA, a.data(), sizeof(double) * n);
    std::memcpy(cC, c.data(), sizeof(double) * n);
}

// The reference's VTK frame writers (cellBP/iomesh.cpp:690-1047): format 0 positions and
// triangles (:690), 1 strain measure and bond vectors (:730, the substrate's frames), 2
// concentrations, strain measure and integrin force (:844, the cell's frames; the kMD
// variant takes kint, k1 and k31 do not).
void ref_write_vtk(void* mp, int32_t format, int32_t n, const double* x, const double* cA, const double* cC,
                   const double* fau, const double* ea, double time, double kint, const char* path) {
    const NonDestructiveTriMesh& m = *static_cast<NonDestructiveTriMesh*>(mp);
    const std::vector<Vec3d> xv = v3(x, n);
    if (format == 0) {
        write_vtk(m, xv, time, path);
        return;
    }
    const std::vector<Vec3d> fv = v3(fau, n);
    std::vector<Eigen::VectorXd> ev = v6(ea, n);
    if (format == 1) {
        write_vtk(m, xv, ev, fv, time, path);
        return;
    }
    const std::vector<double> a = vd(cA, n), b(n, 0.0), c = vd(cC, n);
#ifdef WCFE_REF_WRITER_KINT
    write_vtk(m, xv, a, b, c, fv, ev, time, path, kint);
#else
    (void)kint;
    write_vtk(m, xv, a, b, c, fv, ev, time, path);
#endif
}

}  // extern "C"
