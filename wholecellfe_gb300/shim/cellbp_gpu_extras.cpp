// cellbp_gpu_extras.cpp — optional additions to the reference's cellBP driver on top of the
// drop-in UL_growth_gpu.cpp (same engine and cell): a deformable substrate coupled to the
// cell, state carried on the device through El Topo's remeshing, frames written without
// stalling the stepping, and the batched exchange of many cells.  Compiled inside cellBP
// against the reference's headers (surftrack.h for the remeshing hook).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "nondestructivetrimesh.h"
#include "surftrack.h"
#include "vec.h"
#include "wcfe.h"

extern wcfe_engine* g_eng;   // UL_growth_gpu.cpp
extern int32_t g_cell;
extern char g_output_path[256];   // main.cpp:121

// A driver that moves the substrate adds it as a second cell of the same FP64 engine and
// couples the two once; wcfe_engine_step then advances the cell and its substrate together
// (the per-function mirrors refuse a coupled engine).
static int32_t g_sub = -1;
void add_deformable_substrate(const NonDestructiveTriMesh& ms, const std::vector<Vec3d>& Xs) {
    std::vector<int32_t> tri(3 * ms.num_triangles());
    for (size_t t = 0; t < ms.num_triangles(); ++t)
        for (int a = 0; a < 3; ++a) tri[3 * t + a] = (int32_t)ms.get_triangle(t)[a];
    wcfe_params ps;
    wcfe_params_default(&ps, WCFE_VARIANT_KMD);   // the cell's variant
    ps.mu = 1.0e6;                                // UL:726
    wcfe_cell_create(g_eng, (int32_t)Xs.size(), (int32_t)ms.num_triangles(), tri.data(), nullptr, nullptr, nullptr,
                     &ps, &g_sub);
    wcfe_cell_set_state(g_eng, g_sub, &Xs[0][0], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    wcfe_cell_couple_substrate(g_eng, g_cell, g_sub, 0.05);
}

// After improve_mesh / defrag_mesh (main.cpp:191-192): El Topo's change list instead of a
// re-upload of every field.  info: captured by a SurfTrackObserver's
// operationOccurred(const SurfTrack&, const SurfTrack::PostDefragInfo&) during defrag_mesh.
void sync_after_remesh(SurfTrack& s, const SurfTrack::PostDefragInfo& info) {
    std::vector<int32_t> ab, keep, tri;
    for (const VertexUpdateEvent& ev : s.m_vertex_change_history)   // splits, in order
        if (ev.is_remove == VertexUpdateEvent::VERTEX_ADD) {
            ab.push_back((int32_t)ev.split_edge[0]);
            ab.push_back((int32_t)ev.split_edge[1]);
        }
    for (const Vec2st& m : info.m_defragged_vertex_map) keep.push_back((int32_t)m[0]);
    for (size_t t = 0; t < s.m_mesh.num_triangles(); ++t)
        for (int a = 0; a < 3; ++a) tri.push_back((int32_t)s.m_mesh.get_triangle(t)[a]);
    const std::vector<Vec3d>& x = s.get_positions();
    wcfe_cell_remesh(g_eng, g_cell, (int32_t)ab.size() / 2, ab.data(), (int32_t)keep.size(), keep.data(),
                     (int32_t)tri.size() / 3, tri.data(), nullptr, nullptr, nullptr, &x[0][0]);
    s.m_vertex_change_history.clear();
}

// The frame output in place of the driver's write_vtk calls (main.cpp:447-454, :721-723):
// a gather on the engine stream, a pinned copy and a writer thread format the file.
static wcfe_frames* g_frames = nullptr;   // wcfe_frames_create(g_eng, 4, 2, &g_frames) at start-up
void write_cell_frame(double t, double kint, int frame) {
    char path[256];
    std::snprintf(path, sizeof path, "%s/cell_frame%04d.vtk", g_output_path, frame);
    wcfe_frames_write(g_frames, g_cell, 2, t, kint, path);   // iomesh.cpp:844 format
}
// before exit: wcfe_frames_flush(g_frames); wcfe_frames_destroy(g_frames);

// Many cells coupled to host integrators: one step of every cell through the packed
// exchange; x_buf holds [sum n][3] doubles (page-locked for asynchronous copies).
void step_all_cells(wcfe_engine* eng, double dt, double dt_real, double* x_buf) {
    wcfe_engine_predict(eng, dt, x_buf);             // x* of every cell -> x_buf
    // the host integrates each cell's slice of x_buf in place (El Topo's integrate)
    wcfe_engine_update(eng, dt, dt_real, x_buf);     // updateFA + updateForces_Explicit of every cell
}
