// wcfe_topology.h — host-side preprocessing of a cell's connectivity (integer
// bookkeeping only; everything here is exact and is compared bit for bit with
// the reference's NonDestructiveTriMesh in the tests).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace wcfe {

struct Topology {
    int32_t nv = 0, nt = 0, nb = 0;
    std::vector<int32_t> tri;        // [3 nt]
    std::vector<int32_t> vt_ptr;     // [nv+1] vertex -> triangle map (mesh order)
    std::vector<int32_t> vt_idx;     // [vt_ptr[nv]]
    std::vector<uint8_t> bnd;        // [nv] boundary flags
    std::vector<int32_t> bnd_rank;   // [nv] index among boundary vertices in vertex order, -1 interior
    std::vector<int32_t> bnd_cptr;   // [nb+1]
    std::vector<int32_t> bnd_cand;   // [2 * bnd_cptr[nb]] (nj, nint) pairs, UL:1500-1531 scan order
    std::vector<int32_t> bnd_optr;   // [nb+1] directed boundary edges leaving each boundary vertex
    std::vector<int32_t> bnd_out;    // their end vertices (edge direction as in its triangle)
};

struct Patches {
    int32_t np = 0, emax = 0, max_ne = 0;
    int32_t max_nvp = 0, max_nh = 0, max_nc = 0;
    std::vector<int32_t> patch;      // [4 np] (v0, nvp, e0, ne)
    std::vector<int32_t> elems;      // element ids of each patch (each patch's list padded to an even length)
    std::vector<uint16_t> vc_code;   // aligned with vt_idx: (slot << 2) | corner
    // staging description of each patch (the mixed form's pipelined patch kernel):
    std::vector<int32_t> xinfo;      // [4 np] (h0, nh, c0, nc): halo list offset and count; one-ring codes
                                     //        vc_code[c0 .. c0 + nc) of the owned vertices
    std::vector<int32_t> halo;       // vertices of a patch's elements outside its owned range, ascending
    std::vector<uint16_t> loc;       // [4 per elems entry] corners as patch-local vertex indices:
                                     //        owned v -> v - v0, halo k -> nvp + k; 4th entry 0
};

// Returns "" on success or an error message.
std::string build_topology(Topology& T, int32_t nv, int32_t nt, const int32_t* tri, const int32_t* vt_ptr,
                           const int32_t* vt_idx, const uint8_t* bnd);
// Greedy patches over consecutive vertex ranges with at most emax elements each.
std::string build_patches(Patches& P, const Topology& T, int32_t emax);

struct SubGrid {
    double ox = 0, oy = 0, inv_h = 1;
    int32_t gx = 0, gy = 0;
    std::vector<int32_t> cell_ptr, cell_tri;
};
// Uniform grid over the substrate triangles' (slightly padded) bounding boxes.
void build_subgrid(SubGrid& G, int32_t nv, int32_t nt, const int32_t* tri, const double* X, double margin = 0.0);

}  // namespace wcfe
