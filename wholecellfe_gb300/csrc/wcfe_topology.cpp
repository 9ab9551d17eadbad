// wcfe_topology.cpp — host-side connectivity preprocessing (see wcfe_topology.h).
#include "wcfe_topology.h"

#include <algorithm>
#include <cmath>
#include <unordered_map>

namespace wcfe {

std::string build_topology(Topology& T, int32_t nv, int32_t nt, const int32_t* tri, const int32_t* vt_ptr,
                           const int32_t* vt_idx, const uint8_t* bnd) {
    if (nv <= 0 || nt <= 0 || !tri) return "empty mesh";
    T.nv = nv;
    T.nt = nt;
    T.tri.assign(tri, tri + 3 * (size_t)nt);
    for (int64_t k = 0; k < 3 * (int64_t)nt; ++k)
        if (T.tri[k] < 0 || T.tri[k] >= nv) return "triangle vertex index out of range";
    // vertex -> triangle map: the caller's (mesh order) or ascending triangle order
    if (vt_ptr && vt_idx) {
        T.vt_ptr.assign(vt_ptr, vt_ptr + nv + 1);
        if (T.vt_ptr[0] != 0) return "vt_ptr[0] != 0";
        for (int v = 0; v < nv; ++v)
            if (T.vt_ptr[v + 1] < T.vt_ptr[v]) return "vt_ptr not monotone";
        T.vt_idx.assign(vt_idx, vt_idx + T.vt_ptr[nv]);
        for (int v = 0; v < nv; ++v)
            for (int k = T.vt_ptr[v]; k < T.vt_ptr[v + 1]; ++k) {
                int t = T.vt_idx[k];
                if (t < 0 || t >= nt) return "vt_idx out of range";
                if (T.tri[3 * t] != v && T.tri[3 * t + 1] != v && T.tri[3 * t + 2] != v)
                    return "vt_idx lists a triangle that does not contain the vertex";
            }
    } else {
        T.vt_ptr.assign(nv + 1, 0);
        for (int64_t k = 0; k < 3 * (int64_t)nt; ++k) T.vt_ptr[T.tri[k] + 1]++;
        for (int v = 0; v < nv; ++v) T.vt_ptr[v + 1] += T.vt_ptr[v];
        T.vt_idx.assign(T.vt_ptr[nv], 0);
        std::vector<int32_t> fill(T.vt_ptr.begin(), T.vt_ptr.end() - 1);
        for (int t = 0; t < nt; ++t)
            for (int a = 0; a < 3; ++a) T.vt_idx[fill[T.tri[3 * t + a]]++] = t;
    }
    for (int v = 0; v < nv; ++v)
        if (T.vt_ptr[v + 1] == T.vt_ptr[v]) return "vertex without triangles";
    // boundary flags: caller's or odd edge counts (rebuild_auxiliary_structures)
    if (bnd) {
        T.bnd.assign(bnd, bnd + nv);
        for (auto& b : T.bnd) b = b ? 1 : 0;
    } else {
        std::unordered_map<int64_t, int32_t> cnt;
        cnt.reserve(3 * (size_t)nt);
        for (int t = 0; t < nt; ++t)
            for (int a = 0; a < 3; ++a) {
                int64_t u = T.tri[3 * t + a], w = T.tri[3 * t + (a + 1) % 3];
                if (u > w) std::swap(u, w);
                cnt[u * nv + w]++;
            }
        T.bnd.assign(nv, 0);
        for (auto& kv : cnt)
            if (kv.second % 2) {
                T.bnd[kv.first / nv] = 1;
                T.bnd[kv.first % nv] = 1;
            }
    }
    // boundary neighbour candidates in the scan order of UL:1500-1531
    T.bnd_rank.assign(nv, -1);
    T.bnd_cptr.assign(1, 0);
    T.bnd_cand.clear();
    int nb = 0;
    for (int v = 0; v < nv; ++v) {
        if (!T.bnd[v]) continue;
        T.bnd_rank[v] = nb++;
        for (int k = T.vt_ptr[v]; k < T.vt_ptr[v + 1]; ++k) {
            const int32_t* t = &T.tri[3 * T.vt_idx[k]];
            for (int a = 0; a < 3; ++a) {
                int nj = t[a];
                if (T.bnd[nj] && nj != v) {
                    int nint = v;  // the reference leaves it unset for a degenerate triangle
                    for (int b = 0; b < 3; ++b)
                        if (t[b] != nj && t[b] != v) { nint = t[b]; break; }
                    T.bnd_cand.push_back(nj);
                    T.bnd_cand.push_back(nint);
                }
            }
        }
        T.bnd_cptr.push_back((int32_t)(T.bnd_cand.size() / 2));
    }
    T.nb = nb;
    // directed boundary edges: an edge of odd triangle count, oriented as in its triangle
    {
        std::unordered_map<int64_t, int32_t> ecount;
        ecount.reserve(3 * (size_t)nt);
        for (int t = 0; t < nt; ++t)
            for (int a = 0; a < 3; ++a) {
                int64_t u = T.tri[3 * t + a], w = T.tri[3 * t + (a + 1) % 3];
                if (u > w) std::swap(u, w);
                ecount[u * nv + w]++;
            }
        std::vector<std::vector<int32_t>> outs(nb);
        for (int t = 0; t < nt; ++t)
            for (int a = 0; a < 3; ++a) {
                int32_t u = T.tri[3 * t + a], w = T.tri[3 * t + (a + 1) % 3];
                int64_t lo = std::min(u, w), hi = std::max(u, w);
                if (ecount[lo * nv + hi] % 2 && T.bnd_rank[u] >= 0) outs[T.bnd_rank[u]].push_back(w);
            }
        T.bnd_optr.assign(1, 0);
        T.bnd_out.clear();
        for (int r = 0; r < nb; ++r) {
            T.bnd_out.insert(T.bnd_out.end(), outs[r].begin(), outs[r].end());
            T.bnd_optr.push_back((int32_t)T.bnd_out.size());
        }
    }
    return "";
}

std::string build_patches(Patches& P, const Topology& T, int32_t emax) {
    if (emax < 16 || emax > 16383) return "patch element limit out of range";
    P.emax = emax;
    P.patch.clear();
    P.elems.clear();
    P.xinfo.clear();
    P.halo.clear();
    P.loc.clear();
    P.max_nvp = P.max_nh = P.max_nc = 0;
    P.vc_code.assign(T.vt_idx.size(), 0);
    P.max_ne = 0;
    std::vector<int32_t> mark(T.nt, -1), slot(T.nt, 0);
    int v = 0, np = 0;
    while (v < T.nv) {
        const int v0 = v;
        const int e0 = (int)P.elems.size();
        int ne = 0;
        while (v < T.nv) {
            int add = 0;
            for (int k = T.vt_ptr[v]; k < T.vt_ptr[v + 1]; ++k)
                if (mark[T.vt_idx[k]] != np) ++add;
            // the same triangle can repeat in a one-ring only for degenerate meshes; count conservatively
            if (ne + add > emax) {
                if (v == v0) return "a vertex one-ring exceeds the patch element limit";
                break;
            }
            for (int k = T.vt_ptr[v]; k < T.vt_ptr[v + 1]; ++k) {
                int t = T.vt_idx[k];
                if (mark[t] != np) {
                    mark[t] = np;
                    slot[t] = ne++;
                    P.elems.push_back(t);
                }
            }
            ++v;
        }
        for (int u = v0; u < v; ++u)
            for (int k = T.vt_ptr[u]; k < T.vt_ptr[u + 1]; ++k) {
                int t = T.vt_idx[k];
                int corner = (T.tri[3 * t] == u) ? 0 : (T.tri[3 * t + 1] == u ? 1 : 2);
                P.vc_code[k] = (uint16_t)((slot[t] << 2) | corner);
            }
        // halo: vertices of the patch's elements outside [v0, v), ascending
        const int nvp = v - v0;
        std::vector<int32_t> hl;
        for (int j = 0; j < ne; ++j)
            for (int q = 0; q < 3; ++q) {
                const int u = T.tri[3 * P.elems[e0 + j] + q];
                if (u < v0 || u >= v) hl.push_back(u);
            }
        std::sort(hl.begin(), hl.end());
        hl.erase(std::unique(hl.begin(), hl.end()), hl.end());
        if (nvp + (int)hl.size() > 65535) return "a patch touches more than 65535 vertices";
        const int h0 = (int)P.halo.size();
        P.halo.insert(P.halo.end(), hl.begin(), hl.end());
        for (int j = 0; j < ne; ++j) {
            for (int q = 0; q < 3; ++q) {
                const int u = T.tri[3 * P.elems[e0 + j] + q];
                const int l = (u >= v0 && u < v) ? u - v0
                                                 : nvp + (int)(std::lower_bound(hl.begin(), hl.end(), u) - hl.begin());
                P.loc.push_back((uint16_t)l);
            }
            P.loc.push_back(0);
        }
        if (ne & 1) {   // keep every patch's element list at an even offset (16-B aligned loc rows)
            P.elems.push_back(P.elems[e0 + ne - 1]);
            for (int q = 0; q < 4; ++q) P.loc.push_back(0);
        }
        P.patch.push_back(v0);
        P.patch.push_back(nvp);
        P.patch.push_back(e0);
        P.patch.push_back(ne);
        const int c0 = T.vt_ptr[v0], nc = T.vt_ptr[v] - T.vt_ptr[v0];
        P.xinfo.push_back(h0);
        P.xinfo.push_back((int)hl.size());
        P.xinfo.push_back(c0);
        P.xinfo.push_back(nc);
        P.max_ne = std::max(P.max_ne, ne);
        P.max_nvp = std::max(P.max_nvp, nvp);
        P.max_nh = std::max(P.max_nh, (int)hl.size());
        P.max_nc = std::max(P.max_nc, nc);
        ++np;
    }
    P.np = np;
    return "";
}

// margin: extra width around the domain and every triangle's box, so that triangles that
// move by less than it are still found in the grid cells of the points they contain
void build_subgrid(SubGrid& G, int32_t nv, int32_t nt, const int32_t* tri, const double* X, double margin) {
    double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
    for (int v = 0; v < nv; ++v)
        for (int c = 0; c < 2; ++c) {
            lo[c] = std::min(lo[c], X[3 * v + c]);
            hi[c] = std::max(hi[c], X[3 * v + c]);
        }
    double span = std::max(hi[0] - lo[0], hi[1] - lo[1]);
    if (!(span > 0)) span = 1.0;
    double pad = 1e-9 * span + std::max(margin, 0.0);
    lo[0] -= pad; lo[1] -= pad; hi[0] += pad; hi[1] += pad;
    int g = std::max(1, (int)std::ceil(std::sqrt((double)nt) / 1.5));
    double h = std::max(hi[0] - lo[0], hi[1] - lo[1]) / g;
    G.ox = lo[0];
    G.oy = lo[1];
    G.inv_h = 1.0 / h;
    G.gx = std::max(1, (int)std::ceil((hi[0] - lo[0]) / h));
    G.gy = std::max(1, (int)std::ceil((hi[1] - lo[1]) / h));
    std::vector<std::vector<int32_t>> cells((size_t)G.gx * G.gy);
    for (int t = 0; t < nt; ++t) {
        double bl[2] = {1e300, 1e300}, bh[2] = {-1e300, -1e300};
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 2; ++c) {
                double q = X[3 * tri[3 * t + a] + c];
                bl[c] = std::min(bl[c], q);
                bh[c] = std::max(bh[c], q);
            }
        int x0 = std::max(0, (int)std::floor((bl[0] - pad - G.ox) * G.inv_h));
        int x1 = std::min(G.gx - 1, (int)std::floor((bh[0] + pad - G.ox) * G.inv_h));
        int y0 = std::max(0, (int)std::floor((bl[1] - pad - G.oy) * G.inv_h));
        int y1 = std::min(G.gy - 1, (int)std::floor((bh[1] + pad - G.oy) * G.inv_h));
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) cells[(size_t)y * G.gx + x].push_back(t);
    }
    G.cell_ptr.assign(cells.size() + 1, 0);
    G.cell_tri.clear();
    for (size_t k = 0; k < cells.size(); ++k) {
        G.cell_tri.insert(G.cell_tri.end(), cells[k].begin(), cells[k].end());
        G.cell_ptr[k + 1] = (int32_t)G.cell_tri.size();
    }
}

}  // namespace wcfe
