// wcfe_vtk.cu — VTK frame output in the reference's formats (cellBP/iomesh.cpp:690-1047),
// byte for byte, without stalling the stepping stream.
//
// A write packs one cell's current state on the engine's stream (a gather kernel that
// reads the ping-pong parity on the device and decodes the float-float layout of a mixed
// engine into binary64) into a device staging slot, copies it to pinned host memory on
// the writer's own stream, and hands it to a host writer thread, which formats the text
// and writes the file.  The engine stream only pays for the gather kernel.
//
// Text formatting follows std::ostream's defaults, which print a double like printf
// "%g" (precision 6), and "%.6f" after `std::fixed` (the strain-frame writer switches to
// fixed after its POINTS header, iomesh.cpp:737); std::to_chars gives exactly those
// strings.  The derived per-vertex quantities repeat the writers' arithmetic: the
// strain measure sqrt(det((I - 2 ea)^-1)) with the 3 x 3 cofactor inverse and
// determinant in Eigen's operation order, and the integrin force column of each
// variant (iomesh.cpp:919-956).
#include <cuda_runtime.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "wcfe_frames.h"

namespace wcfe {
namespace {

// ---------------------------------------------------------------------------- gather
// out (binary64): x [3n], fau [3n], ea [6n], cA [n], cC [n], then the cell's clock
__global__ void k_frame_gather(CellDev c, int mixed, double* __restrict__ out) {
    const int n = c.nv;
    const int par = c.ctl[0];
    const size_t N = (size_t)n;
    double* X = out;
    double* F = out + 3 * N;
    double* E = out + 6 * N;
    double* CA = out + 12 * N;
    double* CC = out + 13 * N;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        if (!mixed) {
            const double4 x = c.pos[par][v], f = c.fau[v];
            X[3 * v] = x.x; X[3 * v + 1] = x.y; X[3 * v + 2] = x.z;
            F[3 * v] = f.x; F[3 * v + 1] = f.y; F[3 * v + 2] = f.z;
            const double* e = c.ea[par] + 6 * (size_t)v;
#pragma unroll
            for (int q = 0; q < 6; ++q) E[6 * v + q] = e[q];
            CA[v] = c.cA[v];
            CC[v] = c.cC[v];
        } else {   // hi planes then lo planes (see the mixed form's state layout)
            const float4* ph = reinterpret_cast<const float4*>(c.pos[par]);
            const float4* fh = reinterpret_cast<const float4*>(c.fau);
            const float4 xh = ph[v], xl = ph[N + v], uh = fh[v], ul = fh[N + v];
            // triple-float x, y (third floats in the w slots): (h + m) exact, one rounding for + l
            X[3 * v] = ((double)xh.x + (double)xl.x) + (double)xh.w;
            X[3 * v + 1] = ((double)xh.y + (double)xl.y) + (double)xl.w;
            X[3 * v + 2] = (double)xh.z + (double)xl.z;
            F[3 * v] = (double)uh.x + (double)ul.x;
            F[3 * v + 1] = (double)uh.y + (double)ul.y;
            F[3 * v + 2] = (double)uh.z + (double)ul.z;
            const float4* eh = reinterpret_cast<const float4*>(c.ea[par]);
            const float4 a = eh[v], b = eh[N + v], s = eh[2 * N + v];
            E[6 * v] = (double)a.x + (double)b.x;
            E[6 * v + 1] = (double)a.y + (double)b.y;
            E[6 * v + 2] = (double)a.z + (double)b.z;
            E[6 * v + 3] = (double)a.w + (double)b.w;
            E[6 * v + 4] = (double)s.x + (double)s.z;
            E[6 * v + 5] = (double)s.y + (double)s.w;
            const float* ah = reinterpret_cast<const float*>(c.cA);
            const float* ch = reinterpret_cast<const float*>(c.cC);
            CA[v] = (double)ah[v] + (double)ah[N + v];
            CC[v] = (double)ch[v] + (double)ch[N + v];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[14 * N] = c.clk[0];
}

// ---------------------------------------------------------------------------- text
struct Text {
    std::string s;
    void put(const char* t) { s += t; }
    void g(double v) {   // std::ostream default: %g, precision 6
        char b[64];
        const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::general, 6);
        s.append(b, r.ptr);
    }
    void f(double v) {   // after std::fixed: %.6f
        char b[400];
        const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::fixed, 6);
        s.append(b, r.ptr);
    }
    void i(long long v) {
        char b[32];
        const auto r = std::to_chars(b, b + sizeof b, v);
        s.append(b, r.ptr);
    }
};

// Eigen's 3 x 3 cofactor C(i, j) = m(i1, j1) m(i2, j2) - m(i1, j2) m(i2, j1), i1 = (i + 1) % 3 ...
inline double cof3(const double (&m)[3][3], int i, int j) {
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return m[i1][j1] * m[i2][j2] - m[i1][j2] * m[i2][j1];
}

// sqrt(det(be)) with be = (I - 2 ea)^-1: the area change of the strain frames (iomesh.cpp:905-919)
double strain_theta(const double* ea) {
    const double E[3][3] = {{ea[0], ea[3], ea[4]}, {ea[3], ea[1], ea[5]}, {ea[4], ea[5], ea[2]}};
    double a[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r][c] = (r == c ? 1.0 : 0.0) - 2.0 * E[r][c];
    // inverse: the cofactors of column 0, det from them, then the adjugate times 1/det
    const double c0 = cof3(a, 0, 0), c1 = cof3(a, 1, 0), c2 = cof3(a, 2, 0);
    const double det = (c0 * a[0][0] + c1 * a[1][0]) + c2 * a[2][0];
    const double inv = 1.0 / det;
    double b[3][3];
    b[0][0] = c0 * inv; b[0][1] = c1 * inv; b[0][2] = c2 * inv;
    b[1][0] = cof3(a, 0, 1) * inv; b[1][1] = cof3(a, 1, 1) * inv; b[1][2] = cof3(a, 2, 1) * inv;
    b[2][0] = cof3(a, 0, 2) * inv; b[2][1] = cof3(a, 1, 2) * inv; b[2][2] = cof3(a, 2, 2) * inv;
    // determinant: m00 (m11 m22 - m12 m21) - m01 (m10 m22 - m12 m20) + m02 (m10 m21 - m11 m20)
    const double d = (b[0][0] * (b[1][1] * b[2][2] - b[1][2] * b[2][1]) -
                      b[0][1] * (b[1][0] * b[2][2] - b[1][2] * b[2][0])) +
                     b[0][2] * (b[1][0] * b[2][1] - b[1][1] * b[2][0]);
    return std::sqrt(d);
}

// the fourth scalar of the concentration frames: the MD table / kint |u| spring force of the
// kMD writer (iomesh.cpp:924-949), or |k_FA u| in the plane of the k1 and k31 writers
double force_column(const double* u, int law, double kint, double k_fa) {
    if (law == WCFE_LAW_MD_TABLE) {
        static const double px[6] = {0., 2.51250583e-03, 4.40265201e-03, 5.91408228e-03, 11.76817302e-03, 17.001e-03};
        static const double py[6] = {-7.15514497, 71.80501308, 356.62420075, 356.96656556, 126.21811585,
                                     528.40481124};
        static const double km[6] = {31426.8556, 99485.86235, 67080.67086, -7908.39043, 21978.66923, 76858.39733};
        const double D = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (kint >= 0) return kint * D;
        double f = 0.0;
        for (int j = 0; j < 5; ++j) {
            if (D < px[j + 1] && D >= px[j]) f = py[j] + km[j] * (D - px[j]);
            else if (D >= px[5]) f = py[5] + km[5] * (D - px[5]);
        }
        return f;
    }
    const double fx = k_fa * u[0], fy = k_fa * u[1];
    return std::sqrt(fx * fx + fy * fy);
}

void vtk_text(Text& t, int format, int n, int nt, const int32_t* tri, const double* x, const double* cA,
              const double* cC, const double* fau, const double* ea, double time, double kint, int law, double k_fa) {
    t.put("# vtk DataFile Version 2.0\nCellBP Time: ");
    t.g(time);
    t.put("\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS ");
    t.i(n);
    t.put(" double\n");
    const bool fixed = format == 1;
    auto num = [&](double v) { fixed ? t.f(v) : t.g(v); };
    for (int v = 0; v < n; ++v) {
        num(x[3 * v]);
        t.put(" ");
        num(x[3 * v + 1]);
        t.put(" ");
        num(x[3 * v + 2]);
        t.put("\n");
    }
    t.put("CELLS ");
    t.i(nt);
    t.put(" ");
    t.i(4LL * nt);
    t.put("\n");
    for (int e = 0; e < nt; ++e) {
        t.put("3");
        for (int k = 0; k < 3; ++k) {
            t.put(" ");
            t.i(tri[3 * e + k]);
        }
        t.put("\n");
    }
    t.put("CELL_TYPES ");
    t.i(nt);
    t.put("\n");
    for (int e = 0; e < nt; ++e) t.put("5\n");
    if (format == 0) return;
    t.put("POINT_DATA ");
    t.i(n);
    if (format == 1) {
        t.put("\nSCALARS theta_e float 1\nLOOKUP_TABLE default\n");
        for (int v = 0; v < n; ++v) {
            t.f(strain_theta(ea + 6 * v));
            t.put("\n");
        }
    } else {
        t.put("\nSCALARS concentrations float 4\nLOOKUP_TABLE default\n");
        for (int v = 0; v < n; ++v) {
            t.g(cA[v]);
            t.put(" ");
            t.g(strain_theta(ea + 6 * v));
            t.put(" ");
            t.g(cC[v]);
            t.put(" ");
            t.g(force_column(fau + 3 * v, law, kint, k_fa));
            t.put("\n");
        }
    }
    t.put("VECTORS fa_u float\n");
    for (int v = 0; v < n; ++v) {
        num(fau[3 * v]);
        t.put(" ");
        num(fau[3 * v + 1]);
        t.put(" ");
        num(fau[3 * v + 2]);
        t.put("\n");
    }
}

// ---------------------------------------------------------------------------- writer
struct Slot {
    double* dev = nullptr;     // staging buffer on the device
    double* host = nullptr;    // pinned copy
    size_t cap = 0;            // doubles
    cudaEvent_t gathered = nullptr, copied = nullptr;
    bool busy = false;
};
struct Job {
    int slot, format, n, nt, law;
    std::vector<int32_t> tri;
    double time, kint, k_fa;
    bool clock_time;
    std::string path;
};

}  // namespace
}  // namespace wcfe

struct wcfe_frames {
    wcfe_engine* eng = nullptr;
    int device = 0;
    cudaStream_t side = nullptr;
    std::vector<wcfe::Slot> slots;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_job, cv_slot;
    std::deque<wcfe::Job> queue;
    int in_flight = 0;
    bool stop = false;
    std::string error;         // the first failed write
};

namespace wcfe {
namespace {

void writer_main(wcfe_frames* f) {
    cudaSetDevice(f->device);
    for (;;) {
        Job job;
        {
            std::unique_lock<std::mutex> lk(f->mu);
            f->cv_job.wait(lk, [&] { return f->stop || !f->queue.empty(); });
            if (f->queue.empty()) return;
            job = std::move(f->queue.front());
            f->queue.pop_front();
        }
        Slot& s = f->slots[job.slot];
        std::string err;
        if (cudaEventSynchronize(s.copied) != cudaSuccess) err = "frame copy failed";
        if (err.empty()) {
            const size_t N = (size_t)job.n;
            const double* h = s.host;
            Text t;
            t.s.reserve(64 * N + 16 * (size_t)job.nt + 256);
            vtk_text(t, job.format, job.n, job.nt, job.tri.data(), h, h + 12 * N, h + 13 * N, h + 3 * N, h + 6 * N,
                     job.clock_time ? h[14 * N] : job.time, job.kint, job.law, job.k_fa);
            FILE* fp = std::fopen(job.path.c_str(), "wb");
            if (!fp) err = "cannot open " + job.path;
            else {
                if (std::fwrite(t.s.data(), 1, t.s.size(), fp) != t.s.size()) err = "cannot write " + job.path;
                if (std::fclose(fp) != 0 && err.empty()) err = "cannot write " + job.path;
            }
        }
        {
            std::lock_guard<std::mutex> lk(f->mu);
            if (!err.empty() && f->error.empty()) f->error = err;
            s.busy = false;
            --f->in_flight;
        }
        f->cv_slot.notify_all();
    }
}

}  // namespace
}  // namespace wcfe

using namespace wcfe;

extern "C" {

int wcfe_vtk_format(int32_t format, int32_t n, int32_t nt, const int32_t* tri, const double* x, const double* cA,
                    const double* cC, const double* fau, const double* ea, double time, double kint, int32_t law,
                    double k_fa, char* out, int64_t cap, int64_t* len) {
    if (format < 0 || format > 2 || n < 0 || nt < 0 || (nt && !tri) || (n && !x) || !len)
        return set_error("bad argument", WCFE_ERR_ARG);
    if (format >= 1 && n && (!fau || !ea)) return set_error("bad argument", WCFE_ERR_ARG);
    if (format == 2 && n && (!cA || !cC)) return set_error("bad argument", WCFE_ERR_ARG);
    Text t;
    vtk_text(t, format, n, nt, tri, x, cA, cC, fau, ea, time, kint, law, k_fa);
    *len = (int64_t)t.s.size();
    if (out && cap > 0) std::memcpy(out, t.s.data(), (size_t)std::min<int64_t>(cap, *len));
    return WCFE_OK;
}

int wcfe_frames_create(wcfe_engine* e, int32_t slots, int32_t threads, wcfe_frames** out) {
    if (!e || !out || slots < 1 || slots > 64 || threads < 1 || threads > 16) return set_error("bad argument", WCFE_ERR_ARG);
    wcfe_frames* f = new wcfe_frames();
    f->eng = e;
    f->device = engine_device(e);
    cudaSetDevice(f->device);
    if (cudaStreamCreateWithFlags(&f->side, cudaStreamNonBlocking) != cudaSuccess) {
        delete f;
        return set_error("cudaStreamCreateWithFlags failed", WCFE_ERR_CUDA);
    }
    f->slots.resize((size_t)slots);
    for (auto& s : f->slots)
        if (cudaEventCreateWithFlags(&s.gathered, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming) != cudaSuccess) {
            wcfe_frames_destroy(f);
            return set_error("cudaEventCreate failed", WCFE_ERR_CUDA);
        }
    for (int i = 0; i < threads; ++i) f->threads.emplace_back(writer_main, f);
    *out = f;
    return WCFE_OK;
}

int wcfe_frames_write(wcfe_frames* f, int32_t cell, int32_t format, double time, double kint, const char* path) {
    if (!f || !path || format < 0 || format > 2) return set_error("bad argument", WCFE_ERR_ARG);
    FrameSource src;
    int r = engine_frame_source(f->eng, cell, &src);
    if (r) return r;
    const size_t need = 14 * (size_t)src.nv + 1;
    int k = -1;
    {
        std::unique_lock<std::mutex> lk(f->mu);
        f->cv_slot.wait(lk, [&] {
            for (size_t i = 0; i < f->slots.size(); ++i)
                if (!f->slots[i].busy) return true;
            return false;
        });
        for (size_t i = 0; i < f->slots.size(); ++i)
            if (!f->slots[i].busy) {
                k = (int)i;
                break;
            }
        f->slots[k].busy = true;
        ++f->in_flight;
    }
    Slot& s = f->slots[k];
    auto release = [&](const char* msg) {
        {
            std::lock_guard<std::mutex> lk(f->mu);
            s.busy = false;
            --f->in_flight;
        }
        f->cv_slot.notify_all();
        return set_error(msg, WCFE_ERR_CUDA);
    };
    cudaSetDevice(src.device);
    if (s.cap < need) {   // a free slot has no copy in flight
        if (s.dev) cudaFree(s.dev);
        if (s.host) cudaFreeHost(s.host);
        s.dev = nullptr;
        s.host = nullptr;
        s.cap = 0;
        if (cudaMalloc(&s.dev, sizeof(double) * need) != cudaSuccess ||
            cudaMallocHost(&s.host, sizeof(double) * need) != cudaSuccess)
            return release("frame staging allocation failed");
        s.cap = need;
    }
    const int grid = std::max(1, std::min((src.nv + 255) / 256, 1024));
    k_frame_gather<<<grid, 256, 0, src.stream>>>(src.dev, src.mixed, s.dev);
    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(s.gathered, src.stream) != cudaSuccess ||
        cudaStreamWaitEvent(f->side, s.gathered, 0) != cudaSuccess ||
        cudaMemcpyAsync(s.host, s.dev, sizeof(double) * need, cudaMemcpyDeviceToHost, f->side) != cudaSuccess ||
        cudaEventRecord(s.copied, f->side) != cudaSuccess)
        return release("frame gather or copy failed");
    Job job;
    job.slot = k;
    job.format = format;
    job.n = src.nv;
    job.nt = src.nt;
    job.law = src.prm.force_law;
    job.k_fa = src.prm.k_lin;
    job.tri = std::move(src.tri);
    job.time = time;
    job.clock_time = std::isnan(time);
    job.kint = kint;
    job.path = path;
    {
        std::lock_guard<std::mutex> lk(f->mu);
        f->queue.push_back(std::move(job));
    }
    f->cv_job.notify_one();
    return WCFE_OK;
}

int wcfe_frames_flush(wcfe_frames* f) {
    if (!f) return set_error("bad argument", WCFE_ERR_ARG);
    std::unique_lock<std::mutex> lk(f->mu);
    f->cv_slot.wait(lk, [&] { return f->in_flight == 0; });
    if (!f->error.empty()) {
        std::string e = f->error;
        f->error.clear();
        return set_error(e.c_str(), WCFE_ERR_STATE);
    }
    return WCFE_OK;
}

int wcfe_frames_destroy(wcfe_frames* f) {
    if (!f) return WCFE_OK;
    {
        std::unique_lock<std::mutex> lk(f->mu);
        f->cv_slot.wait(lk, [&] { return f->in_flight == 0; });
        f->stop = true;
    }
    f->cv_job.notify_all();
    for (auto& t : f->threads) t.join();
    cudaSetDevice(f->device);
    for (auto& s : f->slots) {
        if (s.dev) cudaFree(s.dev);
        if (s.host) cudaFreeHost(s.host);
        if (s.gathered) cudaEventDestroy(s.gathered);
        if (s.copied) cudaEventDestroy(s.copied);
    }
    if (f->side) cudaStreamDestroy(f->side);
    delete f;
    return WCFE_OK;
}

}  // extern "C"
