// les_io.cu -- device-resident statistics (les-model src/statistics.cpp) and
// the reference's output files (src/io.cpp) written from device fields.
//
// Statistics: the ten running sums of update_statistics
// (src/statistics.cpp:98-131) live on the device and are accumulated by one
// elementwise kernel per step, so a step loop that collects statistics no
// longer copies the fields to the host; finalize_and_save (:133-186) forms
// the means and Reynolds stresses on the device.  FP64 with the reference's
// operation order (this file is compiled with -fmad=false): bit-identical.
//
// Files: the byte layouts of write_field_vtk (src/io.cpp:225-256),
// write_statistics_vtk (src/statistics.cpp:11-71) and save_state / load_state
// (src/io.cpp:14-120).  Text is formatted as the reference's ostream does
// (default precision: %.6g; the statistics file's values: %.10g; the
// checkpoint time and dt: %.17g), in parallel chunks on host threads.  A write
// from the device first snapshots the fields on the device (a copy at HBM
// speed on the context's stream), then copies the snapshot to pinned host
// memory on a separate stream and formats/writes it on a host thread, so the
// time steps continue while the file is produced.  les_io_wait joins it.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "les_internal.cuh"

using namespace les;

namespace les {

struct IoWork {
    size_t n = 0;
    double* dev = nullptr;          // snapshot: u, v, w, p, nu_t, u_new, v_new, w_new
    uint8_t* dev_mask = nullptr;
    double* host = nullptr;         // pinned copy of the snapshot
    uint8_t* host_mask = nullptr;
    cudaStream_t copy = nullptr;
    cudaEvent_t ready = nullptr;    // snapshot taken (on the context's stream)
    cudaEvent_t copied = nullptr;   // pinned copy complete (on the copy stream)
    std::thread writer;
    les_status result = LES_OK;
    std::string err;
    // statistics
    double* sums = nullptr;         // 10 x n: u, v, w, p, uu, vv, ww, uv, uw, vw
    int samples = 0, start_step = 0;
};

void io_work_free(IoWork* w)
{
    if (!w) return;
    if (w->writer.joinable()) w->writer.join();
    cudaFree(w->dev);
    cudaFree(w->dev_mask);
    cudaFree(w->sums);
    if (w->host) cudaFreeHost(w->host);
    if (w->host_mask) cudaFreeHost(w->host_mask);
    if (w->copy) cudaStreamDestroy(w->copy);
    if (w->ready) cudaEventDestroy(w->ready);
    if (w->copied) cudaEventDestroy(w->copied);
    delete w;
}

}  // namespace les

namespace {

// ---- text formatting ---------------------------------------------------------
// One value as std::ostream prints a double with the given precision and
// default floatfield (the %g conversion).
inline void put_g(std::string& s, double v, int prec)
{
    char buf[40];
    const int k = std::snprintf(buf, sizeof buf, "%.*g", prec, v);
    s.append(buf, (size_t)k);
}

inline void put_i(std::string& s, long long v)
{
    char buf[24];
    const int k = std::snprintf(buf, sizeof buf, "%lld", v);
    s.append(buf, (size_t)k);
}

// Formats lines [0, n) with fmt(i, out) on host threads, in order.
template <class F>
bool write_lines(FILE* f, size_t n, F fmt)
{
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(nt, 32u));
    const size_t chunk = 1 << 16;
    std::vector<std::string> bufs(nt);
    for (size_t base = 0; base < n; base += chunk * nt) {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t) {
            const size_t a = base + t * chunk, b = std::min(n, a + chunk);
            bufs[t].clear();
            if (a >= b) continue;
            th.emplace_back([&, a, b, t] {
                bufs[t].reserve((b - a) * 16);
                for (size_t i = a; i < b; ++i) fmt(i, bufs[t]);
            });
        }
        for (auto& x : th) x.join();
        for (unsigned t = 0; t < nt; ++t)
            if (!bufs[t].empty() && std::fwrite(bufs[t].data(), 1, bufs[t].size(), f) != bufs[t].size()) return false;
    }
    return true;
}

std::string vtk_header(const les_mesh& m, const char* title)
{
    std::string h = "# vtk DataFile Version 3.0\n";
    h += title;
    h += "\nASCII\nDATASET STRUCTURED_POINTS\nDIMENSIONS ";
    put_i(h, m.nx); h += ' '; put_i(h, m.ny); h += ' '; put_i(h, m.nz);
    h += "\nORIGIN 0 0 0\nSPACING ";
    put_g(h, m.dx, 6); h += ' '; put_g(h, m.dy, 6); h += ' '; put_g(h, m.dz, 6);
    h += "\nPOINT_DATA ";
    put_i(h, (long long)(m.nx * m.ny * m.nz));   // int product, as the reference computes it
    h += '\n';
    return h;
}

bool put_str(FILE* f, const std::string& s) { return std::fwrite(s.data(), 1, s.size(), f) == s.size(); }

les_status field_vtk(const les_mesh& m, int step, const double* u, const double* v, const double* w, const double* p,
                     const double* nu_t, const uint8_t* solid, const char* path, std::string* err)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        if (err) *err = std::string("cannot open ") + path + ": " + std::strerror(errno);
        return LES_BAD_ARG;
    }
    const size_t n = (size_t)m.nx * m.ny * m.nz;
    std::string title = "LES output step ";
    put_i(title, step);
    bool ok = put_str(f, vtk_header(m, title.c_str()));
    ok = ok && put_str(f, "VECTORS velocity double\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) {
        put_g(s, u[i], 6); s += ' '; put_g(s, v[i], 6); s += ' '; put_g(s, w[i], 6); s += '\n';
    });
    ok = ok && put_str(f, "SCALARS pressure double 1\nLOOKUP_TABLE default\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) { put_g(s, p[i], 6); s += '\n'; });
    ok = ok && put_str(f, "SCALARS nu_t double 1\nLOOKUP_TABLE default\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) { put_g(s, nu_t[i], 6); s += '\n'; });
    ok = ok && put_str(f, "SCALARS solid int 1\nLOOKUP_TABLE default\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) { s += solid[i] ? "1\n" : "0\n"; });
    ok = (std::fclose(f) == 0) && ok;
    if (!ok && err) *err = std::string("write failed: ") + path;
    return ok ? LES_OK : LES_BAD_ARG;
}

les_status stats_vtk(const les_mesh& m, const double* const* mean4, const double* const* st6, const char* path,
                     std::string* err)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        if (err) *err = std::string("cannot open ") + path + ": " + std::strerror(errno);
        return LES_BAD_ARG;
    }
    const size_t n = (size_t)m.nx * m.ny * m.nz;
    bool ok = put_str(f, vtk_header(m, "Time-averaged statistics"));
    ok = ok && put_str(f, "VECTORS mean_velocity double\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) {
        put_g(s, mean4[0][i], 10); s += ' '; put_g(s, mean4[1][i], 10); s += ' '; put_g(s, mean4[2][i], 10);
        s += '\n';
    });
    ok = ok && put_str(f, "SCALARS mean_pressure double 1\nLOOKUP_TABLE default\n");
    ok = ok && write_lines(f, n, [&](size_t i, std::string& s) { put_g(s, mean4[3][i], 10); s += '\n'; });
    const char* names[6] = {"uu", "vv", "ww", "uv", "uw", "vw"};
    for (int q = 0; q < 6 && ok; ++q) {
        ok = put_str(f, std::string("SCALARS ") + names[q] + "_stress double 1\nLOOKUP_TABLE default\n");
        ok = ok && write_lines(f, n, [&](size_t i, std::string& s) { put_g(s, st6[q][i], 10); s += '\n'; });
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok && err) *err = std::string("write failed: ") + path;
    return ok ? LES_OK : LES_BAD_ARG;
}

std::string join(const char* dir, const char* name) { return std::string(dir) + "/" + name; }

les_status write_checkpoint(const les_mesh& m, const double* const* f5, const uint8_t* solid, double time_sim,
                            double dt, int next_step, const char* dir, const double* const* unew3, std::string* err)
{
    const size_t n = (size_t)m.nx * m.ny * m.nz;
    // metadata (text): next step, then time and dt with max_digits10 = 17
    std::string meta;
    put_i(meta, next_step);
    meta += '\n';
    put_g(meta, time_sim, 17);
    meta += '\n';
    put_g(meta, dt, 17);
    meta += '\n';
    const std::string mp = join(dir, "checkpoint.meta"), dp = join(dir, "checkpoint.data");
    FILE* f = std::fopen(mp.c_str(), "wb");
    if (!f) {
        if (err) *err = "cannot create " + mp;
        return LES_BAD_ARG;
    }
    bool ok = put_str(f, meta);
    ok = (std::fclose(f) == 0) && ok;
    // data (binary): u, v, w, p, nu_t as raw doubles, then one byte per cell
    f = ok ? std::fopen(dp.c_str(), "wb") : nullptr;
    if (!f) {
        if (err) *err = "cannot create " + dp;
        return LES_BAD_ARG;
    }
    for (int q = 0; q < 5 && ok; ++q) ok = std::fwrite(f5[q], sizeof(double), n, f) == n;
    if (ok) {
        std::vector<char> b(n);
        for (size_t i = 0; i < n; ++i) b[i] = solid[i] ? 1 : 0;
        ok = std::fwrite(b.data(), 1, n, f) == n;
    }
    ok = (std::fclose(f) == 0) && ok;
    // optional side file: u_new, v_new, w_new, so that a resume is exact (the
    // divergence of the first step after a resume reads u_new)
    if (ok && unew3) {
        const std::string up = join(dir, "checkpoint.unew");
        f = std::fopen(up.c_str(), "wb");
        ok = f != nullptr;
        for (int q = 0; q < 3 && ok; ++q) ok = std::fwrite(unew3[q], sizeof(double), n, f) == n;
        if (f) ok = (std::fclose(f) == 0) && ok;
    }
    if (!ok && err) *err = "checkpoint write failed in " + std::string(dir);
    return ok ? LES_OK : LES_BAD_ARG;
}

// load_state (src/io.cpp:73-120): 0 with LES_OK when there is no metadata file
les_status read_checkpoint(const les_mesh& m, const char* dir, double* const* f5, uint8_t* solid, double* time_sim,
                           double* dt, int* step, double* const* unew3, std::string* err)
{
    const size_t n = (size_t)m.nx * m.ny * m.nz;
    *step = 0;
    const std::string mp = join(dir, "checkpoint.meta"), dp = join(dir, "checkpoint.data");
    FILE* f = std::fopen(mp.c_str(), "rb");
    if (!f) return LES_OK;   // no checkpoint: start from scratch
    int st = 0;
    double t = 0, d = 0;
    const bool parsed = std::fscanf(f, "%d %lf %lf", &st, &t, &d) == 3;
    std::fclose(f);
    if (!parsed) {
        if (err) *err = "cannot parse " + mp;
        return LES_BAD_ARG;
    }
    f = std::fopen(dp.c_str(), "rb");
    if (!f) {
        if (err) *err = "found " + mp + " but not " + dp;
        return LES_BAD_ARG;
    }
    bool ok = true;
    for (int q = 0; q < 5 && ok; ++q) ok = std::fread(f5[q], sizeof(double), n, f) == n;
    std::vector<char> b(n);
    ok = ok && std::fread(b.data(), 1, n, f) == n;
    std::fclose(f);
    if (!ok) {
        if (err) *err = "checkpoint data too short: " + dp;
        return LES_BAD_ARG;
    }
    for (size_t i = 0; i < n; ++i) solid[i] = b[i] == 1 ? 1 : 0;
    if (unew3) {
        f = std::fopen(join(dir, "checkpoint.unew").c_str(), "rb");
        if (!f) {
            if (err) *err = "no checkpoint.unew side file in " + std::string(dir);
            return LES_BAD_ARG;
        }
        for (int q = 0; q < 3 && ok; ++q) ok = std::fread(unew3[q], sizeof(double), n, f) == n;
        std::fclose(f);
        if (!ok) {
            if (err) *err = "checkpoint.unew too short";
            return LES_BAD_ARG;
        }
    }
    *time_sim = t;
    *dt = d;
    *step = st;
    return LES_OK;
}

// ---- statistics kernels (src/statistics.cpp) -----------------------------------
__global__ void k_stats_update(int n, const double* __restrict__ u, const double* __restrict__ v,
                               const double* __restrict__ w, const double* __restrict__ p, double* __restrict__ s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = u[i], b = v[i], c = w[i], d = p[i];
    const size_t N = (size_t)n;
    s[0 * N + i] += a;
    s[1 * N + i] += b;
    s[2 * N + i] += c;
    s[3 * N + i] += d;
    s[4 * N + i] += a * a;
    s[5 * N + i] += b * b;
    s[6 * N + i] += c * c;
    s[7 * N + i] += a * b;
    s[8 * N + i] += a * c;
    s[9 * N + i] += b * c;
}

// means u, v, w, p and <u'u'> = <u^2> - <u>^2, ... into o (10 x n)
__global__ void k_stats_finalize(int n, double n_inv, const double* __restrict__ s, double* __restrict__ o)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    const double um = s[0 * N + i] * n_inv, vm = s[1 * N + i] * n_inv, wm = s[2 * N + i] * n_inv;
    o[0 * N + i] = um;
    o[1 * N + i] = vm;
    o[2 * N + i] = wm;
    o[3 * N + i] = s[3 * N + i] * n_inv;
    o[4 * N + i] = (s[4 * N + i] * n_inv) - (um * um);
    o[5 * N + i] = (s[5 * N + i] * n_inv) - (vm * vm);
    o[6 * N + i] = (s[6 * N + i] * n_inv) - (wm * wm);
    o[7 * N + i] = (s[7 * N + i] * n_inv) - (um * vm);
    o[8 * N + i] = (s[8 * N + i] * n_inv) - (um * wm);
    o[9 * N + i] = (s[9 * N + i] * n_inv) - (vm * wm);
}

IoWork& io(les_ctx* c)
{
    if (!c->io) c->io = new IoWork();
    return *c->io;
}

// device snapshot + pinned staging for 8 fields and the mask
les_status ensure_staging(les_ctx* c)
{
    IoWork& w = io(c);
    const size_t n = c->g.n;
    if (w.n == n && w.dev) return LES_OK;
    les_status st = check_cuda(c, cudaMalloc(&w.dev, sizeof(double) * 8 * n), "cudaMalloc(io snapshot)");
    if (!st) st = check_cuda(c, cudaMalloc(&w.dev_mask, n), "cudaMalloc(io snapshot)");
    if (!st) st = check_cuda(c, cudaMallocHost(&w.host, sizeof(double) * 8 * n), "cudaMallocHost(io staging)");
    if (!st) st = check_cuda(c, cudaMallocHost(&w.host_mask, n), "cudaMallocHost(io staging)");
    if (!st) st = check_cuda(c, cudaStreamCreateWithFlags(&w.copy, cudaStreamNonBlocking), "io stream");
    if (!st) st = check_cuda(c, cudaEventCreateWithFlags(&w.ready, cudaEventDisableTiming), "io event");
    if (!st) st = check_cuda(c, cudaEventCreateWithFlags(&w.copied, cudaEventDisableTiming), "io event");
    if (!st) w.n = n;
    return st;
}

// Snapshot (u, v, w, p, nu_t[, u_new, v_new, w_new], mask) on the context's
// stream, then copy it to pinned memory on the copy stream.
les_status snapshot(les_ctx* c, int nf)
{
    IoWork& w = io(c);
    if (w.writer.joinable()) w.writer.join();
    les_status st = ensure_staging(c);
    if (st) return st;
    const size_t n = c->g.n;
    const int sl[8] = {LES_U, LES_V, LES_W, LES_P, LES_NU_T, LES_U_NEW, LES_V_NEW, LES_W_NEW};
    for (int q = 0; q < nf && !st; ++q)
        st = check_cuda(c, cudaMemcpyAsync(w.dev + q * n, c->slot[sl[q]], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                           c->stream), "snapshot");
    if (!st) st = check_cuda(c, cudaMemcpyAsync(w.dev_mask, c->mask, n, cudaMemcpyDeviceToDevice, c->stream), "snapshot");
    if (!st) st = check_cuda(c, cudaEventRecord(w.ready, c->stream), "snapshot");
    if (!st) st = check_cuda(c, cudaStreamWaitEvent(w.copy, w.ready, 0), "snapshot");
    if (!st) st = check_cuda(c, cudaMemcpyAsync(w.host, w.dev, sizeof(double) * nf * n, cudaMemcpyDeviceToHost, w.copy),
                             "stage");
    if (!st) st = check_cuda(c, cudaMemcpyAsync(w.host_mask, w.dev_mask, n, cudaMemcpyDeviceToHost, w.copy), "stage");
    if (!st) st = check_cuda(c, cudaEventRecord(w.copied, w.copy), "stage");
    return st;
}

}  // namespace

extern "C" {

// ---- host-only writers/readers (no device needed) ------------------------------
les_status les_format_field_vtk(const les_mesh* m, int step, const double* u, const double* v, const double* w,
                                const double* p, const double* nu_t, const uint8_t* solid, const char* path)
{
    if (!m || !u || !v || !w || !p || !nu_t || !solid || !path) return LES_BAD_ARG;
    return field_vtk(*m, step, u, v, w, p, nu_t, solid, path, nullptr);
}

les_status les_format_stats_vtk(const les_mesh* m, const double* const* mean4, const double* const* stress6,
                                const char* path)
{
    if (!m || !mean4 || !stress6 || !path) return LES_BAD_ARG;
    return stats_vtk(*m, mean4, stress6, path, nullptr);
}

les_status les_write_checkpoint_files(const les_mesh* m, const double* const* fields5, const uint8_t* solid,
                                      double time_simulated, double dt, int next_step, const char* dir,
                                      const double* const* unew3)
{
    if (!m || !fields5 || !solid || !dir) return LES_BAD_ARG;
    return write_checkpoint(*m, fields5, solid, time_simulated, dt, next_step, dir, unew3, nullptr);
}

les_status les_read_checkpoint_files(const les_mesh* m, const char* dir, double* const* fields5, uint8_t* solid,
                                     double* time_simulated, double* dt, int* step, double* const* unew3)
{
    if (!m || !dir || !fields5 || !solid || !time_simulated || !dt || !step) return LES_BAD_ARG;
    return read_checkpoint(*m, dir, fields5, solid, time_simulated, dt, step, unew3, nullptr);
}

// ---- device-resident statistics -----------------------------------------------
les_status les_stats_begin(les_ctx* c, int start_step)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    IoWork& w = io(c);
    const size_t n = c->g.n;
    if (!w.sums) {
        les_status st = check_cuda(c, cudaMalloc(&w.sums, sizeof(double) * 10 * n), "cudaMalloc(statistics)");
        if (st) return st;
    }
    w.samples = 0;
    w.start_step = start_step;
    return check_cuda(c, cudaMemsetAsync(w.sums, 0, sizeof(double) * 10 * n, c->stream), "statistics init");
}

les_status les_stats_update(les_ctx* c, int current_step)
{
    if (!c || !c->io || !c->io->sums) return c ? fail(c, LES_BAD_ARG, "statistics: call les_stats_begin first")
                                               : LES_BAD_ARG;
    cudaSetDevice(c->device);
    IoWork& w = *c->io;
    if (current_step <= w.start_step) return LES_OK;   // src/statistics.cpp:101-103
    ++w.samples;
    const int n = c->g.n;
    launch(c, k_stats_update, (n + 255) / 256, 256, n, (const double*)c->slot[LES_U], (const double*)c->slot[LES_V],
           (const double*)c->slot[LES_W], (const double*)c->slot[LES_P], w.sums);
    return check_launch(c, "statistics update");
}

les_status les_stats_sums(les_ctx* c, double* const* out10, int* samples)
{
    if (!c || !c->io || !c->io->sums) return c ? fail(c, LES_BAD_ARG, "statistics: call les_stats_begin first")
                                               : LES_BAD_ARG;
    cudaSetDevice(c->device);
    IoWork& w = *c->io;
    const size_t n = c->g.n;
    les_status st = LES_OK;
    for (int q = 0; q < 10 && !st; ++q)
        if (out10 && out10[q])
            st = check_cuda(c, cudaMemcpyAsync(out10[q], w.sums + q * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                               c->stream), "statistics read");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "statistics read");
    if (samples) *samples = w.samples;
    return st;
}

les_status les_stats_finalize(les_ctx* c, double* const* out10, int* samples)
{
    if (!c || !c->io || !c->io->sums) return c ? fail(c, LES_BAD_ARG, "statistics: call les_stats_begin first")
                                               : LES_BAD_ARG;
    cudaSetDevice(c->device);
    IoWork& w = *c->io;
    if (samples) *samples = w.samples;
    if (w.samples == 0) return LES_OK;   // src/statistics.cpp:135-138: nothing to average
    les_status st = ensure_staging(c);
    if (st) return st;
    if (w.writer.joinable()) w.writer.join();   // the snapshot buffer is reused below
    const int n = c->g.n;
    double* o = nullptr;
    st = check_cuda(c, cudaMalloc(&o, sizeof(double) * 10 * (size_t)n), "cudaMalloc(statistics)");
    if (st) return st;
    launch(c, k_stats_finalize, (n + 255) / 256, 256, n, 1.0 / (double)w.samples, (const double*)w.sums, o);
    st = check_launch(c, "statistics finalize");
    for (int q = 0; q < 10 && !st; ++q)
        if (out10 && out10[q])
            st = check_cuda(c, cudaMemcpyAsync(out10[q], o + (size_t)q * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                               c->stream), "statistics read");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "statistics read");
    cudaFree(o);
    return st;
}

les_status les_stats_save_vtk(les_ctx* c, const char* path)
{
    if (!c || !path) return LES_BAD_ARG;
    if (!c->io || !c->io->sums) return fail(c, LES_BAD_ARG, "statistics: call les_stats_begin first");
    if (c->io->samples == 0) return LES_OK;   // the reference skips the file
    const size_t n = c->g.n;
    std::vector<double> h(10 * n);
    double* out[10];
    for (int q = 0; q < 10; ++q) out[q] = h.data() + q * n;
    les_status st = les_stats_finalize(c, out, nullptr);
    if (st) return st;
    const double* mean4[4] = {out[0], out[1], out[2], out[3]};
    const double* st6[6] = {out[4], out[5], out[6], out[7], out[8], out[9]};
    std::string err;
    st = stats_vtk(c->mesh, mean4, st6, path, &err);
    return st ? fail(c, st, err) : LES_OK;
}

// ---- files from device fields ----------------------------------------------------
les_status les_write_vtk(les_ctx* c, int step, const char* path)
{
    if (!c || !path) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    les_status st = snapshot(c, 5);
    if (st) return st;
    IoWork& w = *c->io;
    const std::string p = path;
    const les_mesh m = c->mesh;
    const int dev = c->device;
    w.result = LES_OK;
    w.writer = std::thread([&w, p, m, step, dev] {
        cudaSetDevice(dev);
        if (cudaEventSynchronize(w.copied) != cudaSuccess) {
            w.result = LES_CUDA_ERROR;
            w.err = "field file: staging copy failed";
            return;
        }
        const size_t n = w.n;
        w.result = field_vtk(m, step, w.host, w.host + n, w.host + 2 * n, w.host + 3 * n, w.host + 4 * n, w.host_mask,
                             p.c_str(), &w.err);
    });
    return LES_OK;
}

les_status les_save_state(les_ctx* c, const char* dir, double time_simulated, double dt, int next_step, int with_unew)
{
    if (!c || !dir) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    les_status st = snapshot(c, with_unew ? 8 : 5);
    if (st) return st;
    IoWork& w = *c->io;
    const std::string d = dir;
    const les_mesh m = c->mesh;
    const int dev = c->device;
    w.result = LES_OK;
    w.writer = std::thread([&w, d, m, time_simulated, dt, next_step, with_unew, dev] {
        cudaSetDevice(dev);
        if (cudaEventSynchronize(w.copied) != cudaSuccess) {
            w.result = LES_CUDA_ERROR;
            w.err = "checkpoint: staging copy failed";
            return;
        }
        const size_t n = w.n;
        const double* f5[5] = {w.host, w.host + n, w.host + 2 * n, w.host + 3 * n, w.host + 4 * n};
        const double* u3[3] = {w.host + 5 * n, w.host + 6 * n, w.host + 7 * n};
        w.result = write_checkpoint(m, f5, w.host_mask, time_simulated, dt, next_step, d.c_str(),
                                    with_unew ? u3 : nullptr, &w.err);
    });
    return LES_OK;
}

les_status les_io_wait(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    if (!c->io) return LES_OK;
    IoWork& w = *c->io;
    if (w.writer.joinable()) w.writer.join();
    const les_status st = w.result;
    w.result = LES_OK;
    return st ? fail(c, st, w.err) : LES_OK;
}

les_status les_load_state(les_ctx* c, const char* dir, double* time_simulated, double* dt, int* step, int with_unew)
{
    if (!c || !dir || !time_simulated || !dt || !step) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    const size_t n = c->g.n;
    std::vector<double> h((with_unew ? 8 : 5) * n);
    std::vector<uint8_t> solid(n);
    double* f5[5] = {h.data(), h.data() + n, h.data() + 2 * n, h.data() + 3 * n, h.data() + 4 * n};
    double* u3[3] = {with_unew ? h.data() + 5 * n : nullptr, with_unew ? h.data() + 6 * n : nullptr,
                     with_unew ? h.data() + 7 * n : nullptr};
    std::string err;
    les_status st = read_checkpoint(c->mesh, dir, f5, solid.data(), time_simulated, dt, step, with_unew ? u3 : nullptr,
                                    &err);
    if (st) return fail(c, st, err);
    if (*step == 0) return LES_OK;   // no checkpoint
    const int sl[8] = {LES_U, LES_V, LES_W, LES_P, LES_NU_T, LES_U_NEW, LES_V_NEW, LES_W_NEW};
    for (int q = 0; q < (with_unew ? 8 : 5) && !st; ++q) st = les_upload(c, sl[q], h.data() + q * n);
    if (!st) st = les_upload_mask(c, solid.data());
    return st;
}

}  // extern "C"
