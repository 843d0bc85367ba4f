// les_wavefront.cu -- the three lexicographically ordered loops of les-model
// src/pressure.cpp on the device: the IC(0) factorisation (:495-556), the
// IC forward/backward substitution (:442-482) and the GS-SOR sweep
// (:212-246).
//
// Each cell of these loops depends only on its (i-1), (j-1), (k-1)
// neighbours (the backward solve: on i+1, j+1, k+1), so all cells on one
// hyperplane i+j+k = s can be processed at once, and processing hyperplanes in
// order s = 0, 1, 2, ... performs exactly the same floating-point operations
// on exactly the same operand values as the serial lexicographic loop.  The
// result is therefore bit-identical to the reference.
//
// Hyperplanes run inside one cooperative (co-resident) persistent kernel,
// separated by a grid barrier whose waits are bounded (les_internal.cuh); a
// timed-out wait sets an error flag, every block leaves, and the host reports
// LES_TIMEOUT.  Neighbour values written by other blocks are read through L2
// (__ldcg).  Compiled with -fmad=false.
#include <cmath>

#include "les_internal.cuh"

using namespace les;

namespace {

struct Plane {
    int nx, ny, nz, si, sj;
};

__device__ __forceinline__ int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int gthreads() { return gridDim.x * blockDim.x; }

// IC(0) factorisation, src/pressure.cpp:506-555, hyperplane by hyperplane.
// L arrays must be zero on entry (fresh matrix semantics).
__global__ void k_ic_build(Plane P, StencilView A, double* Lc, double* Lw, double* Ls, double* Lb,
                           GridSync gs)
{
    const double small_val = 1e-30;
    const int smax = P.nx + P.ny + P.nz - 3;
    const int njk = P.ny * P.nz;
    for (int s = 0; s <= smax; ++s) {
        for (int t = gtid(); t < njk; t += gthreads()) {
            int j = t / P.nz, k = t - j * P.nz;
            int i = s - j - k;
            if (i < 0 || i >= P.nx) continue;
            int id = i * P.si + j * P.sj + k;
            Coef7 a = A.at(id);
            double sum_sq = 0.0;
            if (i > 0) {
                double lc = __ldcg(Lc + id - P.si);
                if (fabs(lc) > small_val) { double l = a.w / lc; Lw[id] = l; sum_sq += l * l; }
            }
            if (j > 0) {
                double lc = __ldcg(Lc + id - P.sj);
                if (fabs(lc) > small_val) { double l = a.s / lc; Ls[id] = l; sum_sq += l * l; }
            }
            if (k > 0) {
                double lc = __ldcg(Lc + id - 1);
                if (fabs(lc) > small_val) { double l = a.b / lc; Lb[id] = l; sum_sq += l * l; }
            }
            double diag = a.c - sum_sq;
            Lc[id] = (diag <= small_val) ? 1.0 : sqrt(diag);
        }
        if (!grid_barrier(gs)) return;
    }
}

// apply_ic_preconditioner, src/pressure.cpp:442-482: forward substitution in
// increasing hyperplane order, then backward substitution in decreasing order.
// T = double is the reference's arithmetic; T = float serves the FP32 inner
// solve of the mixed-precision path (st == nullptr: never skipped).
template <typename T>
__global__ void k_ic_apply(Plane P, const T* __restrict__ Lc, const T* __restrict__ Lw,
                           const T* __restrict__ Ls, const T* __restrict__ Lb,
                           const T* __restrict__ r, T* z, GridSync gs, const SolverState* st,
                           int skip_done)
{
    if (skip_done && st && st->done) return;   // uniform across blocks: no barrier is entered
    const int smax = P.nx + P.ny + P.nz - 3;
    const int njk = P.ny * P.nz;
    for (int s = 0; s <= smax; ++s) {
        for (int t = gtid(); t < njk; t += gthreads()) {
            int j = t / P.nz, k = t - j * P.nz;
            int i = s - j - k;
            if (i < 0 || i >= P.nx) continue;
            int id = i * P.si + j * P.sj + k;
            T sum = r[id];
            if (i > 0) sum -= Lw[id] * __ldcg(z + id - P.si);
            if (j > 0) sum -= Ls[id] * __ldcg(z + id - P.sj);
            if (k > 0) sum -= Lb[id] * __ldcg(z + id - 1);
            z[id] = sum / Lc[id];
        }
        if (!grid_barrier(gs)) return;
    }
    for (int s = smax; s >= 0; --s) {
        for (int t = gtid(); t < njk; t += gthreads()) {
            int j = t / P.nz, k = t - j * P.nz;
            int i = s - j - k;
            if (i < 0 || i >= P.nx) continue;
            int id = i * P.si + j * P.sj + k;
            T sum = __ldcg(z + id);
            if (i < P.nx - 1) sum -= Lw[id + P.si] * __ldcg(z + id + P.si);
            if (j < P.ny - 1) sum -= Ls[id + P.sj] * __ldcg(z + id + P.sj);
            if (k < P.nz - 1) sum -= Lb[id + 1] * __ldcg(z + id + 1);
            z[id] = sum / Lc[id];
        }
        if (!grid_barrier(gs)) return;
    }
}

// solve_pressure_GS, src/pressure.cpp:212-246: up to max_iter SOR sweeps over
// the interior in hyperplane order, each followed by apply_pressure_BCs
// (face closed form, then the obstacle copy) and the max|dp| < tol test.
__global__ void k_gs_sor(Plane P, double dx2, double dy2, double dz2, double omega, double coef,
                         double tol, int max_iter, const double* __restrict__ rhs, double* p,
                         const uint8_t* __restrict__ solid, const int* __restrict__ solid_list,
                         int n_solid, double* block_max, SolverState* st, GridSync gs)
{
    __shared__ double smax_w[32];
    const int nyi = P.ny - 2, nzi = P.nz - 2;
    const int njk = nyi * nzi;
    const int s_lo = 3, s_hi = (P.nx - 2) + (P.ny - 2) + (P.nz - 2);
    const int nfaces_i = P.ny * P.nz;
    const double one_m_omega = 1 - omega;
    const double omega_coef = omega * coef;
    int sweeps = 0;
    bool converged = false;
    for (int iter = 0; iter < max_iter; ++iter) {
        double lmax = 0.0;
        for (int s = s_lo; s <= s_hi; ++s) {
            for (int t = gtid(); t < njk; t += gthreads()) {
                int jj = t / nzi, kk = t - jj * nzi;
                int j = jj + 1, k = kk + 1;
                int i = s - j - k;
                if (i < 1 || i > P.nx - 2) continue;
                int id = i * P.si + j * P.sj + k;
                double p_old = __ldcg(p + id);
                double v = one_m_omega * p_old +
                           omega_coef * ((__ldcg(p + id + P.si) + __ldcg(p + id - P.si)) / dx2 +
                                         (__ldcg(p + id + P.sj) + __ldcg(p + id - P.sj)) / dy2 +
                                         (__ldcg(p + id + 1) + __ldcg(p + id - 1)) / dz2 - rhs[id]);
                p[id] = v;
                double res = fabs(v - p_old);
                if (res > lmax) lmax = res;
            }
            if (!grid_barrier(gs)) return;
        }
        // apply_pressure_BCs faces: every face cell from interior values
        {
            const int nface = 2 * nfaces_i + 2 * (P.nx - 2) * P.nz + 2 * (P.nx - 2) * (P.ny - 2);
            for (int t = gtid(); t < nface; t += gthreads()) {
                int i, j, k;
                if (t < 2 * nfaces_i) {
                    int q = t % nfaces_i;
                    i = (t < nfaces_i) ? 0 : P.nx - 1;
                    j = q / P.nz; k = q - j * P.nz;
                } else if (t < 2 * nfaces_i + 2 * (P.nx - 2) * P.nz) {
                    int q = t - 2 * nfaces_i, half = (P.nx - 2) * P.nz;
                    j = (q < half) ? 0 : P.ny - 1;
                    q = q % half;
                    i = 1 + q / P.nz; k = q % P.nz;
                } else {
                    int q = t - 2 * nfaces_i - 2 * (P.nx - 2) * P.nz, half = (P.nx - 2) * (P.ny - 2);
                    k = (q < half) ? 0 : P.nz - 1;
                    q = q % half;
                    i = 1 + q / (P.ny - 2); j = 1 + q % (P.ny - 2);
                }
                int id = i * P.si + j * P.sj + k;
                if (i == P.nx - 1) { p[id] = 0.0; continue; }
                int jc = j < 1 ? 1 : (j > P.ny - 2 ? P.ny - 2 : j);
                int kc = k < 1 ? 1 : (k > P.nz - 2 ? P.nz - 2 : k);
                int ic = i == 0 ? 1 : i;
                p[id] = __ldcg(p + ic * P.si + jc * P.sj + kc);
            }
        }
        if (!grid_barrier(gs)) return;
        for (int t = gtid(); t < n_solid; t += gthreads()) {
            const int id = solid_list[t];
            if (!solid[id + P.si]) p[id] = __ldcg(p + id + P.si);
            else if (!solid[id - P.si]) p[id] = __ldcg(p + id - P.si);
            else if (!solid[id + P.sj]) p[id] = __ldcg(p + id + P.sj);
            else if (!solid[id - P.sj]) p[id] = __ldcg(p + id - P.sj);
            else if (!solid[id + 1]) p[id] = __ldcg(p + id + 1);
            else if (!solid[id - 1]) p[id] = __ldcg(p + id - 1);
        }
        // block max -> global max (exact), identical in every block
        lmax = warp_max(lmax);
        if ((threadIdx.x & 31) == 0) smax_w[threadIdx.x >> 5] = lmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) m = fmax(m, smax_w[q]);
            block_max[blockIdx.x] = m;
        }
        if (!grid_barrier(gs)) return;
        double gmax = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) gmax = fmax(gmax, __ldcg(block_max + b));
        sweeps = iter + 1;
        if (gmax < tol) { converged = true; break; }
        // block_max is rewritten next sweep only after the hyperplane barriers
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->iters = sweeps;
        st->k = sweeps;
        st->done = 1;
        st->status = converged ? LES_OK : LES_NOT_CONVERGED;
    }
}

__global__ void k_stat_rhs_gs(Plane P, double coef, double two_dx, double two_dy, double two_dz,
                              const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, double* __restrict__ rhs, int n)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    int i = id / P.si, rem = id - i * P.si, j = rem / P.sj, k = rem - j * P.sj;
    if (i < 1 || i > P.nx - 2 || j < 1 || j > P.ny - 2 || k < 1 || k > P.nz - 2) { rhs[id] = 0.0; return; }
    double div = (u[id + P.si] - u[id - P.si]) / two_dx + (v[id + P.sj] - v[id - P.sj]) / two_dy +
                 (w[id + 1] - w[id - 1]) / two_dz;
    rhs[id] = coef * div;
}

Plane plane_of(const Geo& g) { return Plane{g.nx, g.ny, g.nz, g.si, g.sj}; }

les_status coop_launch(les_ctx* c, const void* fn, void** args, int* grid_out, int pid = -1)
{
    int per_sm = 0;
    les_status st = check_cuda(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0), "occupancy");
    if (st) return st;
    if (per_sm < 1) return fail(c, LES_CUDA_ERROR, "wavefront kernel cannot be resident");
    int grid = c->sms;   // one block per SM: enough threads for the widest hyperplane
    if (grid_out) *grid_out = grid;
    st = check_cuda(c, cudaMemsetAsync(c->gsync, 0, sizeof(unsigned) * 4, c->stream), "reset barrier");
    if (st) return st;
    cudaEvent_t e1 = nullptr;
    if (pid >= 0 && c->prof_on) prof_begin(c, pid, &e1);
    st = check_cuda(c, cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, c->stream),
                    "cooperative launch");
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return st;
}

GridSync grid_sync(les_ctx* c, int grid)
{
    GridSync gs;
    gs.count = c->gsync + 0;
    gs.gen = c->gsync + 1;
    gs.error = (int*)(c->gsync + 2);
    gs.nblocks = (unsigned)grid;
    return gs;
}

les_status check_barrier(les_ctx* c)
{
    unsigned h[4];
    les_status st = check_cuda(c, cudaMemcpyAsync(h, c->gsync, sizeof(h), cudaMemcpyDeviceToHost, c->stream),
                               "read barrier");
    if (st) return st;
    st = check_cuda(c, cudaStreamSynchronize(c->stream), "sync");
    if (st) return st;
    if (h[2]) return fail(c, LES_TIMEOUT, "a wavefront grid barrier timed out");
    return LES_OK;
}

}  // namespace

namespace les {

les_status ic_apply_dev(les_ctx* c, const double* r, double* z, const double* const* Lsrc, int skip_done)
{
    const double* const* L = Lsrc ? Lsrc : (const double* const*)c->L;
    Plane P = plane_of(c->g);
    const double *Lc = L[0], *Lw = L[4], *Ls = L[2], *Lb = L[6];
    GridSync gs = grid_sync(c, c->sms);
    const SolverState* stp = c->state;
    int skip = skip_done;
    void* args[] = {&P, (void*)&Lc, (void*)&Lw, (void*)&Ls, (void*)&Lb, (void*)&r, (void*)&z, &gs, (void*)&stp, &skip};
    return coop_launch(c, (const void*)k_ic_apply<double>, args, nullptr, PROF_IC);
}

les_status ic_apply_dev32(les_ctx* c, const float* r, float* z, const float* const* L, SolverState* st)
{
    Plane P = plane_of(c->g);
    const float *Lc = L[0], *Lw = L[4], *Ls = L[2], *Lb = L[6];
    GridSync gs = grid_sync(c, c->sms);
    const SolverState* stp = st;
    int skip = st ? 1 : 0;
    void* args[] = {&P, (void*)&Lc, (void*)&Lw, (void*)&Ls, (void*)&Lb, (void*)&r, (void*)&z, &gs, (void*)&stp, &skip};
    return coop_launch(c, (const void*)k_ic_apply<float>, args, nullptr, PROF_IC);
}

les_status build_ic_dev(les_ctx* c)
{
    const size_t nb = sizeof(double) * (size_t)c->g.n;
    for (int q = 0; q < 7; ++q) {
        if (!c->L[q]) {
            les_status st = check_cuda(c, cudaMalloc(&c->L[q], nb), "cudaMalloc(L)");
            if (st) return st;
        }
        cudaMemsetAsync(c->L[q], 0, nb, c->stream);
    }
    Plane P = plane_of(c->g);
    StencilView A = stencil_view(c);
    GridSync gs = grid_sync(c, c->sms);
    double *Lc = c->L[0], *Lw = c->L[4], *Ls = c->L[2], *Lb = c->L[6];
    void* args[] = {&P, &A, &Lc, &Lw, &Ls, &Lb, &gs};
    les_status st = coop_launch(c, (const void*)k_ic_build, args, nullptr);
    if (st) return st;
    st = check_barrier(c);
    if (st) return st;
    c->have_L = true;
    return LES_OK;
}

les_status solve_gs_dev(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps)
{
    les_status st = ensure_work(c);
    if (st) return st;
    const les_mesh& m = c->mesh;
    Plane P = plane_of(c->g);
    double* rhs = c->w[0];
    // one slot per block of the cooperative grid (partials holds >= 4096)
    double* block_max = c->partials;
    if ((size_t)c->sms > c->partials_len) return fail(c, LES_BAD_ARG, "internal: partials too small");
    launch(c, k_stat_rhs_gs, (c->g.n + 255) / 256, 256, P, rho / dt, 2 * m.dx, 2 * m.dy, 2 * m.dz,
                                                               c->slot[LES_U], c->slot[LES_V], c->slot[LES_W],
                                                               rhs, c->g.n);
    st = check_launch(c, "gs rhs");
    if (st) return st;
    const double dx2 = m.dx * m.dx, dy2 = m.dy * m.dy, dz2 = m.dz * m.dz;
    const double coef = 1.0 / (2.0 * (1.0 / dx2 + 1.0 / dy2 + 1.0 / dz2));
    double* p = c->slot[LES_P];
    const uint8_t* solid = c->mask;
    const int* list = c->solid_list;
    int ns = c->n_solid;
    SolverState* stp = c->state;
    GridSync gs = grid_sync(c, c->sms);
    void* args[] = {&P, (void*)&dx2, (void*)&dy2, (void*)&dz2, &omega, (void*)&coef, &tol, &max_iter,
                    (void*)&rhs, &p, (void*)&solid, (void*)&list, &ns, &block_max, &stp, &gs};
    st = coop_launch(c, (const void*)k_gs_sor, args, nullptr);
    if (st) return st;
    st = check_barrier(c);
    if (st) return st;
    st = read_state(c);
    if (st) return st;
    if (sweeps) *sweeps = max_iter > 0 ? c->h_state->iters : 0;
    return LES_OK;
}

}  // namespace les

extern "C" {

les_status les_build_ic(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix: call les_build_stencil or les_set_stencil");
    cudaSetDevice(c->device);
    return build_ic_dev(c);
}

les_status les_solve_gs(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps)
{
    if (!c || max_iter < 0) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return solve_gs_dev(c, dt, rho, max_iter, omega, tol, sweeps);
}

}  // extern "C"
