// les_mixed.cu -- mixed-precision pressure solve: FP32 inner PCG inside FP64
// defect correction (iterative refinement) for the system A p = b of les-model
// src/pressure.cpp:342-414.
//
//   r = b - A x            FP64 (exact coefficients, FP64 accumulation)
//   while ||r||_2 >= tol:  FP64 norm
//       solve A e = r      FP32 PCG from e = 0 to ||r_in|| < inner_rtol*||r||,
//                          with the same preconditioner family (Jacobi,
//                          Chebyshev, IC) in FP32; every inner product and
//                          norm is accumulated in FP64
//       x += e             FP64
//       r = b - A x        FP64
//
// The outer residual, its norm and the solution stay FP64, so the stopping
// test is the reference's absolute test on the true FP64 residual.  The
// system has no null space (the outlet rows are Dirichlet), so there is no
// mean-pressure removal step.
//
// Kernels here may contract a*b+c into FMA (this file is compiled without
// -fmad=false): the FP64 defect is a sum of fused multiply-adds, at least as
// accurate as the reference's separately rounded products.
#include <cmath>
#include <utility>

#include "les_bits.cuh"
#include "les_internal.cuh"
#include "les_mixed.cuh"

using namespace les;

namespace les {
les_status ensure_stored_A(les_ctx* c);
les_status ic_apply_dev32(les_ctx* c, const float* r, float* z, const float* const* L32, SolverState* st);
les_status wave_check(les_ctx* c);
}

namespace {

__device__ __forceinline__ bool cell_coords(const Geo& g, int& i, int& j, int& k)
{
    k = blockIdx.x * TBK + threadIdx.x;
    j = blockIdx.y * TBJ + threadIdx.y;
    i = blockIdx.z;
    return k < g.nz && j < g.ny;
}


// (A x)_id in FP64 fused multiply-adds (GB300 runs about 2 FP64 instructions
// per SM and clock, so the defect is bound by their count)
__device__ __forceinline__ double row64(const StencilView& A, const double* __restrict__ x, const Geo& g,
                                        int i, int j, int k, int id)
{
    Coef7 a = A.at(id);
    double val = a.c * x[id];
    if (i > 0) val = fma(a.w, x[id - g.si], val);
    if (i < g.nx - 1) val = fma(a.e, x[id + g.si], val);
    if (j > 0) val = fma(a.s, x[id - g.sj], val);
    if (j < g.ny - 1) val = fma(a.n, x[id + g.sj], val);
    if (k > 0) val = fma(a.b, x[id - 1], val);
    if (k < g.nz - 1) val = fma(a.t, x[id + 1], val);
    return val;
}

constexpr int RES_PLANES = 4;   // planes per thread of the defect kernel

inline dim3 resid_grid(const Geo& g)
{
    const dim3 c = cell_grid(g);
    return dim3(c.x, c.y, (g.nx + RES_PLANES - 1) / RES_PLANES);
}

// Outer residual: r = b - A x in FP64, its FP32 copy for the inner solve, and
// ||r||^2 in FP64.  Sets the outer state done once ||r|| < tol.
// (bx, by, bz): block coordinates in the grid of resid_grid(g); (lb, nb):
// this block among the blocks of the reduction
__device__ __forceinline__ void outer_resid(const Geo& g, const StencilView& A, const double* __restrict__ x,
                                            const double* __restrict__ b, float* __restrict__ r32, double* partials,
                                            unsigned* counter, SolverState* st, int outer, int bx, int by, int bz,
                                            int lb, int nb)
{
    __shared__ double sm[32];
    const int k = bx * TBK + threadIdx.x, j = by * TBJ + threadIdx.y;
    double rr[1] = {0.0};
    if (k < g.nz && j < g.ny) {   // bz: a group of RES_PLANES planes
        const int i0 = bz * RES_PLANES, i1 = min(g.nx, i0 + RES_PLANES);
        for (int i = i0; i < i1; ++i) {
            const int id = i * g.si + j * g.sj + k;
            const double r = b[id] - row64(A, x, g, i, j, k, id);
            r32[id] = d2f_bits(r);
            rr[0] = fma(r, r, rr[0]);
        }
    }
    if (last_block_sum<1>(rr, partials, counter, sm, lb, nb)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double e = sqrt(rr[0]);
            st->err = e;
            st->rr = rr[0];
            st->k = outer >= 0 ? outer : st->k + 1;   // outer < 0: count on the device (graph replay)
            if (e < st->tol) { st->done = 1; st->status = LES_OK; }
            else if (!isfinite(e)) { st->done = 1; st->status = LES_NONFINITE; }
        }
    }
}

__global__ void k_outer_resid(Geo g, StencilView A, const double* __restrict__ x, const double* __restrict__ b,
                              float* __restrict__ r32, double* partials, unsigned* counter, SolverState* st,
                              int outer)
{
    outer_resid(g, A, x, b, r32, partials, counter, st, outer, blockIdx.x, blockIdx.y, blockIdx.z, block_linear_id(),
                block_count());
}

// The defects of the cases in their correction round of a batched ensemble
// solve (each counts the round on the device).
__global__ void k_outer_resid_batch(const BatchCase* __restrict__ cs, const int* __restrict__ pre, int n)
{
    const int c = batch_case(pre, n, blockIdx.x);
    const BatchCase& C = cs[c];
    if (!C.act) return;
    const int b0 = __ldg(pre + c), nb = __ldg(pre + c + 1) - b0, lb = blockIdx.x - b0;
    const int gx = (C.g.nz + TBK - 1) / TBK, gy = (C.g.ny + TBJ - 1) / TBJ;
    outer_resid(C.g, C.A, C.x, C.b, C.r0, C.partials, C.counters + 8, C.out, -1, lb % gx, (lb / gx) % gy,
                lb / (gx * gy), lb, nb);
}

__global__ void k_x_add(Geo g, double* __restrict__ x, const float* __restrict__ e)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    x[id] = __dadd_rn(x[id], (double)e[id]);
}

// Inner state init: tolerance relative to the current outer residual, but no
// tighter than the outer tolerance needs (less the LAST_MARGIN for the FP32
// rounding of the correction): the last correction is not over-solved.
__global__ void k_inner_init(SolverState* in, const SolverState* out, double inner_rtol, int max_iter)
{
    in->tol = fmax(inner_rtol * out->err, out->tol / LAST_MARGIN);
    in->max_iter = max_iter;
    in->k = 0;
    in->done = 0;
    in->frozen = 0;
    in->iters = 0;
    in->status = LES_OK;
    in->beta = 0.0;
}

// z = M^-1 r for the first inner iteration (Jacobi or Chebyshev step 0),
// plus rho = r.z.  e = 0.
__global__ void k_in_pc0(Geo g, ViewF A, int mode, float alpha0, const float* __restrict__ r,
                         float* __restrict__ z, float* __restrict__ e, double* partials, unsigned* counter,
                         SolverState* st)
{
    __shared__ double sm[32];
    int i, j, k;
    double rz[1] = {0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        float rv = r[id];
        float zv = mode == 0 ? rv * A.inv_diag(id) : alpha0 * rv;
        z[id] = zv;
        e[id] = 0.f;
        rz[0] = (double)(rv * zv);
    }
    if (last_block_sum<1>(rz, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) st->rho = rz[0];
    }
}

// p_new = z + beta p_old (first: p_new = z), q = A p_new, alpha = rho / p.q.
// p_new at the neighbours is formed on the fly, so p is double-buffered.
__global__ void k_in_spmv(Geo g, ViewF A, const float* __restrict__ z, const float* __restrict__ pold,
                          float* __restrict__ pnew, float* __restrict__ q, int first, double* partials,
                          unsigned* counter, SolverState* st)
{
    __shared__ double sm[32];
    if (st->done) return;
    const float beta = first ? 0.f : (float)st->beta;
    int i, j, k;
    double pq[1] = {0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        auto P = [&](int t) -> float { return first ? z[t] : z[t] + beta * pold[t]; };
        CoefF a = A.at(id);
        float pc = P(id);
        float val = a.c * pc;
        if (i > 0) val += a.w * P(id - g.si);
        if (i < g.nx - 1) val += a.e * P(id + g.si);
        if (j > 0) val += a.s * P(id - g.sj);
        if (j < g.ny - 1) val += a.n * P(id + g.sj);
        if (k > 0) val += a.b * P(id - 1);
        if (k < g.nz - 1) val += a.t * P(id + 1);
        pnew[id] = pc;
        q[id] = val;
        pq[0] = (double)(pc * val);
    }
    if (last_block_sum<1>(pq, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) st->alpha = st->rho / pq[0];
    }
}

// e += alpha p; r -= alpha q; ||r||; inner convergence; the preconditioner's
// first stage (Jacobi: z = r/A_c and r.z; Chebyshev: z0 = alpha0 r).
__global__ void k_in_update(Geo g, ViewF A, int mode, float alpha0, float* __restrict__ e,
                            float* __restrict__ r, const float* __restrict__ p, const float* __restrict__ q,
                            float* __restrict__ z, double* partials, unsigned* counter, SolverState* st,
                            SolverState* outer, int total_cap)
{
    __shared__ double sm[64];
    if (st->done) return;
    const float alpha = (float)st->alpha;
    int i, j, k;
    double acc[2] = {0.0, 0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        e[id] += alpha * p[id];
        float rv = r[id] - alpha * q[id];
        r[id] = rv;
        acc[0] = (double)(rv * rv);
        if (mode == 0) {
            float zv = rv * A.inv_diag(id);
            z[id] = zv;
            acc[1] = (double)(rv * zv);
        } else if (mode == 1) {
            z[id] = alpha0 * rv;
        }
    }
    if (last_block_sum<2>(acc, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double err = sqrt(acc[0]);
            int kk = st->k + 1;
            st->k = kk;
            st->err = err;
            int total = outer->iters + 1;
            outer->iters = total;
            if (err < st->tol) { st->done = 1; st->status = LES_OK; }
            else if (!isfinite(err)) { st->done = 1; st->status = LES_NONFINITE; }
            else if (kk >= st->max_iter || total >= total_cap) { st->done = 1; st->status = LES_NOT_CONVERGED; }
            if (mode == 0) {
                st->beta = acc[1] / st->rho;
                st->rho = acc[1];
            }
        }
    }
}

// Chebyshev inner step in FP32 (same recurrence as src/pressure.cpp:888-905).
// The last step also reduces r.z and forms beta.
__global__ void k_in_cheb(Geo g, ViewF A, float alpha, float beta, const float* __restrict__ r,
                          const float* __restrict__ zin, const float* pin, float* pout, float* __restrict__ zout,
                          int last, double* partials, unsigned* counter, SolverState* st, int skip_done)
{
    __shared__ double sm[32];
    if (skip_done && st->done) return;
    int i, j, k;
    double rz[1] = {0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        CoefF a = A.at(id);
        float val = a.c * zin[id];
        if (i > 0) val += a.w * zin[id - g.si];
        if (i < g.nx - 1) val += a.e * zin[id + g.si];
        if (j > 0) val += a.s * zin[id - g.sj];
        if (j < g.ny - 1) val += a.n * zin[id + g.sj];
        if (k > 0) val += a.b * zin[id - 1];
        if (k < g.nz - 1) val += a.t * zin[id + 1];
        float rv = r[id];
        float pv = (rv - val) + beta * (pin ? pin[id] : rv);
        pout[id] = pv;
        float zv = zin[id] + alpha * pv;
        zout[id] = zv;
        rz[0] = (double)(rv * zv);
    }
    if (!last) return;
    if (last_block_sum<1>(rz, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (skip_done) {   // inside the iteration: beta and rho
                st->beta = rz[0] / st->rho;
                st->rho = rz[0];
            } else {
                st->rho = rz[0];
            }
        }
    }
}

__global__ void k_in_dot_beta(Geo g, const float* __restrict__ r, const float* __restrict__ z, double* partials,
                              unsigned* counter, SolverState* st, int init)
{
    __shared__ double sm[32];
    if (!init && st->done) return;
    int i, j, k;
    double rz[1] = {0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        rz[0] = (double)(r[id] * z[id]);
    }
    if (last_block_sum<1>(rz, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (init) st->rho = rz[0];
            else { st->beta = rz[0] / st->rho; st->rho = rz[0]; }
        }
    }
}

__global__ void k_zero_f(Geo g, float* __restrict__ a)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    a[i * g.si + j * g.sj + k] = 0.f;
}

__global__ void k_to_f(int n, const double* __restrict__ a, float* __restrict__ b)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}

__global__ void k_set_outer(SolverState* st, double tol, int keep_tol)
{
    if (!keep_tol) st->tol = tol;
    st->done = 0;
    st->iters = 0;
    st->k = 0;
    st->status = LES_OK;
}

ViewF view32(les_ctx* c)
{
    ViewF v{};
    if (c->stencil_mode == 1) {
        v.code = c->code;
        v.k.c0 = (float)c->coef.c0;
        v.k.x1 = (float)c->coef.x1; v.k.x2 = (float)c->coef.x2;
        v.k.y1 = (float)c->coef.y1; v.k.y2 = (float)c->coef.y2;
        v.k.z1 = (float)c->coef.z1; v.k.z2 = (float)c->coef.z2;
    } else {
        v.code = nullptr;
        for (int q = 0; q < 7; ++q) v.d[q] = c->A32[q];
    }
    return v;
}

les_status ensure_f32_copy(les_ctx* c, float** dst, double* const* src)
{
    const int n = c->g.n;
    for (int q = 0; q < 7; ++q) {
        if (!src[q]) continue;
        if (!dst[q]) {
            les_status st = check_cuda(c, cudaMalloc(&dst[q], sizeof(float) * (size_t)n), "cudaMalloc(f32 copy)");
            if (st) return st;
        }
        launch(c, k_to_f, (n + 255) / 256, 256, n, src[q], dst[q]);
    }
    return check_launch(c, "f32 copy");
}

}  // namespace

namespace les {

// Preconditioner in FP32 inside the inner loop: r -> z.  mode 0 Jacobi (fused
// in k_in_update), 1 Chebyshev, 2 IC (L or A).
static les_status inner_precond(les_ctx* c, const les_pcg_opts* o, ViewF A, float* r, float* z, SolverState* in,
                                const float* const* L32, int skip_done, int init)
{
    const Geo& g = c->g;
    const dim3 gr = cell_grid(g), bl = cell_block();
    if (o->precond == LES_PC_CHEBYSHEV) {
        const double d = (o->lambda_max + o->lambda_min) / 2.0;
        const double cc = (o->lambda_max - o->lambda_min) / 2.0;
        double alpha = 2.0 / d;
        const int steps = o->degree - 1;
        float* zb[2] = {z, c->f[6]};
        // step 0 (z0 = alpha0 r) was written into zb[start] by the caller
        int cur = (steps % 2 == 0) ? 0 : 1;
        float* pbuf = c->f[7];
        for (int kq = 1; kq <= steps; ++kq) {
            double beta = (cc * alpha / 2.0) * (cc * alpha / 2.0);
            alpha = 1.0 / (d - beta);
            launch_p(c, PROF_IN_CHEB, k_in_cheb, gr, bl, g, A, (float)alpha, (float)beta, r, zb[cur], kq == 1 ? nullptr : pbuf,
                                                pbuf, zb[cur ^ 1], kq == steps, c->partials, c->counters + 12, in,
                                                skip_done);
            cur ^= 1;
        }
        if (steps == 0)
            launch(c, k_in_dot_beta, gr, bl, g, r, z, c->partials, c->counters + 13, in, init);
        return check_launch(c, "inner chebyshev");
    }
    // IC: wavefront solve in FP32, then r.z
    les_status st = ic_apply_dev32(c, r, z, L32, skip_done ? in : nullptr);
    if (st) return st;
    launch(c, k_in_dot_beta, gr, bl, g, r, z, c->partials, c->counters + 13, in, init);
    return check_launch(c, "inner ic");
}

les_status pcg_mixed_impl(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol)
{
    const Geo& g = c->g;
    les_status st = ensure_work(c);
    if (st) return st;
    st = ensure_work32(c);
    if (st) return st;
    if (o->precond == LES_PC_CHEBYSHEV && o->degree < 1) return fail(c, LES_BAD_ARG, "Chebyshev degree must be >= 1");
    if (c->stencil_mode == 2) {
        st = ensure_f32_copy(c, c->A32, c->A);
        if (st) return st;
    }
    const float* L32[7] = {};
    if (o->precond == LES_PC_IC || o->precond == LES_PC_IC_A) {
        if (o->precond == LES_PC_IC && !c->have_L) return fail(c, LES_BAD_ARG, "IC preconditioner needs a factor");
        if (o->precond == LES_PC_IC_A) {
            st = ensure_stored_A(c);
            if (st) return st;
        }
        double* src[7] = {};
        double* const* from = (o->precond == LES_PC_IC) ? c->L : c->A;
        src[0] = from[0]; src[2] = from[2]; src[4] = from[4]; src[6] = from[6];
        st = ensure_f32_copy(c, c->L32, src);
        if (st) return st;
        for (int q = 0; q < 7; ++q) L32[q] = c->L32[q];
    }
    const int mode = o->precond == LES_PC_JACOBI ? 0 : (o->precond == LES_PC_CHEBYSHEV ? 1 : 2);
    ViewF A32 = view32(c);
    StencilView A = stencil_view(c);
    SolverState* out = c->state;
    SolverState* in = c->state + 1;
    double* x = c->slot[LES_P];
    const double* b = c->slot[LES_B];
    float *r = c->f[0], *z = c->f[1], *pb[2] = {c->f[2], c->f[3]}, *q = c->f[4], *e = c->f[5];
    const dim3 gr = cell_grid(g), bl = cell_block();
    const double dcheb = (o->lambda_max + o->lambda_min) / 2.0;
    const float alpha0 = (float)(2.0 / dcheb);
    const int inner_cap = o->inner_max_iter > 0 ? o->inner_max_iter : o->max_iter;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 50;

    launch(c, k_set_outer, 1, 1, out, o->tol, keep_tol);
    launch_p(c, PROF_OUTER, k_outer_resid, resid_grid(g), bl, g, A, x, b, r, c->partials, c->counters + 8, out, 0);
    st = check_launch(c, "outer residual");
    if (st) return st;
    st = read_state(c);
    if (st) return st;
    int outer = 0;
    while (!c->h_state[0].done && outer < max_outer && c->h_state[0].iters < o->max_iter) {
        // ---- inner FP32 PCG on A e = r, e0 = 0
        launch(c, k_inner_init, 1, 1, in, out, o->inner_rtol, inner_cap);
        if (c->fused && fused_supported(o)) {
            st = inner_solve_fused(c, o, A32, in, out, inner_cap);
            if (st) return st;
        } else if (mode == 2) {
            launch(c, k_zero_f, gr, bl, g, e);
            st = inner_precond(c, o, A32, r, z, in, L32, 0, 1);
        } else {
            // Chebyshev: the first z must land where the recurrence expects it
            int steps = o->degree - 1;
            float* z0 = (mode == 1 && steps % 2 == 1) ? c->f[6] : z;
            launch(c, k_in_pc0, gr, bl, g, A32, mode, alpha0, r, z0, e, c->partials, c->counters + 9, in);
            if (mode == 1 && steps > 0) st = inner_precond(c, o, A32, r, z, in, L32, 0, 1);
        }
        if (st) return st;
        int cur = 0, launched = 0, batch = 4;
        for (; !(c->fused && fused_supported(o));) {   // unfused kernels (IC; fused path off)
            for (int it = 0; it < batch; ++it) {
                launch_p(c, PROF_IN_SPMV, k_in_spmv, gr, bl, g, A32, z, pb[cur], pb[cur ^ 1], q, launched + it == 0 ? 1 : 0,
                                                    c->partials, c->counters + 10, in);
                cur ^= 1;
                if (mode == 1) {
                    int steps = o->degree - 1;
                    float* z0 = (steps % 2 == 1) ? c->f[6] : z;
                    launch_p(c, PROF_IN_UPDATE, k_in_update, gr, bl, g, A32, mode, alpha0, e, r, pb[cur], q, z0, c->partials,
                                                          c->counters + 11, in, out, o->max_iter);
                    if (steps > 0) st = inner_precond(c, o, A32, r, z, in, L32, 1, 0);
                    else launch(c, k_in_dot_beta, gr, bl, g, r, z, c->partials, c->counters + 13, in, 0);
                } else {
                    launch_p(c, PROF_IN_UPDATE, k_in_update, gr, bl, g, A32, mode, alpha0, e, r, pb[cur], q, z, c->partials,
                                                          c->counters + 11, in, out, o->max_iter);
                    if (mode == 2) st = inner_precond(c, o, A32, r, z, in, L32, 1, 0);
                }
                if (st) return st;
            }
            launched += batch;
            st = check_launch(c, "inner iteration");
            if (st) return st;
            st = read_state(c);
            if (st) return st;
            if (c->h_state[1].done || launched >= inner_cap) break;
            batch = batch < 32 ? batch * 2 : 32;
        }
        // ---- correction and the new FP64 residual
        if (c->fused && col_supported(c, o)) {
            st = col_x_update(c);   // x += e + alpha p: the column passes defer the last update of e
            if (st) return st;
        } else {
            launch(c, k_x_add, gr, bl, g, x, e);
        }
        ++outer;
        launch_p(c, PROF_OUTER, k_outer_resid, resid_grid(g), bl, g, A, x, b, r, c->partials, c->counters + 8, out, outer);
        st = check_launch(c, "outer correction");
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        if (c->h_state[1].status == LES_NONFINITE) break;
    }
    if (mode == 2) {   // the IC wavefront's bounded waits
        st = wave_check(c);
        if (st) return st;
    }
    const SolverState& h = c->h_state[0];
    if (res) {
        res->iters = h.iters;
        res->outer = outer;
        res->residual = h.err;
    }
    if (h.done) return (les_status)h.status;
    return LES_NOT_CONVERGED;
}

ViewF view32_of(les_ctx* c) { return view32(c); }
StencilView stencil_view_of(les_ctx* c) { return stencil_view(c); }

int batch_resid_blocks(const Geo& g)
{
    const dim3 r = resid_grid(g);
    return (int)(r.x * r.y * r.z);
}

les_status batch_outer_resid(cudaStream_t s, const BatchCase* cs, const int* pre, int n, int blocks)
{
    k_outer_resid_batch<<<blocks, cell_block(), 0, s>>>(cs, pre, n);
    return cudaPeekAtLastError() == cudaSuccess ? LES_OK : LES_CUDA_ERROR;
}

// Launch helpers for the graph-captured mixed solve (les_fused.cu): the same
// kernels as pcg_mixed_impl, with the outer count kept on the device.
les_status emit_outer_start(les_ctx* c, const les_pcg_opts* o, int keep_tol)
{
    const Geo& g = c->g;
    launch(c, k_set_outer, 1, 1, c->state, o->tol, keep_tol);
    launch_p(c, PROF_OUTER, k_outer_resid, resid_grid(g), cell_block(), g, stencil_view(c), (const double*)c->slot[LES_P],
             (const double*)c->slot[LES_B], c->f[0], c->partials, c->counters + 8, c->state, 0);
    return check_launch(c, "outer start");
}

les_status emit_inner_start(les_ctx* c, const les_pcg_opts* o, int inner_cap)
{
    launch(c, k_inner_init, 1, 1, c->state + 1, (const SolverState*)c->state, o->inner_rtol, inner_cap);
    return check_launch(c, "inner start");
}

les_status emit_outer_update(les_ctx* c, bool deferred)
{
    const Geo& g = c->g;
    if (deferred) {
        les_status st = col_x_update(c);
        if (st) return st;
    } else {
        launch(c, k_x_add, cell_grid(g), cell_block(), g, c->slot[LES_P], (const float*)c->f[5]);
    }
    launch_p(c, PROF_OUTER, k_outer_resid, resid_grid(g), cell_block(), g, stencil_view(c), (const double*)c->slot[LES_P],
             (const double*)c->slot[LES_B], c->f[0], c->partials, c->counters + 8, c->state, -1);
    return check_launch(c, "outer update");
}

les_status pcg_mixed(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res)
{
    return pcg_mixed_impl(c, o, res, 0);
}

}  // namespace les
