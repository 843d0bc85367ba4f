// les_pressure.cu -- the pressure system of les-model src/pressure.cpp on the
// device: divergence RHS, b vector, stencil assembly, the 7-point SpMV, the
// Jacobi and Chebyshev preconditioners, PCG in FP64, the power iteration for
// lambda_max, the pressure boundary conditions and the stationary Jacobi
// solver.  (IC(0) and GS-SOR, which need wavefront ordering, are in
// les_wavefront.cu; the mixed-precision solve is in les_mixed.cu.)
//
// Compiled with -fmad=false: every elementwise expression keeps the
// reference's rounding.  Dot products and norms are deterministic two-stage
// reductions (block tree, then the last block sums the block partials in
// order), so they differ from the reference's sequential sum only by
// reassociation.
#include <cmath>
#include <random>
#include <utility>
#include <vector>

#include "les_internal.cuh"

using namespace les;

namespace les {
les_status ic_apply_dev(les_ctx* c, const double* r, double* z, const double* const* Lsrc, int skip_done);
les_status wave_check(les_ctx* c);
les_status build_ic_dev(les_ctx* c);
les_status pcg_mixed(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res);
}

namespace {

__device__ __forceinline__ bool cell_coords(const Geo& g, int& i, int& j, int& k)
{
    k = blockIdx.x * TBK + threadIdx.x;
    j = blockIdx.y * TBJ + threadIdx.y;
    i = blockIdx.z;
    return k < g.nz && j < g.ny;
}

// fast_apply_laplacian body, src/pressure.cpp:721-744 (bounds tests kept so
// that the summation matches term for term).
__device__ __forceinline__ double apply_row(const StencilView& A, const double* __restrict__ p,
                                            const Geo& g, int i, int j, int k, int id)
{
    Coef7 a = A.at(id);
    double val = a.c * p[id];
    if (i > 0) val += a.w * p[id - g.si];
    if (i < g.nx - 1) val += a.e * p[id + g.si];
    if (j > 0) val += a.s * p[id - g.sj];
    if (j < g.ny - 1) val += a.n * p[id + g.sj];
    if (k > 0) val += a.b * p[id - 1];
    if (k < g.nz - 1) val += a.t * p[id + 1];
    return val;
}

// calculate_divergence (src/pressure.cpp:256-329) + build_b_vector
// (:566-599) in one pass, with ||b||^2 reduced on the side.
__global__ void k_div_b(Geo g, double scale, double idx, double idy, double idz, double idx1,
                        double idy1, double idz1, const double* __restrict__ un,
                        const double* __restrict__ vn, const double* __restrict__ wn,
                        const uint8_t* __restrict__ solid, double* __restrict__ rhs,
                        double* __restrict__ b, double* partials, unsigned* counter, SolverState* st,
                        double rel_tol, const double* dtp, double rho)
{
    __shared__ double sm[32];
    int i, j, k;
    double bb[1] = {0.0};
    if (dtp) scale = rho / *dtp;   // src/pressure.cpp:260, from the device dt
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        double r = 0.0;
        if (!(solid[id] || i == g.nx - 1)) {
            double du_dx, dv_dy, dw_dz;
            if (i == 0) du_dx = (un[id + g.si] - un[id]) * idx1;
            else du_dx = (un[id + g.si] - un[id - g.si]) * idx;
            if (j == 0) dv_dy = (vn[id + g.sj] - vn[id]) * idy1;
            else if (j == g.ny - 1) dv_dy = (vn[id] - vn[id - g.sj]) * idy1;
            else dv_dy = (vn[id + g.sj] - vn[id - g.sj]) * idy;
            if (k == 0) dw_dz = (wn[id + 1] - wn[id]) * idz1;
            else if (k == g.nz - 1) dw_dz = (wn[id] - wn[id - 1]) * idz1;
            else dw_dz = (wn[id + 1] - wn[id - 1]) * idz;
            r = scale * (du_dx + dv_dy + dw_dz);
            rhs[id] = r;
            double bv = -r;
            if (b) b[id] = bv;
            bb[0] = bv * bv;
        } else {
            rhs[id] = 0.0;
            if (b) b[id] = 0.0;
        }
    }
    if (!b) return;
    if (last_block_sum<1>(bb, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            st->bnorm = sqrt(bb[0]);
            if (rel_tol > 0) st->tol = rel_tol * st->bnorm;
        }
    }
}

__global__ void k_build_b(Geo g, const double* __restrict__ rhs, const uint8_t* __restrict__ solid,
                          double* __restrict__ b)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    b[id] = (solid[id] || i == g.nx - 1) ? 0.0 : -rhs[id];
}

// build_stencil (src/pressure.cpp:608-699) as one code byte per cell.
__global__ void k_build_code(Geo g, const uint8_t* __restrict__ solid, uint8_t* __restrict__ code,
                             unsigned* any_solid)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    if (solid[id]) *any_solid = 1u;   // every writer stores the same value
    if (solid[id] || i == g.nx - 1) { code[id] = 0; return; }
    bool W = (i == 0) || solid[id - g.si];
    bool E1 = (i == g.nx - 2);
    bool E2 = !E1 && solid[id + g.si];
    unsigned xs;
    if (E1) xs = W ? 3u : 2u;
    else if (E2) xs = W ? 2u : 4u;
    else xs = W ? 1u : 0u;
    bool S = (j == 0) || solid[id - g.sj];
    bool N = (j == g.ny - 1) || solid[id + g.sj];
    unsigned ys = S ? (N ? 3u : 1u) : (N ? 2u : 0u);
    bool B = (k == 0) || solid[id - 1];
    bool T = (k == g.nz - 1) || solid[id + 1];
    unsigned zs = B ? (T ? 3u : 1u) : (T ? 2u : 0u);
    code[id] = (uint8_t)(1u + xs + 5u * (ys + 4u * zs));
}

__global__ void k_expand_stencil(Geo g, StencilView A, double* c, double* n, double* s, double* e,
                                 double* w, double* t, double* b)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    Coef7 a = A.at(id);
    c[id] = a.c; n[id] = a.n; s[id] = a.s; e[id] = a.e; w[id] = a.w; t[id] = a.t; b[id] = a.b;
}

// out = A in (+ optional dot in.out reduced into the state).
enum { DOT_NONE = 0, DOT_ALPHA = 1, DOT_SCAL0 = 2 };

__global__ void k_spmv(Geo g, StencilView A, const double* __restrict__ p, double* __restrict__ q,
                       double* partials, unsigned* counter, SolverState* st, int dot_mode)
{
    __shared__ double sm[32];
    if (dot_mode == DOT_ALPHA && st->done) return;
    int i, j, k;
    double pq[1] = {0.0};
    if (cell_coords(g, i, j, k))
        for (; i < g.nx; i += gridDim.z) {   // planes blockIdx.z, + gridDim.z, ...
            const int id = i * g.si + j * g.sj + k;
            double val = apply_row(A, p, g, i, j, k, id);
            q[id] = val;
            pq[0] += p[id] * val;
        }
    if (dot_mode == DOT_NONE) return;
    if (last_block_sum<1>(pq, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (dot_mode == DOT_ALPHA) {
                st->pq = pq[0];
                st->alpha = st->rho / pq[0];   // src/pressure.cpp:378
            } else {
                st->scal[0] = pq[0];
            }
        }
    }
}

// r = b - q, ||r|| and the already-converged test of src/pressure.cpp:355-359.
__global__ void k_resid(Geo g, const double* __restrict__ b, const double* __restrict__ q,
                        double* __restrict__ r, double* partials, unsigned* counter, SolverState* st)
{
    __shared__ double sm[32];
    int i, j, k;
    double rr[1] = {0.0};
    if (cell_coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        double v = b[id] - q[id];   // 1.0*b + (-1.0)*q
        r[id] = v;
        rr[0] = v * v;
    }
    if (last_block_sum<1>(rr, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double e = sqrt(rr[0]);
            st->rr = rr[0];
            st->err = e;
            st->k = 0;
            if (e < st->tol) { st->done = 1; st->iters = 0; st->status = LES_OK; }
            else if (!isfinite(e)) { st->done = 1; st->iters = st->max_iter; st->status = LES_NONFINITE; }
        }
    }
}

// x += alpha p; r -= alpha q; ||r||; convergence test; k += 1
// (src/pressure.cpp:381-392).  With the Jacobi preconditioner fused
// (z = r / A_c, :420-428) it also forms r.z and the next beta.
__global__ void k_update(Geo g, StencilView A, double* __restrict__ x, double* __restrict__ r,
                         const double* __restrict__ p, const double* __restrict__ q,
                         double* __restrict__ z, double* partials, unsigned* counter,
                         SolverState* st, int jacobi)
{
    __shared__ double sm[64];
    if (st->done) return;
    const double alpha = st->alpha;
    int i, j, k;
    double acc[2] = {0.0, 0.0};
    if (cell_coords(g, i, j, k))
        for (; i < g.nx; i += gridDim.z) {   // planes blockIdx.z, + gridDim.z, ...
            const int id = i * g.si + j * g.sj + k;
            x[id] += alpha * p[id];
            double rv = r[id] + (-alpha) * q[id];
            r[id] = rv;
            acc[0] += rv * rv;
            if (jacobi) {
                double zv = rv / A.diag(id);
                z[id] = zv;
                acc[1] += rv * zv;
            }
        }
    if (last_block_sum<2>(acc, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double e = sqrt(acc[0]);
            int kk = st->k + 1;
            st->k = kk;
            st->rr = acc[0];
            st->err = e;
            if (e < st->tol) { st->done = 1; st->iters = kk; st->status = LES_OK; }
            else if (!isfinite(e)) { st->done = 1; st->iters = st->max_iter; st->status = LES_NONFINITE; }
            else if (kk >= st->max_iter) { st->done = 1; st->iters = st->max_iter; st->status = LES_NOT_CONVERGED; }
            if (jacobi) {
                st->rz = acc[1];
                st->beta = acc[1] / st->rho;   // :399-402
                st->rho = acc[1];
            }
        }
    }
}

enum { RD_RHO = 0, RD_BETA = 1, RD_SCAL0 = 2 };

// dot(a, b) reduced into the state: RD_RHO sets rho (:369); RD_BETA forms
// beta = rz/rho and rho = rz (:399-408); RD_SCAL0 stores into scal[0].
__global__ void k_dot(Geo g, const double* __restrict__ a, const double* __restrict__ b,
                      double* partials, unsigned* counter, SolverState* st, int mode, int skip_done)
{
    __shared__ double sm[32];
    if (skip_done && st->done) return;
    int i, j, k;
    double s[1] = {0.0};
    if (cell_coords(g, i, j, k))
        for (; i < g.nx; i += gridDim.z) {   // planes blockIdx.z, + gridDim.z, ...
            const int id = i * g.si + j * g.sj + k;
            s[0] += a[id] * b[id];
        }
    if (last_block_sum<1>(s, partials, counter, sm)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (mode == RD_RHO) st->rho = s[0];
            else if (mode == RD_BETA) { st->rz = s[0]; st->beta = s[0] / st->rho; st->rho = s[0]; }
            else st->scal[0] = s[0];
        }
    }
}

// p = 1.0*z + beta*p (src/pressure.cpp:405).
// out = a*in1 + b*in2 (parallel_saxpy, src/pressure.cpp:995-1002; with
// a = 1, in1 = out it is parallel_axpy, :983-989).  out may alias either input.
__global__ void k_axpby(Geo g, double a, const double* in1, double b, const double* in2, double* out)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    out[id] = a * in1[id] + b * in2[id];
}

__global__ void k_pupdate(Geo g, const double* __restrict__ z, double* __restrict__ p, SolverState* st)
{
    if (st->done) return;
    const double beta = st->beta;
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    p[id] = z[id] + beta * p[id];
}

__global__ void k_jacobi_pc(Geo g, StencilView A, const double* __restrict__ r, double* __restrict__ z,
                            SolverState* st, int skip_done)
{
    if (skip_done && st->done) return;
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    z[id] = r[id] / A.diag(id);
}

// Chebyshev preconditioner, src/pressure.cpp:851-906.  Step 0:
// z = 0.0 + alpha0 * r (p_0 = res_0 = r is implicit).
__global__ void k_cheb0(Geo g, double alpha0, const double* __restrict__ r, double* __restrict__ z,
                        SolverState* st, int skip_done)
{
    if (skip_done && st->done) return;
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    z[id] = 0.0 + alpha0 * r[id];
}

// One inner step: res = r - A z; p = res + beta p; z' = z + alpha p.
// pin == nullptr means p_{k-1} = r (first step).
__global__ void k_cheb_step(Geo g, StencilView A, double alpha, double beta,
                            const double* __restrict__ r, const double* __restrict__ zin,
                            const double* pin, double* pout, double* __restrict__ zout,
                            SolverState* st, int skip_done)
{
    if (skip_done && st->done) return;
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    double az = apply_row(A, zin, g, i, j, k, id);
    double rv = r[id];
    double res = rv - az;
    double pv = res + beta * (pin ? pin[id] : rv);
    pout[id] = pv;
    zout[id] = zin[id] + alpha * pv;
}

// apply_pressure_BCs, src/pressure.cpp:14-93, face part.  The ordered face
// loops leave every face cell equal to g(i, J(j), K(k)) where J, K clamp to
// [1, n-2] and g(i, j', k') = P(1, j', k') for i == 0, 0 for i == nx-1,
// P(i, j', k') otherwise (P: the values before the call).  `in` may equal
// `out` (faces read interior cells only).
__global__ void k_pbc_faces(Geo g, const double* in, double* out)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (jk_in && i > 0 && i < g.nx - 1) return;
    const int id = i * g.si + j * g.sj + k;
    if (i == g.nx - 1) { out[id] = 0.0; return; }
    int jj = j < 1 ? 1 : (j > g.ny - 2 ? g.ny - 2 : j);
    int kk = k < 1 ? 1 : (k > g.nz - 2 ? g.nz - 2 : k);
    int ii = i == 0 ? 1 : i;
    out[id] = in[ii * g.si + jj * g.sj + kk];
}

// Obstacle part (:73-92): first fluid neighbour in the order +i,-i,+j,-j,+k,-k.
__global__ void k_pbc_obstacle(Geo g, const int* __restrict__ list, int n, const uint8_t* __restrict__ solid,
                               double* __restrict__ p)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int id = list[t];
    if (!solid[id + g.si]) p[id] = p[id + g.si];
    else if (!solid[id - g.si]) p[id] = p[id - g.si];
    else if (!solid[id + g.sj]) p[id] = p[id + g.sj];
    else if (!solid[id - g.sj]) p[id] = p[id - g.sj];
    else if (!solid[id + 1]) p[id] = p[id + 1];
    else if (!solid[id - 1]) p[id] = p[id - 1];
}

// Interior RHS of the stationary solvers, src/pressure.cpp:119-132 / :197-210.
__global__ void k_stat_rhs(Geo g, double coef, double two_dx, double two_dy, double two_dz,
                           const double* __restrict__ u, const double* __restrict__ v,
                           const double* __restrict__ w, double* __restrict__ rhs)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 1 || k > g.nz - 2) { rhs[id] = 0.0; return; }
    double div = (u[id + g.si] - u[id - g.si]) / two_dx + (v[id + g.sj] - v[id - g.sj]) / two_dy +
                 (w[id + 1] - w[id - 1]) / two_dz;
    rhs[id] = coef * div;
}

// One Jacobi sweep, src/pressure.cpp:139-157, plus max|dp| reduced into the
// state (max is order-independent, so this is exact).
__global__ void k_jacobi_sweep(Geo g, double dx2, double dy2, double dz2, double denom,
                               const double* __restrict__ cur, double* __restrict__ nxt,
                               const double* __restrict__ rhs, double* partials, unsigned* counter,
                               SolverState* st)
{
    __shared__ double sm[32];
    __shared__ int am_last;
    if (st->done) return;
    int i, j, k;
    double m = 0.0;
    if (cell_coords(g, i, j, k) && i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2 && k >= 1 &&
        k <= g.nz - 2) {
        const int id = i * g.si + j * g.sj + k;
        double p_old = cur[id];
        double v = ((cur[id + g.si] + cur[id - g.si]) / dx2 + (cur[id + g.sj] + cur[id - g.sj]) / dy2 +
                    (cur[id + 1] + cur[id - 1]) / dz2 - rhs[id]) /
                   denom;
        nxt[id] = v;
        m = fabs(v - p_old);
    }
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, lane = tid & 31, warp = tid >> 5;
    m = warp_max(m);
    if (lane == 0) sm[warp] = m;
    __syncthreads();
    const int nw = (blockDim.x * blockDim.y) >> 5, nb = block_count(), bid = block_linear_id();
    if (tid == 0) {
        double a = 0.0;
        for (int q = 0; q < nw; ++q) a = fmax(a, sm[q]);
        partials[bid] = a;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == (unsigned)nb - 1u;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    double a = 0.0;
    for (int q = tid; q < nb; q += blockDim.x * blockDim.y) a = fmax(a, __ldcg(partials + q));
    a = warp_max(a);
    __syncthreads();
    if (lane == 0) sm[warp] = a;
    __syncthreads();
    if (tid == 0) {
        double r = 0.0;
        for (int q = 0; q < nw; ++q) r = fmax(r, sm[q]);
        st->maxdp = r;
        *counter = 0u;
    }
}

// After the BCs of a sweep: count it and test max|dp| < tol (:164-170).
__global__ void k_stat_check(SolverState* st, int sweep_buf)
{
    if (st->done) return;
    st->k += 1;
    st->buf = sweep_buf;
    if (st->maxdp < st->tol) { st->done = 1; st->iters = st->k; st->status = LES_OK; }
    else if (st->k >= st->max_iter) { st->done = 1; st->iters = st->k; st->status = LES_NOT_CONVERGED; }
}

__global__ void k_pbc_faces_guarded(Geo g, const double* in, double* out, SolverState* st)
{
    if (st->done) return;
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (jk_in && i > 0 && i < g.nx - 1) return;
    const int id = i * g.si + j * g.sj + k;
    if (i == g.nx - 1) { out[id] = 0.0; return; }
    int jj = j < 1 ? 1 : (j > g.ny - 2 ? g.ny - 2 : j);
    int kk = k < 1 ? 1 : (k > g.nz - 2 ? g.nz - 2 : k);
    int ii = i == 0 ? 1 : i;
    out[id] = in[ii * g.si + jj * g.sj + kk];
}

__global__ void k_pbc_obstacle_guarded(Geo g, const int* __restrict__ list, int n,
                                       const uint8_t* __restrict__ solid, double* __restrict__ p,
                                       SolverState* st)
{
    if (st->done) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int id = list[t];
    if (!solid[id + g.si]) p[id] = p[id + g.si];
    else if (!solid[id - g.si]) p[id] = p[id - g.si];
    else if (!solid[id + g.sj]) p[id] = p[id + g.sj];
    else if (!solid[id - g.sj]) p[id] = p[id - g.sj];
    else if (!solid[id + 1]) p[id] = p[id + 1];
    else if (!solid[id - 1]) p[id] = p[id - 1];
}

__global__ void k_scale_inv(Geo g, double* __restrict__ v, const double* __restrict__ w, SolverState* st)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    v[id] = w[id] / st->scal[1];
}

__global__ void k_norm_of(SolverState* st)
{
    st->scal[1] = sqrt(st->scal[0]);
}

__global__ void k_init_state(SolverState* st, double tol, int max_iter, int keep_tol)
{
    if (!keep_tol) st->tol = tol;
    st->max_iter = max_iter;
    st->k = 0;
    st->done = 0;
    st->iters = 0;
    st->status = LES_OK;
    st->buf = 0;
    st->err = 0.0;
}

}  // namespace

namespace les {

les_status spmv_dev(les_ctx* c, const double* in, double* out)
{
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix: call les_build_stencil or les_set_stencil");
    launch(c, k_spmv, cell_grid(c->g), cell_block(), c->g, stencil_view(c), in, out, c->partials,
                                                             c->counters + 1, c->state, DOT_NONE);
    return check_launch(c, "spmv");
}

les_status dot_dev(les_ctx* c, const double* a, const double* b, double* out_host)
{
    launch(c, k_dot, cell_grid(c->g), cell_block(), c->g, a, b, c->partials, c->counters + 2,
                                                            c->state, RD_SCAL0, 0);
    les_status st = check_launch(c, "dot");
    if (st) return st;
    st = read_state(c);
    if (st) return st;
    if (out_host) *out_host = c->h_state->scal[0];
    return LES_OK;
}

les_status div_b_dev(les_ctx* c, double dt, double rho, double rel_tol, const double* dtp)
{
    const les_mesh& m = c->mesh;
    launch(c, k_div_b, cell_grid(c->g), cell_block(),
        c->g, rho / dt, 1.0 / (2.0 * m.dx), 1.0 / (2.0 * m.dy), 1.0 / (2.0 * m.dz), 1.0 / m.dx,
        1.0 / m.dy, 1.0 / m.dz, c->slot[LES_U_NEW], c->slot[LES_V_NEW], c->slot[LES_W_NEW], c->mask,
        c->slot[LES_P_RHS], c->slot[LES_B], c->partials, c->counters + 3, c->state, rel_tol, dtp, rho);
    return check_launch(c, "divergence+b");
}

les_status pressure_bcs_dev(les_ctx* c, double* p)
{
    launch(c, k_pbc_faces, cell_grid(c->g), cell_block(), c->g, p, p);
    if (c->n_solid)
        launch(c, k_pbc_obstacle, (c->n_solid + 255) / 256, 256, c->g, c->solid_list, c->n_solid,
                                                                          c->mask, p);
    return check_launch(c, "pressure bcs");
}

// Preconditioner application r -> z for PCG; kernels are skipped once the
// state says done (skip_done).
les_status precond_dev(les_ctx* c, const les_pcg_opts* o, const double* r, double* z, int skip_done)
{
    const Geo& g = c->g;
    StencilView A = stencil_view(c);
    switch (o->precond) {
    case LES_PC_JACOBI:
        launch(c, k_jacobi_pc, cell_grid(g), cell_block(), g, A, r, z, c->state, skip_done);
        return check_launch(c, "jacobi pc");
    case LES_PC_CHEBYSHEV: {
        if (o->degree < 1) return fail(c, LES_BAD_ARG, "Chebyshev degree must be >= 1");
        les_status st = ensure_work(c);
        if (st) return st;
        const double d = (o->lambda_max + o->lambda_min) / 2.0;
        const double cc = (o->lambda_max - o->lambda_min) / 2.0;
        double alpha = 2.0 / d;
        const int steps = o->degree - 1;
        // ping-pong z so that the last write lands in `z`
        double* zb[2] = {z, c->w[6]};
        int cur = (steps % 2 == 0) ? 0 : 1;
        launch(c, k_cheb0, cell_grid(g), cell_block(), g, alpha, r, zb[cur], c->state, skip_done);
        double* pbuf = c->w[7];
        for (int kq = 1; kq <= steps; ++kq) {
            double beta = (cc * alpha / 2.0) * (cc * alpha / 2.0);
            alpha = 1.0 / (d - beta);
            launch_p(c, PROF_CHEB64, k_cheb_step, cell_grid(g), cell_block(), 
                g, A, alpha, beta, r, zb[cur], kq == 1 ? nullptr : pbuf, pbuf, zb[cur ^ 1], c->state,
                skip_done);
            cur ^= 1;
        }
        return check_launch(c, "chebyshev pc");
    }
    case LES_PC_IC:
        if (!c->have_L) return fail(c, LES_BAD_ARG, "IC preconditioner needs les_build_ic or les_set_ic_factor");
        return ic_apply_dev(c, r, z, nullptr, skip_done);
    case LES_PC_IC_A: {
        // the factor arrays are A itself (src/pressure.cpp:363, :396)
        if (!c->A_valid) return fail(c, LES_BAD_ARG, "internal: IC-with-A needs A as arrays");
        const double* Ad[7] = {c->A[0], c->A[1], c->A[2], c->A[3], c->A[4], c->A[5], c->A[6]};
        return ic_apply_dev(c, r, z, Ad, skip_done);
    }
    default:
        return fail(c, LES_BAD_ARG, "unknown preconditioner");
    }
}

// The IC-with-A mode needs A as arrays; expand the coded matrix on demand.
les_status ensure_stored_A(les_ctx* c)
{
    if (c->A_valid) return LES_OK;
    if (c->stencil_mode != 1) return fail(c, LES_BAD_ARG, "no matrix");
    const size_t nb = sizeof(double) * (size_t)c->g.n;
    for (int q = 0; q < 7; ++q)
        if (!c->A[q]) {
            les_status st = check_cuda(c, cudaMalloc(&c->A[q], nb), "cudaMalloc(A)");
            if (st) return st;
        }
    launch(c, k_expand_stencil, cell_grid(c->g), cell_block(), 
        c->g, stencil_view(c), c->A[0], c->A[1], c->A[2], c->A[3], c->A[4], c->A[5], c->A[6]);
    // keep using the codes for the SpMV; the arrays are an exact copy
    c->A_valid = true;
    return check_launch(c, "expand stencil");
}

// Grid of the FP64 solver's reductions in its iterations: every (k, j) tile
// once and the i-planes shared out so that about eight blocks per SM run,
// each summing its planes before the grid sum -- one partial, fence and
// atomic per block instead of one per block and plane (16384 at
// 256x128x128).  The kernels loop over planes i = blockIdx.z + t gridDim.z.
static dim3 reduce_grid(const les_ctx* c)
{
    dim3 gr = cell_grid(c->g);
    const long long tiles = (long long)gr.x * gr.y;
    const long long z = (8LL * c->sms + tiles - 1) / tiles;
    gr.z = (unsigned)(z < 1 ? 1 : (z > c->g.nx ? c->g.nx : z));
    return gr;
}

// PCG of src/pressure.cpp:342-414 in FP64 with the solution in P and the
// right-hand side in B.  The loop runs on the device; the host only polls
// the state between batches of iterations (kernels after convergence exit
// at once).
les_status pcg_fp64(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol)
{
    const Geo& g = c->g;
    les_status st = ensure_work(c);
    if (st) return st;
    if (o->precond == LES_PC_IC_A) {
        st = ensure_stored_A(c);
        if (st) return st;
    }
    StencilView A = stencil_view(c);
    double *x = c->slot[LES_P], *b = c->slot[LES_B];
    double *r = c->w[0], *z = c->w[1], *p = c->w[2], *q = c->w[3];
    const dim3 gr = cell_grid(g), bl = cell_block();
    launch(c, k_init_state, 1, 1, c->state, o->tol, o->max_iter, keep_tol);
    launch(c, k_spmv, gr, bl, g, A, x, q, c->partials, c->counters + 1, c->state, DOT_NONE);
    launch(c, k_resid, gr, bl, g, b, q, r, c->partials, c->counters + 4, c->state);
    st = precond_dev(c, o, r, p, 1);
    if (st) return st;
    launch(c, k_dot, gr, bl, g, r, p, c->partials, c->counters + 2, c->state, RD_RHO, 1);
    st = check_launch(c, "pcg init");
    if (st) return st;
    if (o->max_iter == 0) {
        // the reference's loop does not run; it returns max_iter (= 0)
        st = read_state(c);
        if (st) return st;
        if (res) { res->iters = 0; res->outer = 0; res->residual = c->h_state->err; }
        return c->h_state->done ? (les_status)c->h_state->status : LES_NOT_CONVERGED;
    }
    const bool jac = o->precond == LES_PC_JACOBI;
    const dim3 grr = reduce_grid(c);
    int launched = 0, batch = 4;
    for (;;) {
        for (int it = 0; it < batch; ++it) {
            launch_p(c, PROF_SPMV64, k_spmv, grr, bl, g, A, p, q, c->partials, c->counters + 1, c->state, DOT_ALPHA);
            launch_p(c, PROF_UPDATE64, k_update, grr, bl, g, A, x, r, p, q, z, c->partials, c->counters + 5, c->state,
                                                jac ? 1 : 0);
            if (!jac) {
                st = precond_dev(c, o, r, z, 1);
                if (st) return st;
                launch(c, k_dot, grr, bl, g, r, z, c->partials, c->counters + 2, c->state, RD_BETA, 1);
            }
            launch(c, k_pupdate, gr, bl, g, z, p, c->state);
        }
        launched += batch;
        st = check_launch(c, "pcg iteration");
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        if (c->h_state->done || launched >= o->max_iter + 1) break;
        batch = batch < 32 ? batch * 2 : 32;
        if (launched + batch > o->max_iter + 1) batch = o->max_iter + 1 - launched;
        if (batch < 1) batch = 1;
    }
    if (o->precond == LES_PC_IC || o->precond == LES_PC_IC_A) {   // the wavefront's bounded waits
        st = wave_check(c);
        if (st) return st;
    }
    const SolverState& h = *c->h_state;
    if (res) {
        res->iters = h.iters;
        res->outer = 0;
        res->residual = h.err;
    }
    if (!h.done) return fail(c, LES_NOT_CONVERGED, "pcg: state not finalised");
    return (les_status)h.status;
}

les_status solve_jacobi_dev(les_ctx* c, double dt, double rho, int max_iter, double tol, int* sweeps)
{
    const Geo& g = c->g;
    les_status st = ensure_work(c);
    if (st) return st;
    const les_mesh& m = c->mesh;
    const dim3 gr = cell_grid(g), bl = cell_block();
    double* rhs = c->w[0];
    double* bufs[2] = {c->slot[LES_P], c->w[1]};
    const double dx2 = m.dx * m.dx, dy2 = m.dy * m.dy, dz2 = m.dz * m.dz;
    const double denom = 2 * (1.0 / dx2 + 1.0 / dy2 + 1.0 / dz2);
    launch(c, k_stat_rhs, gr, bl, g, rho / dt, 2 * m.dx, 2 * m.dy, 2 * m.dz, c->slot[LES_U],
                                         c->slot[LES_V], c->slot[LES_W], rhs);
    launch(c, k_init_state, 1, 1, c->state, tol, max_iter, 0);
    int launched = 0, batch = 8;
    int cur = 0;
    for (;;) {
        for (int it = 0; it < batch && launched < max_iter; ++it, ++launched) {
            launch(c, k_jacobi_sweep, gr, bl, g, dx2, dy2, dz2, denom, bufs[cur], bufs[cur ^ 1], rhs,
                                                     c->partials, c->counters + 6, c->state);
            cur ^= 1;
            launch(c, k_pbc_faces_guarded, gr, bl, g, bufs[cur], bufs[cur], c->state);
            if (c->n_solid)
                launch(c, k_pbc_obstacle_guarded, (c->n_solid + 255) / 256, 256, 
                    g, c->solid_list, c->n_solid, c->mask, bufs[cur], c->state);
            launch(c, k_stat_check, 1, 1, c->state, cur);
        }
        st = check_launch(c, "jacobi sweeps");
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        if (c->h_state->done || launched >= max_iter) break;
        batch = 16;
    }
    if (max_iter <= 0) {
        if (sweeps) *sweeps = 0;
        return LES_OK;
    }
    // the converged field sits in bufs[state.buf]; mirror f.p.swap(p_new)
    if (c->h_state->buf == 1) std::swap(c->slot[LES_P], c->w[1]);
    if (sweeps) *sweeps = c->h_state->iters;
    return LES_OK;
}

}  // namespace les

extern "C" {

les_status les_divergence(les_ctx* c, double dt, double rho)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    const les_mesh& m = c->mesh;
    launch(c, k_div_b, cell_grid(c->g), cell_block(), 
        c->g, rho / dt, 1.0 / (2.0 * m.dx), 1.0 / (2.0 * m.dy), 1.0 / (2.0 * m.dz), 1.0 / m.dx,
        1.0 / m.dy, 1.0 / m.dz, c->slot[LES_U_NEW], c->slot[LES_V_NEW], c->slot[LES_W_NEW], c->mask,
        c->slot[LES_P_RHS], nullptr, c->partials, c->counters + 3, c->state, 0.0, nullptr, rho);
    return check_launch(c, "divergence");
}

les_status les_build_b(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    launch(c, k_build_b, cell_grid(c->g), cell_block(), c->g, c->slot[LES_P_RHS], c->mask,
                                                                c->slot[LES_B]);
    return check_launch(c, "build b");
}

les_status les_pressure_bcs(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return pressure_bcs_dev(c, c->slot[LES_P]);
}

les_status les_build_stencil(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    if (!c->code) {
        les_status st = check_cuda(c, cudaMalloc(&c->code, (size_t)c->g.n), "cudaMalloc(code)");
        if (st) return st;
    }
    const les_mesh& m = c->mesh;
    const double idx2 = 1.0 / (m.dx * m.dx), idy2 = 1.0 / (m.dy * m.dy), idz2 = 1.0 / (m.dz * m.dz);
    // src/pressure.cpp:613-623, and the doubled ghost coefficients of :663-696
    c->coef.c0 = (2.0 * idx2 + 2.0 * idy2 + 2.0 * idz2);
    c->coef.x1 = -idx2; c->coef.x2 = -idx2 + -idx2;
    c->coef.y1 = -idy2; c->coef.y2 = -idy2 + -idy2;
    c->coef.z1 = -idz2; c->coef.z2 = -idz2 + -idz2;
    unsigned* any_solid = c->counters + 30;
    les_status st = check_cuda(c, cudaMemsetAsync(any_solid, 0, sizeof(unsigned), c->stream), "memset");
    if (st) return st;
    launch(c, k_build_code, cell_grid(c->g), cell_block(), c->g, c->mask, c->code, any_solid);
    c->stencil_mode = 1;
    ++c->version;
    c->A_valid = false;   // a stale expansion of an older matrix must not be used
    if ((st = check_launch(c, "build stencil"))) return st;
    unsigned h = 1;
    st = check_cuda(c, cudaMemcpyAsync(&h, any_solid, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "copy");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "build stencil");
    c->code_plain = st == LES_OK && h == 0u;
    return st;
}

les_status les_get_stencil(les_ctx* c, double* const* diag7)
{
    if (!c || !diag7) return LES_BAD_ARG;
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix");
    cudaSetDevice(c->device);
    les_status st = ensure_work(c);
    if (st) return st;
    const size_t nb = sizeof(double) * (size_t)c->g.n;
    double* tmp[7];
    for (int q = 0; q < 7; ++q) {
        st = check_cuda(c, cudaMalloc(&tmp[q], nb), "cudaMalloc(tmp)");
        if (st) return st;
    }
    launch(c, k_expand_stencil, cell_grid(c->g), cell_block(), c->g, stencil_view(c), tmp[0], tmp[1],
                                                                       tmp[2], tmp[3], tmp[4], tmp[5], tmp[6]);
    for (int q = 0; q < 7; ++q)
        if (diag7[q]) cudaMemcpyAsync(diag7[q], tmp[q], nb, cudaMemcpyDeviceToHost, c->stream);
    st = check_cuda(c, cudaStreamSynchronize(c->stream), "get stencil");
    for (int q = 0; q < 7; ++q) cudaFree(tmp[q]);
    return st;
}

les_status les_spmv(les_ctx* c, int in, int out)
{
    if (!c || in < 0 || in >= LES_NSLOTS || out < 0 || out >= LES_NSLOTS || in == out) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return spmv_dev(c, c->slot[in], c->slot[out]);
}

les_status les_dot(les_ctx* c, int a, int b, double* out)
{
    if (!c || a < 0 || a >= LES_NSLOTS || b < 0 || b >= LES_NSLOTS || !out) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return dot_dev(c, c->slot[a], c->slot[b], out);
}

les_status les_axpby(les_ctx* c, int out, double a, int in1, double b, int in2)
{
    if (!c || out < 0 || out >= LES_NSLOTS || in1 < 0 || in1 >= LES_NSLOTS || in2 < 0 || in2 >= LES_NSLOTS)
        return LES_BAD_ARG;
    cudaSetDevice(c->device);
    launch(c, k_axpby, cell_grid(c->g), cell_block(), c->g, a, (const double*)c->slot[in1], b,
           (const double*)c->slot[in2], c->slot[out]);
    return check_launch(c, "axpby");
}

les_status les_precond_apply(les_ctx* c, const les_pcg_opts* o, int in, int out)
{
    if (!c || !o || in < 0 || in >= LES_NSLOTS || out < 0 || out >= LES_NSLOTS || in == out) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    if (!c->stencil_mode && o->precond != LES_PC_IC) return fail(c, LES_BAD_ARG, "no matrix");
    if (o->precond == LES_PC_IC_A) {
        les_status st = ensure_stored_A(c);
        if (st) return st;
    }
    les_status st = precond_dev(c, o, c->slot[in], c->slot[out], 0);
    if (!st && (o->precond == LES_PC_IC || o->precond == LES_PC_IC_A))
        st = wave_check(c);   // waits for the wavefront: LES_TIMEOUT if a bounded wait gave up
    return st;
}

les_status les_pcg(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res)
{
    if (!c || !o || o->max_iter < 0) return LES_BAD_ARG;
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix: call les_build_stencil or les_set_stencil");
    cudaSetDevice(c->device);
    if (o->precision == LES_MIXED) return pcg_mixed(c, o, res);
    return pcg_fp64(c, o, res, 0);
}

les_status les_solve_jacobi(les_ctx* c, double dt, double rho, int max_iter, double tol, int* sweeps)
{
    if (!c || max_iter < 0) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return solve_jacobi_dev(c, dt, rho, max_iter, tol, sweeps);
}

les_status les_lambda_max(les_ctx* c, int n_iter, const double* v0, double* lambda)
{
    if (!c || !lambda || n_iter < 0) return LES_BAD_ARG;
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix");
    cudaSetDevice(c->device);
    les_status st = ensure_work(c);
    if (st) return st;
    const Geo& g = c->g;
    std::vector<double> h;
    if (!v0) {
        // src/pressure.cpp:926-931 as drawn by one thread
        h.resize(g.n);
        std::mt19937 gen(1337);
        std::uniform_real_distribution<> dis(-1.0, 1.0);
        for (int i = 0; i < g.n; ++i) h[i] = dis(gen);
        v0 = h.data();
    }
    double *v = c->w[0], *w = c->w[1];
    st = check_cuda(c, cudaMemcpyAsync(v, v0, sizeof(double) * g.n, cudaMemcpyHostToDevice, c->stream), "upload v0");
    if (st) return st;
    const dim3 gr = cell_grid(g), bl = cell_block();
    StencilView A = stencil_view(c);
    double lam = 0.0;
    for (int it = 0; it < n_iter; ++it) {
        launch(c, k_spmv, gr, bl, g, A, v, w, c->partials, c->counters + 1, c->state, DOT_SCAL0);
        // lambda = v.w (spmv's fused dot is p.q = v.w)
        st = read_state(c);
        if (st) return st;
        lam = c->h_state->scal[0];
        launch(c, k_dot, gr, bl, g, w, w, c->partials, c->counters + 2, c->state, RD_SCAL0, 0);
        launch(c, k_norm_of, 1, 1, c->state);
        launch(c, k_scale_inv, gr, bl, g, v, w, c->state);   // v = w / ||w||
        st = check_launch(c, "lambda iteration");
        if (st) return st;
    }
    st = check_cuda(c, cudaStreamSynchronize(c->stream), "sync");
    if (st) return st;
    *lambda = lam;
    return LES_OK;
}

}  // extern "C"
