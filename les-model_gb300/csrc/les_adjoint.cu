// les_adjoint.cu -- discrete adjoint of the time step for gradients of a
// time-averaged objective with respect to the inlet u-profile and Cs.
//
// Forward map of one step (src/main.cpp:115-144, FP64 PCG, fixed dt), from
// the velocity U = (u, v, w) after the previous step's boundary conditions:
//     nu_t = SGS(U; Cs) with the nu_t boundary values
//     X1   = M(U, nu_t)              momentum, interior cells
//     X2   = BC(X1; u_in)            velocity boundary conditions
//     b    = -(rho/dt) D U           divergence of the velocity *before* the
//                                    momentum update (the reference's
//                                    u <-> u_new swap precedes it), masked
//     p    = A^-1 b
//     X3   = X2 - (dt/rho) G p       interior cells
//     U'   = BC(X3; u_in)
// The adjoint runs these backwards with hand-written transposes (all in
// gather form: each cell collects what its neighbours' outputs owe it, so
// there are no atomics):
//     lX3 = BC^T lU' (+ inlet gradient);   lp = -(dt/rho) G^T lX3
//     lb  = A^-T lp;                       lU  = -(rho/dt) D^T lb
//     lX1 = BC^T lX3 (+ inlet gradient);   lU += M_U^T lX1, lnu = M_nu^T lX1
//     lnu = 0 where the nu_t boundary values overwrite it
//     lU += SGS_U^T lnu;                   dJ/dCs += SGS_Cs^T lnu
// The matrix A is non-symmetric only through the Neumann rows with doubled
// coefficients: S = W A is symmetric for W = 1/2 per mirrored axis (inlet
// plane, j walls, k walls), so A^-T g = W A^-1 (W^-1 g) and the adjoint solve
// is the forward PCG on a scaled right-hand side.
//
// Objective: J = (1/N) sum_{n=1..N} sum_{cells in the probe box} |U_n|^2 / 2.
// Checkpoints: U and p every K steps; the backward sweep restores each
// checkpoint, recomputes its segment (keeping each step's input U) and
// reverses it.  dt is fixed (the adaptive dt is a maximum over the grid, not
// differentiable).
#include <cmath>
#include <cstring>
#include <vector>

#include "les_internal.cuh"

using namespace les;

namespace les {
les_status sgs_nut_dev(les_ctx* c, double cs, int want_tau);
les_status velocity_bcs_dev(les_ctx* c);
les_status pcg_fp64(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status pcg_mixed_impl(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status dot_dev(les_ctx* c, const double* a, const double* b, double* out_host);

struct AdjWork {
    les_adjoint_params prm{};
    int nck = 0;                   // checkpoints
    size_t n = 0;
    std::vector<double*> ck;       // nck x (u, v, w, p)
    std::vector<double*> seg;      // K x (u, v, w): inputs of the steps of a segment
    double* lu[3] = {};            // adjoint of the current velocity
    double* lx[3] = {};            // adjoint of an intermediate velocity
    double* lnu = nullptr;         // adjoint of nu_t
    double* h[6] = {};             // SGS adjoint fields (xx, yy, zz, xy, xz, yz)
    double* lp = nullptr;          // adjoint of p, then W^-1 lp
    double* lb = nullptr;          // A^-1 W^-1 lp (warm start between steps), then W (...)
    double* grad_in = nullptr;     // ny*nz
    double* acc = nullptr;         // [0] J, [1] dJ/dCs
    bool forward_done = false;
};

void adj_work_free(AdjWork* a)
{
    if (!a) return;
    for (double* p : a->ck) cudaFree(p);
    for (double* p : a->seg) cudaFree(p);
    for (double* p : a->lu) cudaFree(p);
    for (double* p : a->lx) cudaFree(p);
    for (double* p : a->h) cudaFree(p);
    cudaFree(a->lnu);
    cudaFree(a->lp);
    cudaFree(a->lb);
    cudaFree(a->grad_in);
    cudaFree(a->acc);
    delete a;
}
}  // namespace les

namespace {

struct Dx {
    double i2dx, i2dy, i2dz;   // 1/(2h)
    double idx, idy, idz;      // 1/h
    double idx2, idy2, idz2;   // 1/h^2
};

Dx dx_of(const les_mesh& m)
{
    Dx d;
    d.i2dx = 1.0 / (2.0 * m.dx); d.i2dy = 1.0 / (2.0 * m.dy); d.i2dz = 1.0 / (2.0 * m.dz);
    d.idx = 1.0 / m.dx; d.idy = 1.0 / m.dy; d.idz = 1.0 / m.dz;
    d.idx2 = 1.0 / (m.dx * m.dx); d.idy2 = 1.0 / (m.dy * m.dy); d.idz2 = 1.0 / (m.dz * m.dz);
    return d;
}

__device__ __forceinline__ bool interior(const Geo& g, int i, int j, int k)
{
    return i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
}

__device__ __forceinline__ bool coords(const Geo& g, int& i, int& j, int& k)
{
    k = blockIdx.x * TBK + threadIdx.x;
    j = blockIdx.y * TBJ + threadIdx.y;
    i = blockIdx.z;
    return k < g.nz && j < g.ny;
}

// objective: acc[0] += scale * sum_box |U|^2 / 2; lu = (or +=) scale * U in the box
__global__ void k_objective(Geo g, int i0, int i1, int j0, int j1, int k0, int k1, double scale,
                            const double* __restrict__ u, const double* __restrict__ v,
                            const double* __restrict__ w, double* lu, double* lv, double* lw, int add_adjoint,
                            double* partials, unsigned* counter, double* acc)
{
    __shared__ double sm[32];
    int i, j, k;
    double e[1] = {0.0};
    if (coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        if (i >= i0 && i < i1 && j >= j0 && j < j1 && k >= k0 && k < k1) {
            e[0] = 0.5 * (u[id] * u[id] + v[id] * v[id] + w[id] * w[id]);
            if (add_adjoint) {
                lu[id] += scale * u[id];
                lv[id] += scale * v[id];
                lw[id] += scale * w[id];
            }
        }
    }
    if (last_block_sum<1>(e, partials, counter, sm))
        if (threadIdx.x == 0 && threadIdx.y == 0) acc[0] += scale * e[0];
}

// transpose of the velocity boundary conditions (k_velocity_faces then the
// interior solid overwrite): lx from ly; the inlet u of each non-solid inlet
// cell is the control, so its adjoint accumulates into grad_in
__global__ void k_adj_bc(Geo g, const uint8_t* __restrict__ solid, const double* __restrict__ ly,
                         const double* __restrict__ lyv, const double* __restrict__ lyw, double* __restrict__ lx,
                         double* __restrict__ lxv, double* __restrict__ lxw, double* __restrict__ grad_in)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    const bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    double a = 0.0, b = 0.0, c = 0.0;
    if (!jk_in) {
        // wall: overwritten with 0
    } else if (i == 0) {
        if (solid[id]) { a = ly[id]; b = lyv[id]; c = lyw[id]; }   // left as it was
        else grad_in[j * g.nz + k] += ly[id];
    } else if (i == g.nx - 1) {
        // outlet: overwritten by the copy of plane nx-2
    } else {
        if (!solid[id]) { a = ly[id]; b = lyv[id]; c = lyw[id]; }
        if (i == g.nx - 2) { a += ly[id + g.si]; b += lyv[id + g.si]; c += lyw[id + g.si]; }
    }
    lx[id] = a; lxv[id] = b; lxw[id] = c;
}

// lp = -(dt/rho) G^T lx over the interior cells that the correction updates
__global__ void k_adj_correct(Geo g, Dx d, double dt_over_rho, const double* __restrict__ lx,
                              const double* __restrict__ lxv, const double* __restrict__ lxw, double* __restrict__ lp)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    double s = 0.0;
    // p[c] enters u at c-ex with +1/(2dx) and at c+ex with -1/(2dx)
    if (interior(g, i - 1, j, k)) s += lx[id - g.si] * d.i2dx;
    if (interior(g, i + 1, j, k)) s -= lx[id + g.si] * d.i2dx;
    if (interior(g, i, j - 1, k)) s += lxv[id - g.sj] * d.i2dy;
    if (interior(g, i, j + 1, k)) s -= lxv[id + g.sj] * d.i2dy;
    if (interior(g, i, j, k - 1)) s += lxw[id - 1] * d.i2dz;
    if (interior(g, i, j, k + 1)) s -= lxw[id + 1] * d.i2dz;
    lp[id] = -dt_over_rho * s;
}

// symmetrising weight of the pressure matrix: 1/2 per mirrored axis
__device__ __forceinline__ double wsym(const Geo& g, int i, int j, int k)
{
    if (i == g.nx - 1) return 1.0;   // identity rows, decoupled
    double w = (i == 0) ? 0.5 : 1.0;
    if (j == 0 || j == g.ny - 1) w *= 0.5;
    if (k == 0 || k == g.nz - 1) w *= 0.5;
    return w;
}

__global__ void k_scale_w(Geo g, double* __restrict__ a, int inverse)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    const double w = wsym(g, i, j, k);
    a[id] = inverse ? a[id] / w : a[id] * w;
}

// lu (= or +=) D^T of gm = -(rho/dt) * mask * lb, D the reference's divergence
// with one-sided differences on the boundary faces (src/pressure.cpp:14-93)
__device__ __forceinline__ double gdiv(const Geo& g, const uint8_t* solid, const double* lb, double s, int i, int id)
{
    return (solid[id] || i == g.nx - 1) ? 0.0 : s * lb[id];
}

__global__ void k_adj_div(Geo g, Dx d, double m_rho_dt, const uint8_t* __restrict__ solid,
                          const double* __restrict__ lb, double* lu, double* lv, double* lw)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    const double s = m_rho_dt;
    double au = 0.0, av = 0.0, aw = 0.0;
    // u: rows r = c-ex (c its +x neighbour), r = c+ex (c its -x neighbour), r = c
    if (i - 1 >= 0) au += gdiv(g, solid, lb, s, i - 1, id - g.si) * (i - 1 == 0 ? d.idx : d.i2dx);
    if (i + 1 <= g.nx - 1 && i + 1 != 0) au -= gdiv(g, solid, lb, s, i + 1, id + g.si) * d.i2dx;
    if (i == 0) au -= gdiv(g, solid, lb, s, i, id) * d.idx;
    // v
    if (j - 1 >= 0) av += gdiv(g, solid, lb, s, i, id - g.sj) * (j - 1 == 0 ? d.idy : d.i2dy);
    if (j + 1 <= g.ny - 1) av -= gdiv(g, solid, lb, s, i, id + g.sj) * (j + 1 == g.ny - 1 ? d.idy : d.i2dy);
    if (j == 0) av -= gdiv(g, solid, lb, s, i, id) * d.idy;
    if (j == g.ny - 1) av += gdiv(g, solid, lb, s, i, id) * d.idy;
    // w
    if (k - 1 >= 0) aw += gdiv(g, solid, lb, s, i, id - 1) * (k - 1 == 0 ? d.idz : d.i2dz);
    if (k + 1 <= g.nz - 1) aw -= gdiv(g, solid, lb, s, i, id + 1) * (k + 1 == g.nz - 1 ? d.idz : d.i2dz);
    if (k == 0) aw -= gdiv(g, solid, lb, s, i, id) * d.idz;
    if (k == g.nz - 1) aw += gdiv(g, solid, lb, s, i, id) * d.idz;
    lu[id] = au; lv[id] = av; lw[id] = aw;
}

// transpose of the momentum update (interior outputs o = f + dt(-(u.grad) f +
// (nu + nu_t) lap f), f = u, v, w): lu += M_U^T lx, lnu = dt sum_c lx_c lap f_c
__global__ void k_adj_momentum(Geo g, Dx d, double dt, double nu, const double* __restrict__ u,
                               const double* __restrict__ v, const double* __restrict__ w,
                               const double* __restrict__ nu_t, const double* __restrict__ lx,
                               const double* __restrict__ lxv, const double* __restrict__ lxw, double* lu,
                               double* lv, double* lw, double* __restrict__ lnu)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    const double* f3[3] = {u, v, w};
    const double* l3[3] = {lx, lxv, lxw};
    double* o3[3] = {lu, lv, lw};
    const double lapc = d.idx2 + d.idy2 + d.idz2;
    const bool in_c = interior(g, i, j, k);
    double adv[3] = {0.0, 0.0, 0.0};   // advecting-velocity part at c
    double ln = 0.0;
    for (int q = 0; q < 3; ++q) {
        const double* f = f3[q];
        const double* l = l3[q];
        double s = 0.0;
        // field part: outputs at c and its six neighbours n that read f[c]
        if (in_c) s += l[id] * (1.0 - 2.0 * dt * (nu + nu_t[id]) * lapc);
        if (interior(g, i - 1, j, k)) {   // c is the east neighbour of n = c-ex
            const int n = id - g.si;
            s += l[n] * dt * (-u[n] * d.i2dx + (nu + nu_t[n]) * d.idx2);
        }
        if (interior(g, i + 1, j, k)) {
            const int n = id + g.si;
            s += l[n] * dt * (u[n] * d.i2dx + (nu + nu_t[n]) * d.idx2);
        }
        if (interior(g, i, j - 1, k)) {
            const int n = id - g.sj;
            s += l[n] * dt * (-v[n] * d.i2dy + (nu + nu_t[n]) * d.idy2);
        }
        if (interior(g, i, j + 1, k)) {
            const int n = id + g.sj;
            s += l[n] * dt * (v[n] * d.i2dy + (nu + nu_t[n]) * d.idy2);
        }
        if (interior(g, i, j, k - 1)) {
            const int n = id - 1;
            s += l[n] * dt * (-w[n] * d.i2dz + (nu + nu_t[n]) * d.idz2);
        }
        if (interior(g, i, j, k + 1)) {
            const int n = id + 1;
            s += l[n] * dt * (w[n] * d.i2dz + (nu + nu_t[n]) * d.idz2);
        }
        o3[q][id] += s;
        if (in_c) {
            const double fe = f[id + g.si], fw = f[id - g.si], fn = f[id + g.sj], fs = f[id - g.sj];
            const double ft = f[id + 1], fb = f[id - 1], fc = f[id];
            const double lc = l[id];
            adv[0] += lc * (-dt) * (fe - fw) * d.i2dx;
            adv[1] += lc * (-dt) * (fn - fs) * d.i2dy;
            adv[2] += lc * (-dt) * (ft - fb) * d.i2dz;
            ln += lc * dt * ((fe - 2 * fc + fw) * d.idx2 + (fn - 2 * fc + fs) * d.idy2 + (ft - 2 * fc + fb) * d.idz2);
        }
    }
    if (in_c) {
        lu[id] += adv[0];
        lv[id] += adv[1];
        lw[id] += adv[2];
    }
    lnu[id] = ln;
}

// SGS adjoint, part 1: per interior fluid cell n, h_ab = lnu K dS/d(grad) for
// nu_t = K S (cells that the nu_t boundary values overwrite carry no
// adjoint); accumulates dJ/dCs = sum lnu * 2 K S / Cs
__global__ void k_adj_sgs_h(Geo g, Dx d, double K, double dK_dCs, const uint8_t* __restrict__ solid,
                            const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w,
                            const double* __restrict__ lnu, double* hxx, double* hyy, double* hzz, double* hxy,
                            double* hxz, double* hyz, double* partials, unsigned* counter, double* acc)
{
    __shared__ double sm[32];
    int i, j, k;
    double gc[1] = {0.0};
    if (coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        double a[6] = {0, 0, 0, 0, 0, 0};
        if (interior(g, i, j, k) && !solid[id]) {
            const int si = g.si, sj = g.sj;
            const double du_dx = (u[id + si] - u[id - si]) * d.i2dx, du_dy = (u[id + sj] - u[id - sj]) * d.i2dy;
            const double du_dz = (u[id + 1] - u[id - 1]) * d.i2dz;
            const double dv_dx = (v[id + si] - v[id - si]) * d.i2dx, dv_dy = (v[id + sj] - v[id - sj]) * d.i2dy;
            const double dv_dz = (v[id + 1] - v[id - 1]) * d.i2dz;
            const double dw_dx = (w[id + si] - w[id - si]) * d.i2dx, dw_dy = (w[id + sj] - w[id - sj]) * d.i2dy;
            const double dw_dz = (w[id + 1] - w[id - 1]) * d.i2dz;
            const double Sxx = du_dx, Syy = dv_dy, Szz = dw_dz;
            const double Sxy = 0.5 * (du_dy + dv_dx), Sxz = 0.5 * (du_dz + dw_dx), Syz = 0.5 * (dv_dz + dw_dy);
            const double S = sqrt(2.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz) + 4.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz));
            const double ln = lnu[id];
            gc[0] = ln * dK_dCs * S;
            if (S > 0.0) {
                const double c = ln * K / S;
                a[0] = 2.0 * c * Sxx; a[1] = 2.0 * c * Syy; a[2] = 2.0 * c * Szz;
                a[3] = 2.0 * c * Sxy; a[4] = 2.0 * c * Sxz; a[5] = 2.0 * c * Syz;
            }
        }
        hxx[id] = a[0]; hyy[id] = a[1]; hzz[id] = a[2]; hxy[id] = a[3]; hxz[id] = a[4]; hyz[id] = a[5];
    }
    if (last_block_sum<1>(gc, partials, counter, sm))
        if (threadIdx.x == 0 && threadIdx.y == 0) acc[1] += gc[0];
}

// SGS adjoint, part 2: gather the central differences' transposes
__global__ void k_adj_sgs_gather(Geo g, Dx d, const double* __restrict__ hxx, const double* __restrict__ hyy,
                                 const double* __restrict__ hzz, const double* __restrict__ hxy,
                                 const double* __restrict__ hxz, const double* __restrict__ hyz, double* lu,
                                 double* lv, double* lw)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    auto dx = [&](const double* h) {   // sum over n = c -+ ex of h[n] * d(central x-difference at n)/d f[c]
        double s = 0.0;
        if (i - 1 >= 0) s += h[id - g.si];
        if (i + 1 <= g.nx - 1) s -= h[id + g.si];
        return s * d.i2dx;
    };
    auto dy = [&](const double* h) {
        double s = 0.0;
        if (j - 1 >= 0) s += h[id - g.sj];
        if (j + 1 <= g.ny - 1) s -= h[id + g.sj];
        return s * d.i2dy;
    };
    auto dz = [&](const double* h) {
        double s = 0.0;
        if (k - 1 >= 0) s += h[id - 1];
        if (k + 1 <= g.nz - 1) s -= h[id + 1];
        return s * d.i2dz;
    };
    lu[id] += dx(hxx) + dy(hxy) + dz(hxz);
    lv[id] += dx(hxy) + dy(hyy) + dz(hyz);
    lw[id] += dx(hxz) + dy(hyz) + dz(hzz);
}

les_status alloc(les_ctx* c, double** p, size_t n)
{
    if (*p) return LES_OK;
    return check_cuda(c, cudaMalloc(p, sizeof(double) * n), "cudaMalloc(adjoint)");
}

les_status copy(les_ctx* c, double* dst, const double* src)
{
    return check_cuda(c, cudaMemcpyAsync(dst, src, sizeof(double) * c->g.n, cudaMemcpyDeviceToDevice, c->stream),
                      "copy");
}

les_status zero(les_ctx* c, double* a, size_t n)
{
    return check_cuda(c, cudaMemsetAsync(a, 0, sizeof(double) * n, c->stream), "memset");
}

les_status objective(les_ctx* c, AdjWork& a, int add_adjoint)
{
    const int* b = a.prm.box;
    launch(c, k_objective, cell_grid(c->g), cell_block(), c->g, b[0], b[1], b[2], b[3], b[4], b[5],
           1.0 / a.prm.steps, (const double*)c->slot[LES_U], (const double*)c->slot[LES_V],
           (const double*)c->slot[LES_W], a.lu[0], a.lu[1], a.lu[2], add_adjoint, c->partials, c->counters + 16,
           a.acc);
    return check_launch(c, "objective");
}

// ---- tangent-linear model: the forward derivative of the same step ------------
// du_in (ny*nz) / dcs are the direction; dU the tangent of the velocity.

// dnu = K dS + dK/dCs S dcs at interior fluid cells (0 where the nu_t
// boundary values overwrite it)
__global__ void k_tl_sgs(Geo g, Dx d, double K, double dK_dCs, double dcs, const uint8_t* __restrict__ solid,
                         const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w,
                         const double* __restrict__ du, const double* __restrict__ dv, const double* __restrict__ dw,
                         double* __restrict__ dnu)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    double r = 0.0;
    if (interior(g, i, j, k) && !solid[id]) {
        const int si = g.si, sj = g.sj;
        auto gx = [&](const double* f) { return (f[id + si] - f[id - si]) * d.i2dx; };
        auto gy = [&](const double* f) { return (f[id + sj] - f[id - sj]) * d.i2dy; };
        auto gz = [&](const double* f) { return (f[id + 1] - f[id - 1]) * d.i2dz; };
        const double Sxx = gx(u), Syy = gy(v), Szz = gz(w);
        const double Sxy = 0.5 * (gy(u) + gx(v)), Sxz = 0.5 * (gz(u) + gx(w)), Syz = 0.5 * (gz(v) + gy(w));
        const double S = sqrt(2.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz) + 4.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz));
        const double dSxx = gx(du), dSyy = gy(dv), dSzz = gz(dw);
        const double dSxy = 0.5 * (gy(du) + gx(dv)), dSxz = 0.5 * (gz(du) + gx(dw)), dSyz = 0.5 * (gz(dv) + gy(dw));
        const double dS = S > 0.0 ? (2.0 * (Sxx * dSxx + Syy * dSyy + Szz * dSzz) +
                                     4.0 * (Sxy * dSxy + Sxz * dSxz + Syz * dSyz)) / S
                                  : 0.0;
        r = K * dS + dK_dCs * S * dcs;
    }
    dnu[id] = r;
}

// dX1 at interior cells: the derivative of o = f + dt(-(u.grad) f + (nu + nu_t) lap f)
__global__ void k_tl_momentum(Geo g, Dx d, double dt, double nu, const double* __restrict__ u,
                              const double* __restrict__ v, const double* __restrict__ w,
                              const double* __restrict__ nu_t, const double* __restrict__ du,
                              const double* __restrict__ dv, const double* __restrict__ dw,
                              const double* __restrict__ dnu, double* __restrict__ ox, double* __restrict__ oy,
                              double* __restrict__ oz)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    double* o3[3] = {ox, oy, oz};
    if (!interior(g, i, j, k)) {
        ox[id] = oy[id] = oz[id] = 0.0;   // overwritten by the boundary conditions
        return;
    }
    const double* f3[3] = {u, v, w};
    const double* d3[3] = {du, dv, dw};
    const int si = g.si, sj = g.sj;
    const double ne = nu + nu_t[id];
    for (int q = 0; q < 3; ++q) {
        const double* f = f3[q];
        const double* df = d3[q];
        auto grad = [&](const double* a, double& gxv, double& gyv, double& gzv, double& lap) {
            const double c = a[id];
            gxv = (a[id + si] - a[id - si]) * d.i2dx;
            gyv = (a[id + sj] - a[id - sj]) * d.i2dy;
            gzv = (a[id + 1] - a[id - 1]) * d.i2dz;
            lap = (a[id + si] - 2 * c + a[id - si]) * d.idx2 + (a[id + sj] - 2 * c + a[id - sj]) * d.idy2 +
                  (a[id + 1] - 2 * c + a[id - 1]) * d.idz2;
        };
        double fx, fy, fz, fl, gx, gy, gz, gl;
        grad(f, fx, fy, fz, fl);
        grad(df, gx, gy, gz, gl);
        const double dadv = du[id] * fx + dv[id] * fy + dw[id] * fz + u[id] * gx + v[id] * gy + w[id] * gz;
        o3[q][id] = df[id] + dt * (-dadv + dnu[id] * fl + ne * gl);
    }
}

// the linearised velocity boundary conditions: the inlet takes the direction
// of the profile, walls and solids 0, the outlet copies plane nx-2
// (faces; the interior solids follow in k_tl_solids, after the outlet copy)
__global__ void k_tl_bc(Geo g, const uint8_t* __restrict__ solid, double* u, double* v, double* w,
                        const double* __restrict__ din)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (jk_in && i > 0 && i < g.nx - 1) return;
    const int id = i * g.si + j * g.sj + k;
    if (!jk_in) { u[id] = v[id] = w[id] = 0.0; return; }
    if (i == 0) {
        if (!solid[id]) { u[id] = din ? din[j * g.nz + k] : 0.0; v[id] = 0.0; w[id] = 0.0; }
        return;
    }
    const int src = id - g.si;
    u[id] = u[src]; v[id] = v[src]; w[id] = w[src];
}

__global__ void k_tl_solids(Geo g, const uint8_t* __restrict__ solid, double* u, double* v, double* w)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    if (!interior(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    if (solid[id]) u[id] = v[id] = w[id] = 0.0;
}

// db = -(rho/dt) D dU (masked like build_b)
__global__ void k_tl_div(Geo g, Dx d, double m_rho_dt, const uint8_t* __restrict__ solid, const double* __restrict__ u,
                         const double* __restrict__ v, const double* __restrict__ w, double* __restrict__ db)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    if (solid[id] || i == g.nx - 1) { db[id] = 0.0; return; }
    double a, b, c;
    if (i == 0) a = (u[id + g.si] - u[id]) * d.idx;
    else a = (u[id + g.si] - u[id - g.si]) * d.i2dx;
    if (j == 0) b = (v[id + g.sj] - v[id]) * d.idy;
    else if (j == g.ny - 1) b = (v[id] - v[id - g.sj]) * d.idy;
    else b = (v[id + g.sj] - v[id - g.sj]) * d.i2dy;
    if (k == 0) c = (w[id + 1] - w[id]) * d.idz;
    else if (k == g.nz - 1) c = (w[id] - w[id - 1]) * d.idz;
    else c = (w[id + 1] - w[id - 1]) * d.i2dz;
    db[id] = m_rho_dt * (a + b + c);
}

// dX3 = dX2 - (dt/rho) G dp at interior cells
__global__ void k_tl_correct(Geo g, Dx d, double dt_over_rho, const double* __restrict__ dp, double* u, double* v,
                             double* w)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    if (!interior(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k;
    u[id] -= dt_over_rho * ((dp[id + g.si] - dp[id - g.si]) * d.i2dx);
    v[id] -= dt_over_rho * ((dp[id + g.sj] - dp[id - g.sj]) * d.i2dy);
    w[id] -= dt_over_rho * ((dp[id + 1] - dp[id - 1]) * d.i2dz);
}

// acc[0] += scale * sum_box U . dU
__global__ void k_tl_objective(Geo g, int i0, int i1, int j0, int j1, int k0, int k1, double scale,
                               const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w,
                               const double* __restrict__ du, const double* __restrict__ dv,
                               const double* __restrict__ dw, double* partials, unsigned* counter, double* acc)
{
    __shared__ double sm[32];
    int i, j, k;
    double e[1] = {0.0};
    if (coords(g, i, j, k)) {
        const int id = i * g.si + j * g.sj + k;
        if (i >= i0 && i < i1 && j >= j0 && j < j1 && k >= k0 && k < k1)
            e[0] = u[id] * du[id] + v[id] * dv[id] + w[id] * dw[id];
    }
    if (last_block_sum<1>(e, partials, counter, sm))
        if (threadIdx.x == 0 && threadIdx.y == 0) acc[0] += scale * e[0];
}

// one forward step with the checks the gradient relies on; the physics is
// the FP64 one that the adjoint and tangent kernels differentiate
les_status fwd_step(les_ctx* c, const les_step_params* prm)
{
    les_step_stats s{};
    const int phys32 = c->phys32;
    c->phys32 = 0;
    les_status st = les_step(c, prm, &s);
    c->phys32 = phys32;
    if (st) return st;
    if (s.status != LES_OK) return fail(c, (les_status)s.status, "adjoint: a forward pressure solve did not converge");
    return LES_OK;
}

// sol = A^-1 rhs with the step's PCG to adj_rel_tol * ||rhs|| (sol holds the
// warm start on entry)
les_status solve_linear(les_ctx* c, AdjWork& a, double* rhs, double* sol, const char* what)
{
    double rr = 0.0;
    les_status st = dot_dev(c, rhs, rhs, &rr);
    if (st) return st;
    if (!(rr > 0.0)) return zero(c, sol, c->g.n);
    les_pcg_opts o = a.prm.step.pcg;
    o.tol = a.prm.adj_rel_tol * std::sqrt(rr);
    if (o.precision == LES_MIXED) {
        // an inner FP32 CG that stagnates on this non-symmetric system ends
        // after a bounded number of iterations; the FP64 outer correction
        // carries on from what it reached
        if (o.inner_max_iter <= 0) o.inner_max_iter = 400;
        if (o.max_outer < 200) o.max_outer = 200;
    }
    double* sb = c->slot[LES_B];
    double* sp = c->slot[LES_P];
    c->slot[LES_B] = rhs;
    c->slot[LES_P] = sol;
    les_pcg_result r{};
    st = o.precision == LES_MIXED ? pcg_mixed_impl(c, &o, &r, 0) : pcg_fp64(c, &o, &r, 0);
    c->slot[LES_B] = sb;
    c->slot[LES_P] = sp;
    if (st == LES_NOT_CONVERGED) return fail(c, st, std::string(what) + ": a pressure solve did not converge");
    return st;
}

// Reverses one step whose input velocity is in the velocity slots (a.lu holds
// dJ/dU' on entry and dJ/dU on return).
les_status step_adjoint(les_ctx* c, AdjWork& a)
{
    const Geo& g = c->g;
    const les_step_params& p = a.prm.step;
    const double dt = p.dt_fixed, rho = p.rho;
    const Dx d = dx_of(c->mesh);
    const dim3 gr = cell_grid(g), bl = cell_block();
    les_status st;
    // nu_t of the input velocity (with its boundary values), as the forward step had it
    if ((st = sgs_nut_dev(c, p.cs, 0))) return st;
    // U' = BC(X3): lx = BC^T lu
    launch(c, k_adj_bc, gr, bl, g, (const uint8_t*)c->mask, (const double*)a.lu[0], (const double*)a.lu[1],
           (const double*)a.lu[2], a.lx[0], a.lx[1], a.lx[2], a.grad_in);
    // X3 = X2 - (dt/rho) G p: lp = -(dt/rho) G^T lx (lx carries over to X2)
    launch(c, k_adj_correct, gr, bl, g, d, dt / rho, (const double*)a.lx[0], (const double*)a.lx[1],
           (const double*)a.lx[2], a.lp);
    // p = A^-1 b: lb = A^-T lp = W A^-1 (W^-1 lp)
    launch(c, k_scale_w, gr, bl, g, a.lp, 1);
    if ((st = check_launch(c, "adjoint correction"))) return st;
    if ((st = solve_linear(c, a, a.lp, a.lb, "adjoint"))) return st;
    // lb holds A^-1 W^-1 lp; the scaled copy goes to lp (lb stays the next warm start)
    if ((st = copy(c, a.lp, a.lb))) return st;
    launch(c, k_scale_w, gr, bl, g, a.lp, 0);
    // b = -(rho/dt) D U: lu = D^T (-(rho/dt) mask lb)
    launch(c, k_adj_div, gr, bl, g, d, -rho / dt, (const uint8_t*)c->mask, (const double*)a.lp, a.lu[0], a.lu[1],
           a.lu[2]);
    // X2 = BC(X1): lx = BC^T lx (through a copy: the transpose reads plane nx-1)
    for (int q = 0; q < 3; ++q)
        if ((st = copy(c, a.h[q], a.lx[q]))) return st;
    launch(c, k_adj_bc, gr, bl, g, (const uint8_t*)c->mask, (const double*)a.h[0], (const double*)a.h[1],
           (const double*)a.h[2], a.lx[0], a.lx[1], a.lx[2], a.grad_in);
    // X1 = M(U, nu_t)
    launch(c, k_adj_momentum, gr, bl, g, d, dt, p.nu, (const double*)c->slot[LES_U], (const double*)c->slot[LES_V],
           (const double*)c->slot[LES_W], (const double*)c->slot[LES_NU_T], (const double*)a.lx[0],
           (const double*)a.lx[1], (const double*)a.lx[2], a.lu[0], a.lu[1], a.lu[2], a.lnu);
    // nu_t = K S(U) at interior fluid cells
    const double delta = std::pow(c->mesh.dx * c->mesh.dy * c->mesh.dz, 1.0 / 3.0);
    const double K = std::pow(p.cs * delta, 2);
    launch(c, k_adj_sgs_h, gr, bl, g, d, K, 2.0 * p.cs * delta * delta, (const uint8_t*)c->mask,
           (const double*)c->slot[LES_U], (const double*)c->slot[LES_V], (const double*)c->slot[LES_W],
           (const double*)a.lnu, a.h[0], a.h[1], a.h[2], a.h[3], a.h[4], a.h[5], c->partials, c->counters + 17, a.acc);
    launch(c, k_adj_sgs_gather, gr, bl, g, d, (const double*)a.h[0], (const double*)a.h[1], (const double*)a.h[2],
           (const double*)a.h[3], (const double*)a.h[4], (const double*)a.h[5], a.lu[0], a.lu[1], a.lu[2]);
    return check_launch(c, "step adjoint");
}

}  // namespace

extern "C" {

les_status les_set_inlet(les_ctx* c, const double* u_in)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    ++c->version;
    if (!u_in) {
        cudaFree(c->inlet);
        c->inlet = nullptr;
        return LES_OK;
    }
    const size_t n = (size_t)c->g.ny * c->g.nz;
    les_status st = alloc(c, &c->inlet, n);
    if (st) return st;
    st = check_cuda(c, cudaMemcpyAsync(c->inlet, u_in, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream),
                    "upload inlet");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "upload inlet");
    return st;
}

les_status les_adjoint_forward(les_ctx* c, const les_adjoint_params* prm, double* J)
{
    if (!c || !prm || prm->steps < 1 || prm->checkpoint_every < 1) return LES_BAD_ARG;
    const les_step_params& s = prm->step;
    if (s.solver != LES_SOLVER_PCG || !(s.dt_fixed > 0) ||
        (s.pcg.precond != LES_PC_JACOBI && s.pcg.precond != LES_PC_CHEBYSHEV) || !(s.cs > 0) || c->stencil_mode != 1 ||
        !(prm->adj_rel_tol > 0))
        return fail(c, LES_BAD_ARG,
                    "adjoint: needs PCG (Jacobi or Chebyshev, FP64 or mixed) on the device-built matrix, a fixed dt, "
                    "Cs > 0 and an adjoint solve tolerance");
    cudaSetDevice(c->device);
    if (!c->adj) c->adj = new AdjWork();
    AdjWork& a = *c->adj;
    const size_t n = c->g.n;
    const int nck = (prm->steps + prm->checkpoint_every - 1) / prm->checkpoint_every;
    const int K = prm->checkpoint_every < prm->steps ? prm->checkpoint_every : prm->steps;
    les_status st;
    if ((int)a.ck.size() < 4 * nck) a.ck.resize(4 * nck, nullptr);
    for (int q = 0; q < 4 * nck; ++q)
        if ((st = alloc(c, &a.ck[q], n))) return st;
    if ((int)a.seg.size() < 3 * K) a.seg.resize(3 * K, nullptr);
    for (int q = 0; q < 3 * K; ++q)
        if ((st = alloc(c, &a.seg[q], n))) return st;
    for (int q = 0; q < 3; ++q) {
        if ((st = alloc(c, &a.lu[q], n))) return st;
        if ((st = alloc(c, &a.lx[q], n))) return st;
    }
    for (int q = 0; q < 6; ++q)
        if ((st = alloc(c, &a.h[q], n))) return st;
    if ((st = alloc(c, &a.lnu, n)) || (st = alloc(c, &a.lp, n)) || (st = alloc(c, &a.lb, n)) ||
        (st = alloc(c, &a.grad_in, (size_t)c->g.ny * c->g.nz)) || (st = alloc(c, &a.acc, 2)))
        return st;
    a.prm = *prm;
    a.nck = nck;
    a.n = n;
    a.forward_done = false;
    if ((st = zero(c, a.acc, 2))) return st;
    for (int q = 0; q < 3; ++q)
        if ((st = zero(c, a.lu[q], n))) return st;
    // U_0 = BC(initial fields): its inlet values are the control too
    if ((st = velocity_bcs_dev(c))) return st;
    for (int step = 0; step < prm->steps; ++step) {
        if (step % prm->checkpoint_every == 0) {
            const int k = step / prm->checkpoint_every;
            const int sl[4] = {LES_U, LES_V, LES_W, LES_P};
            for (int q = 0; q < 4; ++q)
                if ((st = copy(c, a.ck[4 * k + q], c->slot[sl[q]]))) return st;
        }
        if ((st = fwd_step(c, &prm->step))) return st;
        // J term of U_{step+1}; the last one also seeds the adjoint
        if ((st = objective(c, a, step == prm->steps - 1))) return st;
    }
    double h[2];
    st = check_cuda(c, cudaMemcpyAsync(h, a.acc, sizeof h, cudaMemcpyDeviceToHost, c->stream), "read J");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "read J");
    if (st) return st;
    if (J) *J = h[0];
    a.forward_done = true;
    return LES_OK;
}

les_status les_adjoint_backward(les_ctx* c, double* grad_inlet, double* grad_cs)
{
    if (!c || !c->adj || !c->adj->forward_done) return c ? fail(c, LES_BAD_ARG, "adjoint: run the forward first")
                                                         : LES_BAD_ARG;
    cudaSetDevice(c->device);
    AdjWork& a = *c->adj;
    const les_adjoint_params& prm = a.prm;
    const size_t n = a.n;
    les_status st;
    if ((st = zero(c, a.grad_in, (size_t)c->g.ny * c->g.nz)) || (st = zero(c, a.acc, 2)) || (st = zero(c, a.lb, n)))
        return st;
    const int sl[4] = {LES_U, LES_V, LES_W, LES_P};
    for (int s = a.nck - 1; s >= 0; --s) {
        const int n0 = s * prm.checkpoint_every;
        const int n1 = n0 + prm.checkpoint_every < prm.steps ? n0 + prm.checkpoint_every : prm.steps;
        // recompute the segment from its checkpoint, keeping each step's input velocity
        for (int q = 0; q < 4; ++q)
            if ((st = copy(c, c->slot[sl[q]], a.ck[4 * s + q]))) return st;
        for (int step = n0; step < n1; ++step) {
            for (int q = 0; q < 3; ++q)
                if ((st = copy(c, a.seg[3 * (step - n0) + q], c->slot[sl[q]]))) return st;
            if (step + 1 < n1 && (st = fwd_step(c, &prm.step))) return st;
        }
        // reverse it
        for (int step = n1 - 1; step >= n0; --step) {
            for (int q = 0; q < 3; ++q)
                if ((st = copy(c, c->slot[sl[q]], a.seg[3 * (step - n0) + q]))) return st;
            if ((st = step_adjoint(c, a))) return st;
            if (step >= 1 && (st = objective(c, a, 1))) return st;   // J term of U_step
        }
    }
    // U_0 = BC(initial fields): the inlet gradient of the initial state
    launch(c, k_adj_bc, cell_grid(c->g), cell_block(), c->g, (const uint8_t*)c->mask, (const double*)a.lu[0],
           (const double*)a.lu[1], (const double*)a.lu[2], a.lx[0], a.lx[1], a.lx[2], a.grad_in);
    if ((st = check_launch(c, "initial-state adjoint"))) return st;
    std::vector<double> gi((size_t)c->g.ny * c->g.nz);
    double h[2];
    st = check_cuda(c, cudaMemcpyAsync(gi.data(), a.grad_in, sizeof(double) * gi.size(), cudaMemcpyDeviceToHost,
                                       c->stream), "read gradient");
    if (!st) st = check_cuda(c, cudaMemcpyAsync(h, a.acc, sizeof h, cudaMemcpyDeviceToHost, c->stream), "read gradient");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "read gradient");
    if (st) return st;
    if (grad_inlet) std::memcpy(grad_inlet, gi.data(), sizeof(double) * gi.size());
    if (grad_cs) *grad_cs = h[1];
    return LES_OK;
}

les_status les_adjoint_tangent(les_ctx* c, const double* d_inlet, double d_cs, double* dJ)
{
    if (!c || !c->adj || !c->adj->forward_done) return c ? fail(c, LES_BAD_ARG, "tangent: run the forward first")
                                                         : LES_BAD_ARG;
    cudaSetDevice(c->device);
    AdjWork& a = *c->adj;
    const les_adjoint_params& prm = a.prm;
    const les_step_params& p = prm.step;
    const Geo& g = c->g;
    const size_t n = a.n, nin = (size_t)g.ny * g.nz;
    const Dx d = dx_of(c->mesh);
    const dim3 gr = cell_grid(g), bl = cell_block();
    les_status st;
    // tangent work: dU (a.lx), intermediate (a.h[0..2]), dnu (a.lnu), db (a.lp), dp (a.lb), direction (a.h[3])
    if ((st = zero(c, a.acc, 2)) || (st = zero(c, a.lb, n))) return st;
    for (int q = 0; q < 3; ++q)
        if ((st = zero(c, a.lx[q], n))) return st;
    double* din = a.h[3];
    if (d_inlet) {
        st = check_cuda(c, cudaMemcpyAsync(din, d_inlet, sizeof(double) * nin, cudaMemcpyHostToDevice, c->stream),
                        "tangent direction");
        if (st) return st;
    } else if ((st = zero(c, din, nin))) {
        return st;
    }
    // U_0 = BC(initial fields): dU_0 is the profile direction on the inlet
    const int sl[4] = {LES_U, LES_V, LES_W, LES_P};
    for (int q = 0; q < 4; ++q)
        if ((st = copy(c, c->slot[sl[q]], a.ck[q]))) return st;
    launch(c, k_tl_bc, gr, bl, g, (const uint8_t*)c->mask, a.lx[0], a.lx[1], a.lx[2], (const double*)din);
    launch(c, k_tl_solids, gr, bl, g, (const uint8_t*)c->mask, a.lx[0], a.lx[1], a.lx[2]);
    const double delta = std::pow(c->mesh.dx * c->mesh.dy * c->mesh.dz, 1.0 / 3.0);
    const double K = std::pow(p.cs * delta, 2);
    for (int step = 0; step < prm.steps; ++step) {
        if ((st = sgs_nut_dev(c, p.cs, 0))) return st;
        launch(c, k_tl_sgs, gr, bl, g, d, K, 2.0 * p.cs * delta * delta, d_cs, (const uint8_t*)c->mask,
               (const double*)c->slot[LES_U], (const double*)c->slot[LES_V], (const double*)c->slot[LES_W],
               (const double*)a.lx[0], (const double*)a.lx[1], (const double*)a.lx[2], a.lnu);
        launch(c, k_tl_momentum, gr, bl, g, d, p.dt_fixed, p.nu, (const double*)c->slot[LES_U],
               (const double*)c->slot[LES_V], (const double*)c->slot[LES_W], (const double*)c->slot[LES_NU_T],
               (const double*)a.lx[0], (const double*)a.lx[1], (const double*)a.lx[2], (const double*)a.lnu, a.h[0],
               a.h[1], a.h[2]);
        launch(c, k_tl_bc, gr, bl, g, (const uint8_t*)c->mask, a.h[0], a.h[1], a.h[2], (const double*)din);
        launch(c, k_tl_solids, gr, bl, g, (const uint8_t*)c->mask, a.h[0], a.h[1], a.h[2]);
        launch(c, k_tl_div, gr, bl, g, d, -p.rho / p.dt_fixed, (const uint8_t*)c->mask, (const double*)a.lx[0],
               (const double*)a.lx[1], (const double*)a.lx[2], a.lp);
        if ((st = check_launch(c, "tangent step"))) return st;
        if ((st = solve_linear(c, a, a.lp, a.lb, "tangent"))) return st;
        launch(c, k_tl_correct, gr, bl, g, d, p.dt_fixed / p.rho, (const double*)a.lb, a.h[0], a.h[1], a.h[2]);
        launch(c, k_tl_bc, gr, bl, g, (const uint8_t*)c->mask, a.h[0], a.h[1], a.h[2], (const double*)din);
        launch(c, k_tl_solids, gr, bl, g, (const uint8_t*)c->mask, a.h[0], a.h[1], a.h[2]);
        for (int q = 0; q < 3; ++q)
            if ((st = copy(c, a.lx[q], a.h[q]))) return st;
        // the forward step itself (from the same U_n), then the J term of U_{n+1}
        if ((st = fwd_step(c, &p))) return st;
        const int* b = prm.box;
        launch(c, k_tl_objective, gr, bl, g, b[0], b[1], b[2], b[3], b[4], b[5], 1.0 / prm.steps,
               (const double*)c->slot[LES_U], (const double*)c->slot[LES_V], (const double*)c->slot[LES_W],
               (const double*)a.lx[0], (const double*)a.lx[1], (const double*)a.lx[2], c->partials, c->counters + 18,
               a.acc);
        if ((st = check_launch(c, "tangent objective"))) return st;
    }
    double h[2];
    st = check_cuda(c, cudaMemcpyAsync(h, a.acc, sizeof h, cudaMemcpyDeviceToHost, c->stream), "read dJ");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "read dJ");
    if (st) return st;
    if (dJ) *dJ = h[0];
    return LES_OK;
}

}  // extern "C"
