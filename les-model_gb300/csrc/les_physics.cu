// les_physics.cu -- step physics of les-model src/main.cpp on the device.
//
// Every kernel keeps the reference's floating-point operation order (this
// translation unit is compiled with -fmad=false, so a*b+c is a rounded
// multiply followed by a rounded add, as in the reference's x86-64 build),
// so the results are bit-identical to the reference on the same inputs.
//
// Boundary conditions are written as closed forms of the pre-BC field instead
// of the reference's sequence of face loops; the closed forms give the same
// final values (each is derived in the comment of its kernel).
#include "les_internal.cuh"

using namespace les;

namespace {

struct StepConst {
    double inv_dx2, inv_dy2, inv_dz2, inv_2dx, inv_2dy, inv_2dz;
    double two_dx, two_dy, two_dz;
};

StepConst step_const(const les_mesh& m)
{
    StepConst s;
    s.inv_dx2 = 1.0 / (m.dx * m.dx);
    s.inv_dy2 = 1.0 / (m.dy * m.dy);
    s.inv_dz2 = 1.0 / (m.dz * m.dz);
    s.inv_2dx = 1.0 / (2.0 * m.dx);
    s.inv_2dy = 1.0 / (2.0 * m.dy);
    s.inv_2dz = 1.0 / (2.0 * m.dz);
    s.two_dx = 2 * m.dx;
    s.two_dy = 2 * m.dy;
    s.two_dz = 2 * m.dz;
    return s;
}

struct Sgs {
    double nut, Sxx, Syy, Szz, Sxy, Sxz, Syz;
};

// compute_sgs_stress body, src/main.cpp:436-461.
__device__ __forceinline__ Sgs sgs_cell(const double* __restrict__ u, const double* __restrict__ v,
                                        const double* __restrict__ w, int id, const Geo& g,
                                        const StepConst& s, double cs2)
{
    const int si = g.si, sj = g.sj;
    double du_dx = (u[id + si] - u[id - si]) / s.two_dx;
    double du_dy = (u[id + sj] - u[id - sj]) / s.two_dy;
    double du_dz = (u[id + 1] - u[id - 1]) / s.two_dz;
    double dv_dx = (v[id + si] - v[id - si]) / s.two_dx;
    double dv_dy = (v[id + sj] - v[id - sj]) / s.two_dy;
    double dv_dz = (v[id + 1] - v[id - 1]) / s.two_dz;
    double dw_dx = (w[id + si] - w[id - si]) / s.two_dx;
    double dw_dy = (w[id + sj] - w[id - sj]) / s.two_dy;
    double dw_dz = (w[id + 1] - w[id - 1]) / s.two_dz;
    Sgs r;
    r.Sxx = du_dx; r.Syy = dv_dy; r.Szz = dw_dz;
    r.Sxy = 0.5 * (du_dy + dv_dx);
    r.Sxz = 0.5 * (du_dz + dw_dx);
    r.Syz = 0.5 * (dv_dz + dw_dy);
    double smag = sqrt(2.0 * (r.Sxx * r.Sxx + r.Syy * r.Syy + r.Szz * r.Szz) +
                       4.0 * (r.Sxy * r.Sxy + r.Sxz * r.Sxz + r.Syz * r.Syz));
    r.nut = cs2 * smag;
    return r;
}

__device__ __forceinline__ void store_tau(double* tau, int n, int id, const Sgs& r)
{
    tau[0 * (size_t)n + id] = -2.0 * r.nut * r.Sxx;
    tau[1 * (size_t)n + id] = -2.0 * r.nut * r.Sxy;
    tau[2 * (size_t)n + id] = -2.0 * r.nut * r.Sxz;
    tau[3 * (size_t)n + id] = -2.0 * r.nut * r.Syy;
    tau[4 * (size_t)n + id] = -2.0 * r.nut * r.Syz;
    tau[5 * (size_t)n + id] = -2.0 * r.nut * r.Szz;
}

__device__ __forceinline__ bool cell_coords(const Geo& g, int& i, int& j, int& k)
{
    k = blockIdx.x * TBK + threadIdx.x;
    j = blockIdx.y * TBJ + threadIdx.y;
    i = blockIdx.z;
    return k < g.nz && j < g.ny;
}

// compute_sgs_stress alone (interior cells), src/main.cpp:423-472.
__global__ void k_sgs(Geo g, StepConst s, double cs2, const double* __restrict__ u,
                      const double* __restrict__ v, const double* __restrict__ w,
                      double* __restrict__ nu_t, double* __restrict__ tau)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 1 || k > g.nz - 2) return;
    int id = i * g.si + j * g.sj + k;
    Sgs r = sgs_cell(u, v, w, id, g, s, cs2);
    nu_t[id] = r.nut;
    if (tau) store_tau(tau, g.n, id, r);
}

// compute_sgs_stress followed by apply_nut_BCs (src/main.cpp:483-547), one
// pass over all cells.  Final nu_t of the reference sequence:
//   j or k on a wall, or i == 0          -> 0
//   i == nx-1 (j, k interior)            -> raw nu_t of (nx-2, j, k), copied
//                                           before the obstacle is zeroed
//   interior                             -> solid ? 0 : raw nu_t
__global__ void k_sgs_nut(Geo g, StepConst s, double cs2, const double* __restrict__ u,
                          const double* __restrict__ v, const double* __restrict__ w,
                          const uint8_t* __restrict__ solid, double* __restrict__ nu_t,
                          double* __restrict__ tau)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    int id = i * g.si + j * g.sj + k;
    bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (!jk_in || i == 0) { nu_t[id] = 0.0; return; }
    if (i == g.nx - 1) return;  // written by the (nx-2, j, k) thread
    Sgs r = sgs_cell(u, v, w, id, g, s, cs2);
    if (tau) store_tau(tau, g.n, id, r);
    nu_t[id] = solid[id] ? 0.0 : r.nut;
    if (i == g.nx - 2) nu_t[id + g.si] = r.nut;
}

// Face part of apply_nut_BCs alone.  Threads cover the whole grid; only face
// cells act (the interior obstacle pass runs after it).
__global__ void k_nut_faces(Geo g, double* __restrict__ nu_t)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    int id = i * g.si + j * g.sj + k;
    bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (!jk_in || i == 0) { nu_t[id] = 0.0; return; }
    if (i == g.nx - 1) nu_t[id] = nu_t[id - g.si];
}

__global__ void k_zero_list3(const int* __restrict__ list, int n, double* a, double* b, double* c)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int id = list[t];
    a[id] = 0.0;
    if (b) b[id] = 0.0;
    if (c) c[id] = 0.0;
}

// apply_velocity_BCs, src/main.cpp:323-410, face part.  Final values of the
// reference's ordered face loops:
//   j or k on a wall                    -> 0 (y/z walls run after inlet/outlet)
//   i == 0 (j, k interior)              -> solid ? unchanged : (1, 0, 0)
//   i == nx-1 (j, k interior)           -> value of (nx-2, j, k) before the
//                                          obstacle overwrite
// The interior obstacle overwrite (:395-409) runs afterwards (k_zero_list3).
// inlet != nullptr: the inlet u is the per-(j,k) profile inlet[j*nz+k]
// (the adjoint's control) instead of the reference's uniform 1.
__global__ void k_velocity_faces(Geo g, const uint8_t* __restrict__ solid, double* __restrict__ u,
                                 double* __restrict__ v, double* __restrict__ w, const double* __restrict__ inlet)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (jk_in && i > 0 && i < g.nx - 1) return;
    int id = i * g.si + j * g.sj + k;
    if (!jk_in) { u[id] = 0.0; v[id] = 0.0; w[id] = 0.0; return; }
    if (i == 0) {
        if (!solid[id]) { u[id] = inlet ? inlet[j * g.nz + k] : 1.0; v[id] = 0.0; w[id] = 0.0; }
        return;
    }
    int src = id - g.si;
    u[id] = u[src]; v[id] = v[src]; w[id] = w[src];
}

// solve_momentum, src/main.cpp:563-654 (interior; the swap of :656-658 is a
// pointer swap on the host).  One thread updates all three components.
// dtp != nullptr: dt is read from device memory (a graph-captured step whose
// dt comes from compute_adaptive_dt on the device).
__global__ void k_momentum(Geo g, StepConst s, double dt, double nu, const double* __restrict__ u,
                           const double* __restrict__ v, const double* __restrict__ w,
                           const double* __restrict__ nu_t, double* __restrict__ un,
                           double* __restrict__ vn, double* __restrict__ wn, const double* dtp)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    if (dtp) dt = *dtp;
    if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 1 || k > g.nz - 2) return;
    const int id = i * g.si + j * g.sj + k, si = g.si, sj = g.sj;
    const double nu_eff = nu + nu_t[id];
    const double uc = u[id], vc = v[id], wc = w[id];
    const double* f3[3] = {u, v, w};
    double* o3[3] = {un, vn, wn};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double* f = f3[q];
        double fe = f[id + si], fw = f[id - si], fn = f[id + sj], fs = f[id - sj];
        double ft = f[id + 1], fb = f[id - 1], fc = f[id];
        double d_dx = (fe - fw) * s.inv_2dx;
        double d_dy = (fn - fs) * s.inv_2dy;
        double d_dz = (ft - fb) * s.inv_2dz;
        double adv = uc * d_dx + vc * d_dy + wc * d_dz;
        double lap = (fe - 2 * fc + fw) * s.inv_dx2 + (fn - 2 * fc + fs) * s.inv_dy2 +
                     (ft - 2 * fc + fb) * s.inv_dz2;
        o3[q][id] = fc + dt * (-adv + nu_eff * lap);
    }
}

// correct_velocity, src/main.cpp:671-714 (interior).
__global__ void k_correct(Geo g, StepConst s, double dt_over_rho, const double* __restrict__ p,
                          double* __restrict__ u, double* __restrict__ v, double* __restrict__ w,
                          const double* dtp, double rho)
{
    int i, j, k;
    if (!cell_coords(g, i, j, k)) return;
    if (dtp) dt_over_rho = *dtp / rho;   // src/main.cpp:677, from the device dt
    if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 1 || k > g.nz - 2) return;
    const int id = i * g.si + j * g.sj + k;
    u[id] -= dt_over_rho * ((p[id + g.si] - p[id - g.si]) * s.inv_2dx);
    v[id] -= dt_over_rho * ((p[id + g.sj] - p[id - g.sj]) * s.inv_2dy);
    w[id] -= dt_over_rho * ((p[id + 1] - p[id - 1]) * s.inv_2dz);
}

// Running maximum of non-negative doubles as unsigned integers: for such
// values the order of the bit patterns is the order of the numbers, and the
// integer pipe is far faster than GB300's FP64 one.  What the reference's
// `(m < x) ? x : m` never selects from a start of 0 -- NaN and negative
// values -- maps to 0 (+0.0).
__device__ __forceinline__ unsigned long long max_key(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b > 0x7ff0000000000000ull ? 0ull : b;   // sign bit set or NaN
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    return v;
}

// compute_adaptive_dt, src/main.cpp:208-250: max |u|^2 and max nu_t over
// all cells (max is exact, so the reduction order does not matter), then the
// final formula in the last block.
__global__ void k_dt(Geo g, const double* __restrict__ u, const double* __restrict__ v,
                     const double* __restrict__ w, const double* __restrict__ nu_t,
                     double* partials, unsigned* counter, SolverState* st, double nu,
                     double cfl_conv, double cfl_visc, double dt_max, double min_dx)
{
    __shared__ unsigned long long sm[2][32];
    __shared__ int am_last;
    int i, j, k;
    unsigned long long m2 = 0ull, mt = 0ull;
    if (cell_coords(g, i, j, k)) {
        int id = i * g.si + j * g.sj + k;
        double mag = u[id] * u[id] + v[id] * v[id] + w[id] * w[id];
        m2 = max_key(mag);
        mt = max_key(nu_t[id]);
    }
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, lane = tid & 31, warp = tid >> 5;
    m2 = warp_max_u64(m2);
    mt = warp_max_u64(mt);
    if (lane == 0) { sm[0][warp] = m2; sm[1][warp] = mt; }
    __syncthreads();
    const int nw = (blockDim.x * blockDim.y) >> 5, nb = block_count(), bid = block_linear_id();
    unsigned long long* pk = reinterpret_cast<unsigned long long*>(partials);
    if (tid == 0) {
        unsigned long long a = 0ull, b = 0ull;
        for (int q = 0; q < nw; ++q) { a = sm[0][q] > a ? sm[0][q] : a; b = sm[1][q] > b ? sm[1][q] : b; }
        pk[bid] = a;
        pk[nb + bid] = b;
        __threadfence();
        am_last = atomicAdd(counter, 1u) == (unsigned)nb - 1u;
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    unsigned long long a = 0ull, b = 0ull;
    for (int q = tid; q < nb; q += blockDim.x * blockDim.y) {
        const unsigned long long pa = __ldcg(pk + q), pb = __ldcg(pk + nb + q);
        a = pa > a ? pa : a;
        b = pb > b ? pb : b;
    }
    a = warp_max_u64(a);
    b = warp_max_u64(b);
    __syncthreads();
    if (lane == 0) { sm[0][warp] = a; sm[1][warp] = b; }
    __syncthreads();
    if (tid == 0) {
        unsigned long long ka = 0ull, kb = 0ull;
        for (int q = 0; q < nw; ++q) { ka = sm[0][q] > ka ? sm[0][q] : ka; kb = sm[1][q] > kb ? sm[1][q] : kb; }
        const double u_max_sq = __longlong_as_double((long long)ka), nu_t_max = __longlong_as_double((long long)kb);
        double u_max = sqrt(u_max_sq);
        double dt_conv = 1.7976931348623157e308;
        if (u_max > 1e-12) dt_conv = cfl_conv * min_dx / u_max;
        double dt_visc = cfl_visc * (min_dx * min_dx) / (nu + nu_t_max);
        double r = dt_conv;
        if (dt_visc < r) r = dt_visc;
        if (dt_max < r) r = dt_max;
        st->scal[0] = r;
        st->scal[1] = u_max_sq;
        st->scal[2] = nu_t_max;
        *counter = 0u;
    }
}

}  // namespace

namespace les {

les_status velocity_bcs_dev(les_ctx* c)
{
    const Geo& g = c->g;
    launch(c, k_velocity_faces, cell_grid(g), cell_block(), g, c->mask, c->slot[LES_U], c->slot[LES_V],
           c->slot[LES_W], (const double*)c->inlet);
    if (c->n_solid)
        launch(c, k_zero_list3, (c->n_solid + 255) / 256, 256, 
            c->solid_list, c->n_solid, c->slot[LES_U], c->slot[LES_V], c->slot[LES_W]);
    return check_launch(c, "velocity bcs");
}

les_status sgs_nut_dev(les_ctx* c, double cs, int want_tau)
{
    const Geo& g = c->g;
    if (want_tau && !c->tau) {
        les_status st = check_cuda(c, cudaMalloc(&c->tau, sizeof(double) * 6 * (size_t)g.n), "cudaMalloc(tau)");
        if (st) return st;
        cudaMemsetAsync(c->tau, 0, sizeof(double) * 6 * (size_t)g.n, c->stream);
    }
    // pow(Cs*delta, 2) with delta = pow(dx*dy*dz, 1/3), on the host exactly as
    // src/main.cpp:426 and :461 compute it
    double delta = std::pow(c->mesh.dx * c->mesh.dy * c->mesh.dz, 1.0 / 3.0);
    double cs2 = std::pow(cs * delta, 2);
    launch(c, k_sgs_nut, cell_grid(g), cell_block(), 
        g, step_const(c->mesh), cs2, c->slot[LES_U], c->slot[LES_V], c->slot[LES_W], c->mask,
        c->slot[LES_NU_T], want_tau ? c->tau : nullptr);
    return check_launch(c, "sgs+nut");
}

les_status momentum_dev(les_ctx* c, double dt, double nu, const double* dtp)
{
    const Geo& g = c->g;
    launch(c, k_momentum, cell_grid(g), cell_block(),
        g, step_const(c->mesh), dt, nu, c->slot[LES_U], c->slot[LES_V], c->slot[LES_W],
        c->slot[LES_NU_T], c->slot[LES_U_NEW], c->slot[LES_V_NEW], c->slot[LES_W_NEW], dtp);
    std::swap(c->slot[LES_U], c->slot[LES_U_NEW]);
    std::swap(c->slot[LES_V], c->slot[LES_V_NEW]);
    std::swap(c->slot[LES_W], c->slot[LES_W_NEW]);
    return check_launch(c, "momentum");
}

les_status correct_dev(les_ctx* c, double dt, double rho, const double* dtp)
{
    const Geo& g = c->g;
    launch(c, k_correct, cell_grid(g), cell_block(), g, step_const(c->mesh), dt / rho,
                                                             c->slot[LES_P], c->slot[LES_U],
                                                             c->slot[LES_V], c->slot[LES_W], dtp, rho);
    return check_launch(c, "correct velocity");
}

les_status adaptive_dt_dev(les_ctx* c, double nu, double cfl_conv, double cfl_visc, double dt_max)
{
    const Geo& g = c->g;
    double min_dx = c->mesh.dx;
    if (c->mesh.dy < min_dx) min_dx = c->mesh.dy;
    if (c->mesh.dz < min_dx) min_dx = c->mesh.dz;
    launch(c, k_dt, cell_grid(g), cell_block(), 
        g, c->slot[LES_U], c->slot[LES_V], c->slot[LES_W], c->slot[LES_NU_T], c->partials,
        c->counters + 0, c->state, nu, cfl_conv, cfl_visc, dt_max, min_dx);
    return check_launch(c, "adaptive dt");
}

}  // namespace les

extern "C" {

les_status les_adaptive_dt(les_ctx* c, double nu, double cfl_conv, double cfl_visc, double dt_max,
                           double* dt)
{
    if (!c || !dt) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    les_status st = adaptive_dt_dev(c, nu, cfl_conv, cfl_visc, dt_max);
    if (st) return st;
    st = read_state(c);
    if (st) return st;
    *dt = c->h_state->scal[0];
    return LES_OK;
}

les_status les_velocity_bcs(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return velocity_bcs_dev(c);
}

les_status les_sgs(les_ctx* c, double cs, int want_tau)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    const Geo& g = c->g;
    if (want_tau && !c->tau) {
        les_status st = check_cuda(c, cudaMalloc(&c->tau, sizeof(double) * 6 * (size_t)g.n), "cudaMalloc(tau)");
        if (st) return st;
        cudaMemsetAsync(c->tau, 0, sizeof(double) * 6 * (size_t)g.n, c->stream);
    }
    double delta = std::pow(c->mesh.dx * c->mesh.dy * c->mesh.dz, 1.0 / 3.0);
    double cs2 = std::pow(cs * delta, 2);
    launch(c, k_sgs, cell_grid(g), cell_block(), g, step_const(c->mesh), cs2, c->slot[LES_U],
                                                         c->slot[LES_V], c->slot[LES_W],
                                                         c->slot[LES_NU_T], want_tau ? c->tau : nullptr);
    return check_launch(c, "sgs");
}

les_status les_nut_bcs(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    const Geo& g = c->g;
    launch(c, k_nut_faces, cell_grid(g), cell_block(), g, c->slot[LES_NU_T]);
    if (c->n_solid)
        launch(c, k_zero_list3, (c->n_solid + 255) / 256, 256, c->solid_list, c->n_solid,
                                                                        c->slot[LES_NU_T], nullptr, nullptr);
    return check_launch(c, "nut bcs");
}

les_status les_sgs_nut(les_ctx* c, double cs, int want_tau)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return sgs_nut_dev(c, cs, want_tau);
}

les_status les_momentum(les_ctx* c, double dt, double nu)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return momentum_dev(c, dt, nu, nullptr);
}

les_status les_correct_velocity(les_ctx* c, double dt, double rho)
{
    if (!c) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return correct_dev(c, dt, rho, nullptr);
}

}  // extern "C"
