// les_physics32.cu -- the step physics of the mixed-precision path in FP32:
// Smagorinsky nu_t (with its boundary values) and the explicit momentum
// update of les-model src/main.cpp:423-547 and :563-654, computed in FP32 on
// the FP64 fields.
//
// The fields stay FP64 in memory (the reference's Field storage); each
// kernel converts what it loads to FP32 and computes the strain rates,
// advection and diffusion in FP32.  The momentum update adds the FP32
// increment dt * (-adv + nu_eff lap) to the FP64 velocity in FP64, so the
// velocity itself keeps its FP64 precision from step to step.  The kernels
// read and write the same bytes as the FP64 ones (nu_t: 33 B/cell, momentum:
// 56 B/cell) and are bound by HBM; the FP64 kernels are bound by GB300's FP64
// pipe (about 2 operations per SM and clock).  For the same reason the
// conversions are integer operations on the IEEE 754 bit patterns
// (les_bits.cuh) rather than conversion instructions.
//
// Reference operation order is not kept here (the FP64 kernels in
// les_physics.cu keep it): divisions by 2 dx are multiplications by the FP32
// reciprocal and the compiler may contract products into FMAs.
#include <cmath>
#include <utility>

#include "les_bits.cuh"
#include "les_internal.cuh"

using namespace les;

namespace {

struct Inv32 {
    float i2x, i2y, i2z;     // 1 / (2 dx) ...
    float ix2, iy2, iz2;     // 1 / dx^2 ...
};

Inv32 inv32(const les_mesh& m)
{
    Inv32 s;
    s.i2x = (float)(1.0 / (2.0 * m.dx));
    s.i2y = (float)(1.0 / (2.0 * m.dy));
    s.i2z = (float)(1.0 / (2.0 * m.dz));
    s.ix2 = (float)(1.0 / (m.dx * m.dx));
    s.iy2 = (float)(1.0 / (m.dy * m.dy));
    s.iz2 = (float)(1.0 / (m.dz * m.dz));
    return s;
}

__device__ __forceinline__ bool coords(const Geo& g, int& i, int& j, int& k)
{
    k = blockIdx.x * TBK + threadIdx.x;
    j = blockIdx.y * TBJ + threadIdx.y;
    i = blockIdx.z;
    return k < g.nz && j < g.ny;
}

__device__ __forceinline__ float ld32(const double* __restrict__ p, int id) { return d2f_bits(p[id]); }

// compute_sgs_stress + apply_nut_BCs (src/main.cpp:436-461, :483-547) in FP32,
// with the final values of the FP64 kernel k_sgs_nut:
//   j or k on a wall, or i == 0          -> 0
//   i == nx-1 (j, k interior)            -> nu_t of (nx-2, j, k) before the
//                                           obstacle is zeroed
//   interior                             -> solid ? 0 : nu_t
__global__ void k_sgs_nut32(Geo g, Inv32 s, float cs2, const double* __restrict__ u, const double* __restrict__ v,
                            const double* __restrict__ w, const uint8_t* __restrict__ solid,
                            double* __restrict__ nu_t)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    const int id = i * g.si + j * g.sj + k, si = g.si, sj = g.sj;
    const bool jk_in = j >= 1 && j <= g.ny - 2 && k >= 1 && k <= g.nz - 2;
    if (!jk_in || i == 0) { nu_t[id] = 0.0; return; }
    if (i == g.nx - 1) return;   // written by the (nx-2, j, k) thread
    const float du_dx = (ld32(u, id + si) - ld32(u, id - si)) * s.i2x;
    const float du_dy = (ld32(u, id + sj) - ld32(u, id - sj)) * s.i2y;
    const float du_dz = (ld32(u, id + 1) - ld32(u, id - 1)) * s.i2z;
    const float dv_dx = (ld32(v, id + si) - ld32(v, id - si)) * s.i2x;
    const float dv_dy = (ld32(v, id + sj) - ld32(v, id - sj)) * s.i2y;
    const float dv_dz = (ld32(v, id + 1) - ld32(v, id - 1)) * s.i2z;
    const float dw_dx = (ld32(w, id + si) - ld32(w, id - si)) * s.i2x;
    const float dw_dy = (ld32(w, id + sj) - ld32(w, id - sj)) * s.i2y;
    const float dw_dz = (ld32(w, id + 1) - ld32(w, id - 1)) * s.i2z;
    const float sxy = 0.5f * (du_dy + dv_dx), sxz = 0.5f * (du_dz + dw_dx), syz = 0.5f * (dv_dz + dw_dy);
    const float smag = sqrtf(2.f * (du_dx * du_dx + dv_dy * dv_dy + dw_dz * dw_dz) +
                             4.f * (sxy * sxy + sxz * sxz + syz * syz));
    const double nut = f2d_bits(cs2 * smag);
    nu_t[id] = solid[id] ? 0.0 : nut;
    if (i == g.nx - 2) nu_t[id + si] = nut;
}

// solve_momentum (src/main.cpp:563-654) for the interior cells: FP32
// advection and diffusion, the increment added in FP64.  dtp != nullptr: dt
// is read from device memory (the CFL reduction of a graph-captured step).
__global__ void k_momentum32(Geo g, Inv32 s, double dt, float nu, const double* __restrict__ u,
                             const double* __restrict__ v, const double* __restrict__ w,
                             const double* __restrict__ nu_t, double* __restrict__ un, double* __restrict__ vn,
                             double* __restrict__ wn, const double* dtp)
{
    int i, j, k;
    if (!coords(g, i, j, k)) return;
    if (dtp) dt = *dtp;
    if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 1 || k > g.nz - 2) return;
    const int id = i * g.si + j * g.sj + k, si = g.si, sj = g.sj;
    const float dtf = d2f_bits(dt);
    const float nu_eff = nu + ld32(nu_t, id);
    const double c3[3] = {u[id], v[id], w[id]};
    const float uc = d2f_bits(c3[0]), vc = d2f_bits(c3[1]), wc = d2f_bits(c3[2]);
    const double* f3[3] = {u, v, w};
    double* o3[3] = {un, vn, wn};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double* f = f3[q];
        const float fe = ld32(f, id + si), fw = ld32(f, id - si), fn = ld32(f, id + sj), fs = ld32(f, id - sj);
        const float ft = ld32(f, id + 1), fb = ld32(f, id - 1), fc = d2f_bits(c3[q]);
        const float adv = uc * ((fe - fw) * s.i2x) + vc * ((fn - fs) * s.i2y) + wc * ((ft - fb) * s.i2z);
        const float lap = (fe - 2.f * fc + fw) * s.ix2 + (fn - 2.f * fc + fs) * s.iy2 + (ft - 2.f * fc + fb) * s.iz2;
        o3[q][id] = c3[q] + f2d_bits(dtf * (nu_eff * lap - adv));
    }
}

}  // namespace

namespace les {

les_status sgs_nut32_dev(les_ctx* c, double cs)
{
    const Geo& g = c->g;
    // (Cs delta)^2 with delta = (dx dy dz)^(1/3), as src/main.cpp:426 and :461
    const double delta = std::pow(c->mesh.dx * c->mesh.dy * c->mesh.dz, 1.0 / 3.0);
    const float cs2 = (float)std::pow(cs * delta, 2);
    launch(c, k_sgs_nut32, cell_grid(g), cell_block(), g, inv32(c->mesh), cs2, (const double*)c->slot[LES_U],
           (const double*)c->slot[LES_V], (const double*)c->slot[LES_W], (const uint8_t*)c->mask,
           c->slot[LES_NU_T]);
    return check_launch(c, "sgs+nut (FP32)");
}

les_status momentum32_dev(les_ctx* c, double dt, double nu, const double* dtp)
{
    const Geo& g = c->g;
    launch(c, k_momentum32, cell_grid(g), cell_block(), g, inv32(c->mesh), dt, (float)nu,
           (const double*)c->slot[LES_U], (const double*)c->slot[LES_V], (const double*)c->slot[LES_W],
           (const double*)c->slot[LES_NU_T], c->slot[LES_U_NEW], c->slot[LES_V_NEW], c->slot[LES_W_NEW], dtp);
    std::swap(c->slot[LES_U], c->slot[LES_U_NEW]);
    std::swap(c->slot[LES_V], c->slot[LES_V_NEW]);
    std::swap(c->slot[LES_W], c->slot[LES_W_NEW]);
    return check_launch(c, "momentum (FP32)");
}

}  // namespace les
