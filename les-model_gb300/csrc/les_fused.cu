// les_fused.cu -- the FP32 inner PCG iteration of the mixed-precision solve in
// two fused passes over the grid (Jacobi or Chebyshev preconditioner).
//
// Pass A (k_pass_a): p = z + beta p_old, q = A p, p.q -> alpha.
// Pass B (k_pass_b): r' = r - alpha q, e' = e + alpha p, ||r'||^2, then the
//   whole preconditioner z = M^-1 r' (Chebyshev: S = degree-1 stencil levels,
//   the recurrence of les-model src/pressure.cpp:871-905; Jacobi: r'/A_c),
//   and r'.z -> beta, rho.  Convergence is tested on ||r'||.
//
// Both passes march along i (the slowest axis) over a tile of rows (j) and
// columns (k) and a chunk of planes.  Shared-memory rows are exactly 32 cells
// wide, one warp per row, so the tile's output width in k is 32 minus the
// halo: 30 for pass A (halo 1), 32-2S for pass B (halo S).  Pass A keeps a
// ring of three planes of p.  Pass B is temporally blocked: at march step I it
// computes level 0 (r') at plane I and Chebyshev level k at plane I-k, each
// level over the tile grown by S-k halo cells, from rings of planes of the
// level below (and of the stencil codes) held in shared memory; only r, q, p,
// e and the codes are read and r', e', z written, once per cell: 17 + 29 bytes
// per cell per inner iteration instead of 104 for five unfused kernels.
//
// Inner products are accumulated per thread in compensated FP32 (TwoProd +
// TwoSum, i.e. double-float, ~48-bit significand) and summed across threads
// and blocks in FP64; GB300's FP64 pipe is ~70x slower than its FP32 pipe, so
// a per-cell FP64 add tree would dominate these memory-bound kernels.
#include <cmath>
#include <type_traits>

#include "les_internal.cuh"
#include "les_mixed.cuh"
#include "les_tma.cuh"

using namespace les;

namespace {

constexpr int NT = 256;   // 8 warps
constexpr int NW = NT / 32;
constexpr int W = 32;     // shared-memory row width

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }

// The 7-point product at a cell next to a wall, the outlet or a solid (any
// stencil code but 1): decoded coefficients and the reference's bounds tests
// (src/pressure.cpp:735-742), on shared-memory planes whose rows are W wide.
// Rare, so kept out of line.
__device__ __noinline__ float az_general(const ViewF A, int id, int Pk, int j, int kg, const Geo g, const float* zc,
                                         const float* zw, const float* ze, int pt)
{
    CoefF a = A.at(id);
    float az = a.c * zc[pt];
    if (Pk > 0) az += a.w * zw[pt];
    if (Pk < g.nx - 1) az += a.e * ze[pt];
    if (j > 0) az += a.s * zc[pt - W];
    if (j < g.ny - 1) az += a.n * zc[pt + W];
    if (kg > 0) az += a.b * zc[pt - 1];
    if (kg < g.nz - 1) az += a.t * zc[pt + 1];
    return az;
}

// ---- pass A -----------------------------------------------------------------
constexpr int A_TK = W - 2;       // 30 output columns
constexpr int A_TJ = 14;          // output rows
constexpr int A_H = A_TJ + 2;     // 16 rows with halo = 2 per warp
constexpr int A_PL = W * A_H;

template <bool FIRST>
__global__ void __launch_bounds__(NT, 6) k_pass_a(Geo g, ViewF A, int CI, const float* __restrict__ z,
                                                const float* __restrict__ pold, float* __restrict__ pnew,
                                                float* __restrict__ q, double* partials, unsigned* counter,
                                                SolverState* st)
{
    __shared__ float sp[3][A_PL];
    __shared__ double sm[32];
    if (st->done) return;
    const float beta = FIRST ? 0.f : (float)st->beta;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k0 = blockIdx.x * A_TK, j0 = blockIdx.y * A_TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    const int kg = k0 - 1 + lane;
    const bool kin = kg >= 0 && kg < g.nz;
    const bool kcen = lane >= 1 && lane <= A_TK && kg < g.nz;
    constexpr int RA = A_H / NW;   // rows per warp (2)
    float nz_[RA], np_[RA];
    const int Pbeg = imax(i0 - 1, 0), Pend = imin(i1, g.nx - 1);
    // the next plane's z and p_old are fetched into registers while the
    // current plane's products run
    auto fetch = [&](int P) {
#pragma unroll
        for (int m = 0; m < RA; ++m) {
            const int j = j0 - 1 + warp + m * NW;
            if (kin && j >= 0 && j < g.ny) {
                const int id = P * g.si + j * g.sj + kg;
                nz_[m] = z[id];
                if (!FIRST) np_[m] = pold[id];
            }
        }
    };
    if (Pbeg <= Pend) fetch(Pbeg);
    Acc acc;
    for (int P = i0 - 1; P <= i1; ++P) {
        if (P >= Pbeg && P <= Pend) {
            float* buf = sp[P % 3];
#pragma unroll
            for (int m = 0; m < RA; ++m) {
                const int row = warp + m * NW;
                const int j = j0 - 1 + row;
                float v = 0.f;
                if (kin && j >= 0 && j < g.ny) {
                    v = FIRST ? nz_[m] : fmaf(beta, np_[m], nz_[m]);
                    if (kcen && row >= 1 && row <= A_TJ && P >= i0 && P < i1) pnew[P * g.si + j * g.sj + kg] = v;
                }
                buf[row * W + lane] = v;
            }
            if (P + 1 <= Pend) fetch(P + 1);
        }
        __syncthreads();
        const int C = P - 1;
        if (C >= i0 && C < i1 && kcen) {
            const float* __restrict__ cb = sp[C % 3];
            const float* __restrict__ cw = sp[(C + 2) % 3];
            const float* __restrict__ ce = sp[(C + 1) % 3];
#pragma unroll
            for (int m = 0; m < RA; ++m) {
                const int row = 1 + warp + m * NW;
                const int j = j0 - 1 + row;
                if (row > A_TJ || j >= g.ny) break;
                const int pt = row * W + lane;
                const int id = C * g.si + j * g.sj + kg;
                const float pc = cb[pt];
                float val;
                if (A.interior(id)) {
                    val = A.k.c0 * pc + A.k.x1 * (cw[pt] + ce[pt]) + A.k.y1 * (cb[pt - W] + cb[pt + W]) +
                          A.k.z1 * (cb[pt - 1] + cb[pt + 1]);
                } else {
                    val = az_general(A, id, C, j, kg, g, cb, cw, ce, pt);
                }
                q[id] = val;
                acc_prod(acc, pc, val);
            }
        }
        __syncthreads();
    }
    double v[1] = {acc_value(acc)};
    if (last_block_sum<1>(v, partials, counter, sm)) {
        if (threadIdx.x == 0) st->alpha = st->rho / v[0];
    }
}

// ---- pass B -----------------------------------------------------------------
template <int S>
struct BGeom {
    static constexpr int TK = W - 2 * S;   // output columns
    static constexpr int TJ = 16;          // output rows
    static constexpr int H = TJ + 2 * S;   // rows of the level-0 region
    static constexpr int PL = W * H;       // cells per shared-memory plane
    // r' ring (S+1 planes), z_k rings (3 planes each, k = 0..S-1), pc_k rings
    // (2 planes each, k = 1..S-1), then the stencil-code ring (S+1 planes)
    static constexpr int FLOATS = (S + 1) * PL + 3 * S * PL + 2 * (S > 1 ? S - 1 : 0) * PL;
    static constexpr size_t BYTES = sizeof(float) * (size_t)FLOATS + (size_t)(S + 1) * PL;
};

// S = 0: Jacobi (z = r'/A_c, no stencil levels).
template <int S, bool FIRST>
__global__ void __launch_bounds__(NT, 3) k_pass_b(Geo g, ViewF A, int CI, ChebF cf, const float* __restrict__ r_in,
                                                float* __restrict__ r_out, const float* __restrict__ q,
                                                const float* __restrict__ p, float* __restrict__ e,
                                                float* __restrict__ z_out, double* partials, unsigned* counter,
                                                SolverState* st, SolverState* outer, int total_cap)
{
    using GB = BGeom<S>;
    constexpr int TK = GB::TK, TJ = GB::TJ, H = GB::H, PL = GB::PL;
    extern __shared__ float dsm[];
    __shared__ double sm[64];
    if (st->done) return;
    float* rp = dsm;                                        // [(S+1)][PL]
    float* zr = rp + (S + 1) * PL;                          // [S][3][PL]
    float* pcr = zr + 3 * S * PL;                           // [S-1][2][PL]
    uint8_t* cr = reinterpret_cast<uint8_t*>(dsm + GB::FLOATS);   // [(S+1)][PL]
    const float alpha = FIRST ? 0.f : (float)st->alpha;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    const int kg = k0 - S + lane;                          // this lane's global k
    const bool kin = kg >= 0 && kg < g.nz;
    const bool kcen = lane >= S && lane < S + TK && kin;
    // level-0 rows of this warp: warp, warp+8, ... (< H); the next plane's
    // inputs are fetched into registers while the current plane's Chebyshev
    // levels run
    constexpr int R0 = (H + NW - 1) / NW;
    float nr[R0], nq[R0], ne[R0], np[R0];
    uint8_t nc[R0];
    const int Ibeg = imax(i0 - S, 0), Iend = imin(i1 + S, g.nx) - 1;
    auto fetch = [&](int I) {
        const bool centre_plane = I >= i0 && I < i1;
#pragma unroll
        for (int m = 0; m < R0; ++m) {
            const int row = warp + m * NW;
            const int j = j0 - S + row;
            if (row < H && kin && j >= 0 && j < g.ny) {
                const int id = I * g.si + j * g.sj + kg;
                nr[m] = r_in[id];
                if (!FIRST) nq[m] = q[id];
                nc[m] = A.code ? A.code[id] : (uint8_t)2;
                if (!FIRST && centre_plane && kcen && row >= S && row < S + TJ) {
                    ne[m] = e[id];
                    np[m] = p[id];
                }
            }
        }
    };
    if (Ibeg <= Iend) fetch(Ibeg);
    Acc arr, arz;
    for (int I = i0 - S; I < i1 + S; ++I) {
        // ---- level 0 at plane I: r' = r - alpha q over the tile + S halo
        if (I >= Ibeg && I <= Iend) {
            const int slot = I % (S + 1);
            float* rpl = rp + slot * PL;
            uint8_t* crl = cr + slot * PL;
            float* z0 = zr + (I % 3) * PL;
            const bool plane_out = I >= i0 && I < i1;
#pragma unroll
            for (int m = 0; m < R0; ++m) {
                const int row = warp + m * NW;
                const int j = j0 - S + row;
                const int pt = row * W + lane;
                if (row >= H || !kin || j < 0 || j >= g.ny) continue;
                const float rv = FIRST ? nr[m] : fmaf(-alpha, nq[m], nr[m]);
                rpl[pt] = rv;
                crl[pt] = nc[m];
                if (S > 0) z0[pt] = cf.a0 * rv;
                if (plane_out && kcen && row >= S && row < S + TJ) {
                    const int id = I * g.si + j * g.sj + kg;
                    r_out[id] = rv;
                    e[id] = FIRST ? 0.f : fmaf(alpha, np[m], ne[m]);
                    acc_prod(arr, rv, rv);
                    if (S == 0) {
                        const float zv = rv * (nc[m] == 0 ? 1.f : (A.code ? 1.f / A.k.c0 : A.inv_diag(id)));
                        z_out[id] = zv;
                        acc_prod(arz, rv, zv);
                    }
                }
            }
            if (I + 1 <= Iend) fetch(I + 1);
        }
        __syncthreads();
        // ---- Chebyshev levels 1..S at plane I-LV over the tile + (S-LV) halo
        auto level = [&](auto lvc) {
            constexpr int LV = decltype(lvc)::value;
            const int Pk = I - LV;
            if (Pk >= imax(0, i0 - S + LV) && Pk < imin(g.nx, i1 + S - LV) && kin && lane >= LV &&
                lane < W - LV) {
                const float* __restrict__ zc = zr + ((LV - 1) * 3 + Pk % 3) * PL;
                const float* __restrict__ zw = zr + ((LV - 1) * 3 + (Pk + 2) % 3) * PL;
                const float* __restrict__ ze = zr + ((LV - 1) * 3 + (Pk + 1) % 3) * PL;
                const float* __restrict__ rpl = rp + (Pk % (S + 1)) * PL;
                const uint8_t* __restrict__ crl = cr + (Pk % (S + 1)) * PL;
                const float* __restrict__ pcp = LV >= 2 ? pcr + ((LV - 2) * 2 + Pk % 2) * PL : rpl;
                float* __restrict__ zo = LV < S ? zr + (LV * 3 + Pk % 3) * PL : nullptr;
                float* __restrict__ po = LV < S ? pcr + ((LV - 1) * 2 + Pk % 2) * PL : nullptr;
                const bool out_lane = LV == S && kcen && Pk >= i0 && Pk < i1;
                const float bk = cf.b[LV - 1], ak = cf.a[LV - 1];
                constexpr int ITER = (H - 2 * LV + NW - 1) / NW;
#pragma unroll
                for (int m = 0; m < ITER; ++m) {
                    const int row = LV + warp + m * NW;
                    if (row >= H - LV) break;
                    const int j = j0 - S + row;
                    if (j < 0 || j >= g.ny) continue;
                    const int pt = row * W + lane;
                    const float zcv = zc[pt];
                    float az;
                    if (crl[pt] == 1u) {   // all six neighbours present, base coefficients
                        az = A.k.c0 * zcv + A.k.x1 * (zw[pt] + ze[pt]) + A.k.y1 * (zc[pt - W] + zc[pt + W]) +
                             A.k.z1 * (zc[pt - 1] + zc[pt + 1]);
                    } else {
                        az = az_general(A, Pk * g.si + j * g.sj + kg, Pk, j, kg, g, zc, zw, ze, pt);
                    }
                    const float rv = rpl[pt];
                    const float pck = fmaf(bk, pcp[pt], rv - az);
                    const float zk = fmaf(ak, pck, zcv);
                    if (LV < S) {
                        zo[pt] = zk;
                        po[pt] = pck;
                    } else if (out_lane && row >= S && row < S + TJ) {
                        z_out[Pk * g.si + j * g.sj + kg] = zk;
                        acc_prod(arz, rv, zk);
                    }
                }
            }
            __syncthreads();
        };
        if constexpr (S >= 1) level(std::integral_constant<int, 1>{});
        if constexpr (S >= 2) level(std::integral_constant<int, 2>{});
        if constexpr (S >= 3) level(std::integral_constant<int, 3>{});
        if constexpr (S >= 4) level(std::integral_constant<int, 4>{});
        if constexpr (S >= 5) level(std::integral_constant<int, 5>{});
        if constexpr (S >= 6) level(std::integral_constant<int, 6>{});
    }
    double v[2] = {acc_value(arr), acc_value(arz)};
    if (last_block_sum<2>(v, partials, counter, sm)) {
        if (threadIdx.x == 0) {
            if (FIRST) {
                st->rho = v[1];
            } else {
                const double err = sqrt(v[0]);
                const int kk = st->k + 1;
                st->k = kk;
                st->err = err;
                const int total = outer->iters + 1;
                outer->iters = total;
                if (err < st->tol) { st->done = 1; st->status = LES_OK; }
                else if (!isfinite(err)) { st->done = 1; st->status = LES_NONFINITE; }
                else if (kk >= st->max_iter || total >= total_cap) { st->done = 1; st->status = LES_NOT_CONVERGED; }
                st->beta = v[1] / st->rho;
                st->rho = v[1];
            }
        }
    }
}

// ---- TMA versions ------------------------------------------------------------
// The same two passes with every plane of input staged by the Tensor Memory
// Accelerator: one thread issues cp.async.bulk.tensor copies of the next
// planes' tiles into a shared-memory ring two planes ahead of the
// computation, and the block waits on the slot's mbarrier.  Out-of-range halo
// cells read as zero.  A TMA box must start on a 16-byte boundary in k, so
// each box starts at the k rounded down to 4 floats (16 bytes for the byte
// codes) and is a few cells wider; threads index from the remainder.
// Requires nz % 16 == 0 (16-byte row pitch of the byte-coded stencil).

constexpr int TMA_BX = 36;    // float box width (32 + up to 3 alignment cells, rounded to 16 B)
constexpr int TMA_CBX = 48;   // code box width (32 + up to 15 alignment cells)

__device__ __forceinline__ int align_down(int x, int a) { return x & ~(a - 1); }

// error path of a timed-out TMA wait: report through the solver state and
// leave (the host stops on done)
__device__ __forceinline__ void tma_timeout(SolverState* st)
{
    st->status = LES_TIMEOUT;
    st->done = 1;
    __threadfence();
}

constexpr int A2_SLOT = 2 * TMA_BX * A_H * 4 + TMA_CBX * A_H;   // z, pold, code = 5376 B
constexpr int A2_RING = 4;

template <bool FIRST>
__global__ void __launch_bounds__(NT) k_pass_a_tma(Geo g, ViewF A, int CI, const __grid_constant__ CUtensorMap mz,
                                                    const __grid_constant__ CUtensorMap mp,
                                                    const __grid_constant__ CUtensorMap mc, float* __restrict__ pnew,
                                                    float* __restrict__ q, double* partials, unsigned* counter,
                                                    SolverState* st)
{
    __shared__ __align__(128) unsigned char ring[A2_RING][A2_SLOT];
    __shared__ float sp[3][A_PL];
    __shared__ uint8_t sc[3][A_PL];
    __shared__ __align__(8) uint64_t bar[A2_RING];
    __shared__ double sm[32];
    if (st->done) return;
    const float beta = FIRST ? 0.f : (float)st->beta;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k0 = blockIdx.x * A_TK, j0 = blockIdx.y * A_TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    const int kg = k0 - 1 + lane;
    const bool kin = kg >= 0 && kg < g.nz;
    const bool kcen = lane >= 1 && lane <= A_TK && kg < g.nz;
    const int xf = align_down(k0 - 1, 4), of = (k0 - 1) - xf;
    const int xc = align_down(k0 - 1, 16), oc = (k0 - 1) - xc;
    constexpr unsigned FB = TMA_BX * A_H * 4, CB = TMA_CBX * A_H;
    if (threadIdx.x == 0) {
        for (int s = 0; s < A2_RING; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int Pbeg = imax(i0 - 1, 0), Pend = imin(i1, g.nx - 1);   // planes loaded: [Pbeg, Pend]
    auto issue = [&](int P) {
        const int s = P % A2_RING;
        unsigned char* dst = ring[s];
        mbar_arrive_expect_tx(&bar[s], FIRST ? FB + CB : 2 * FB + CB);
        tma_load_3d(dst, &mz, &bar[s], xf, j0 - 1, P);
        if (!FIRST) tma_load_3d(dst + FB, &mp, &bar[s], xf, j0 - 1, P);
        tma_load_3d(dst + 2 * FB, &mc, &bar[s], xc, j0 - 1, P);
    };
    if (threadIdx.x == 0)
        for (int P = Pbeg; P <= imin(Pbeg + 1, Pend); ++P) issue(P);
    unsigned phase = 0;   // bit s: parity of the next wait on slot s
    Acc acc;
    for (int P = i0 - 1; P <= i1; ++P) {
        if (P >= Pbeg && P <= Pend) {
            if (threadIdx.x == 0 && P + 2 <= Pend) issue(P + 2);
            const int s = P % A2_RING;
            if (!mbar_wait_bounded(&bar[s], (phase >> s) & 1u)) {
                tma_timeout(st);
                mbar_drain(bar, phase, A2_RING, P, 2, Pend);   // late copies land before leaving
                return;
            }
            phase ^= 1u << s;
            const float* tz = reinterpret_cast<const float*>(ring[s]);
            const float* tp = tz + TMA_BX * A_H;
            const uint8_t* tc = ring[s] + 2 * FB;
            float* buf = sp[P % 3];
            uint8_t* cbuf = sc[P % 3];
#pragma unroll
            for (int rr = 0; rr < A_H / NW; ++rr) {
                const int row = warp + rr * NW;
                const int j = j0 - 1 + row;
                const int pt = row * W + lane;
                float v = 0.f;
                if (kin && j >= 0 && j < g.ny) {
                    const float zz = tz[row * TMA_BX + of + lane];
                    v = FIRST ? zz : fmaf(beta, tp[row * TMA_BX + of + lane], zz);
                    if (kcen && row >= 1 && row <= A_TJ && P >= i0 && P < i1) pnew[P * g.si + j * g.sj + kg] = v;
                }
                buf[pt] = v;
                cbuf[pt] = tc[row * TMA_CBX + oc + lane];
            }
        }
        __syncthreads();
        const int C = P - 1;
        if (C >= i0 && C < i1 && kcen) {
            const float* cb = sp[C % 3];
            const float* cw = sp[(C + 2) % 3];
            const float* ce = sp[(C + 1) % 3];
            const uint8_t* cc = sc[C % 3];
            for (int row = 1 + warp; row <= A_TJ; row += NW) {
                const int j = j0 - 1 + row;
                if (j >= g.ny) break;
                const int pt = row * W + lane;
                const float pc = cb[pt];
                float val;
                if (cc[pt] == 1u) {
                    val = A.k.c0 * pc + A.k.x1 * (cw[pt] + ce[pt]) + A.k.y1 * (cb[pt - W] + cb[pt + W]) +
                          A.k.z1 * (cb[pt - 1] + cb[pt + 1]);
                } else {
                    CoefF a = A.at(C * g.si + j * g.sj + kg);
                    val = a.c * pc;
                    if (C > 0) val += a.w * cw[pt];
                    if (C < g.nx - 1) val += a.e * ce[pt];
                    if (j > 0) val += a.s * cb[pt - W];
                    if (j < g.ny - 1) val += a.n * cb[pt + W];
                    if (kg > 0) val += a.b * cb[pt - 1];
                    if (kg < g.nz - 1) val += a.t * cb[pt + 1];
                }
                q[C * g.si + j * g.sj + kg] = val;
                acc_prod(acc, pc, val);
            }
        }
        __syncthreads();
    }
    double v[1] = {acc_value(acc)};
    if (last_block_sum<1>(v, partials, counter, sm)) {
        if (threadIdx.x == 0) st->alpha = st->rho / v[0];
    }
}

template <int S>
struct BTma {
    static constexpr int H = BGeom<S>::H;
    static constexpr unsigned FB = TMA_BX * H * 4;        // r or q box
    static constexpr unsigned CB = TMA_CBX * H;           // code box
    static constexpr unsigned EB = W * BGeom<S>::TJ * 4;  // e or p box (output tile)
    static constexpr unsigned R128(unsigned b) { return (b + 127u) & ~127u; }
    static constexpr unsigned OFF_Q = R128(FB), OFF_C = OFF_Q + R128(FB), OFF_E = OFF_C + R128(CB),
                              OFF_P = OFF_E + R128(EB), SLOT = OFF_P + R128(EB);
    static constexpr int RING = 3;
    // ring, then the compute rings of BGeom, then the barriers
    // + 128: the kernel aligns the dynamic shared-memory base to 128 bytes
    static constexpr size_t BYTES = (size_t)RING * SLOT + ((BGeom<S>::BYTES + 127) & ~(size_t)127) + 64 + 128;
};

template <int S, bool FIRST>
__global__ void __launch_bounds__(NT) k_pass_b_tma(Geo g, ViewF A, int CI, ChebF cf,
                                                    const __grid_constant__ CUtensorMap mr,
                                                    const __grid_constant__ CUtensorMap mq,
                                                    const __grid_constant__ CUtensorMap mc,
                                                    const __grid_constant__ CUtensorMap me,
                                                    const __grid_constant__ CUtensorMap mp, float* __restrict__ r_out,
                                                    float* __restrict__ e, float* __restrict__ z_out,
                                                    double* partials, unsigned* counter, SolverState* st,
                                                    SolverState* outer, int total_cap)
{
    using GB = BGeom<S>;
    using TB = BTma<S>;
    constexpr int TK = GB::TK, TJ = GB::TJ, H = GB::H, PL = GB::PL;
    extern __shared__ __align__(128) unsigned char dyn_raw[];
    __shared__ double sm[64];
    if (st->done) return;
    // TMA destinations must be 128-byte aligned
    unsigned char* dyn = dyn_raw + ((128u - (smem_addr(dyn_raw) & 127u)) & 127u);
    unsigned char* ring = dyn;
    float* rp = reinterpret_cast<float*>(dyn + TB::RING * TB::SLOT);
    float* zr = rp + (S + 1) * PL;
    float* pcr = zr + 3 * S * PL;
    uint8_t* cr = reinterpret_cast<uint8_t*>(rp + GB::FLOATS);
    uint64_t* bar = reinterpret_cast<uint64_t*>(dyn + TB::RING * TB::SLOT + ((GB::BYTES + 127) & ~(size_t)127));
    const float alpha = FIRST ? 0.f : (float)st->alpha;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    const int kg = k0 - S + lane;
    const bool kin = kg >= 0 && kg < g.nz;
    const bool kcen = lane >= S && lane < S + TK && kin;
    const int xf = align_down(k0 - S, 4), of = (k0 - S) - xf;
    const int xc = align_down(k0 - S, 16), oc = (k0 - S) - xc;
    const int xe = align_down(k0, 4), oe = k0 - xe;
    if (threadIdx.x == 0) {
        for (int s = 0; s < TB::RING; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int Ibeg = imax(i0 - S, 0), Iend = imin(i1 + S, g.nx) - 1;   // planes loaded
    auto issue = [&](int I) {
        const int s = I % TB::RING;
        unsigned char* dst = ring + s * TB::SLOT;
        const bool centre = I >= i0 && I < i1 && !FIRST;
        mbar_arrive_expect_tx(&bar[s], (FIRST ? TB::FB : 2 * TB::FB) + TB::CB + (centre ? 2 * TB::EB : 0));
        tma_load_3d(dst, &mr, &bar[s], xf, j0 - S, I);
        if (!FIRST) tma_load_3d(dst + TB::OFF_Q, &mq, &bar[s], xf, j0 - S, I);
        tma_load_3d(dst + TB::OFF_C, &mc, &bar[s], xc, j0 - S, I);
        if (centre) {
            tma_load_3d(dst + TB::OFF_E, &me, &bar[s], xe, j0, I);
            tma_load_3d(dst + TB::OFF_P, &mp, &bar[s], xe, j0, I);
        }
    };
    if (threadIdx.x == 0)
        for (int I = Ibeg; I <= imin(Ibeg + 1, Iend); ++I) issue(I);
    unsigned phase = 0;
    Acc arr, arz;
    for (int I = i0 - S; I < i1 + S; ++I) {
        if (I >= Ibeg && I <= Iend) {
            if (threadIdx.x == 0 && I + 2 <= Iend) issue(I + 2);
            const int s = I % TB::RING;
            if (!mbar_wait_bounded(&bar[s], (phase >> s) & 1u)) {
                tma_timeout(st);
                mbar_drain(bar, phase, TB::RING, I, 2, Iend);   // late copies land before leaving
                return;
            }
            phase ^= 1u << s;
            const unsigned char* sl = ring + s * TB::SLOT;
            const float* tr = reinterpret_cast<const float*>(sl);
            const float* tq = reinterpret_cast<const float*>(sl + TB::OFF_Q);
            const uint8_t* tc = sl + TB::OFF_C;
            const float* te = reinterpret_cast<const float*>(sl + TB::OFF_E);
            const float* tp = reinterpret_cast<const float*>(sl + TB::OFF_P);
            const int slot = I % (S + 1);
            float* rpl = rp + slot * PL;
            uint8_t* crl = cr + slot * PL;
            float* z0 = zr + (I % 3) * PL;
            const bool plane_out = I >= i0 && I < i1;
            for (int row = warp; row < H; row += NW) {
                const int j = j0 - S + row;
                if (!kin || j < 0 || j >= g.ny) continue;
                const int pt = row * W + lane;
                const float rold = tr[row * TMA_BX + of + lane];
                const float rv = FIRST ? rold : fmaf(-alpha, tq[row * TMA_BX + of + lane], rold);
                rpl[pt] = rv;
                const uint8_t cd = tc[row * TMA_CBX + oc + lane];
                crl[pt] = cd;
                if (S > 0) z0[pt] = cf.a0 * rv;
                if (plane_out && kcen && row >= S && row < S + TJ) {
                    const int id = I * g.si + j * g.sj + kg;
                    const int ept = (row - S) * W + oe + (lane - S);
                    r_out[id] = rv;
                    e[id] = FIRST ? 0.f : fmaf(alpha, tp[ept], te[ept]);
                    acc_prod(arr, rv, rv);
                    if (S == 0) {
                        const float zv = rv * (cd == 0 ? 1.f : 1.f / A.k.c0);
                        z_out[id] = zv;
                        acc_prod(arz, rv, zv);
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int lv = 1; lv <= S; ++lv) {
            const int Pk = I - lv;
            if (Pk >= imax(0, i0 - S + lv) && Pk < imin(g.nx, i1 + S - lv) && kin && lane >= lv &&
                lane < W - lv) {
                const float* zc = zr + ((lv - 1) * 3 + Pk % 3) * PL;
                const float* zw = zr + ((lv - 1) * 3 + (Pk + 2) % 3) * PL;
                const float* ze = zr + ((lv - 1) * 3 + (Pk + 1) % 3) * PL;
                const float* rpl = rp + (Pk % (S + 1)) * PL;
                const uint8_t* crl = cr + (Pk % (S + 1)) * PL;
                const float* pcp = lv >= 2 ? pcr + ((lv - 2) * 2 + Pk % 2) * PL : rpl;
                float* zo = lv < S ? zr + (lv * 3 + Pk % 3) * PL : nullptr;
                float* po = lv < S ? pcr + ((lv - 1) * 2 + Pk % 2) * PL : nullptr;
                const bool out_lane = lv == S && kcen && Pk >= i0 && Pk < i1;
                for (int row = lv + warp; row < H - lv; row += NW) {
                    const int j = j0 - S + row;
                    if (j < 0 || j >= g.ny) continue;
                    const int pt = row * W + lane;
                    const unsigned cd = crl[pt];
                    const float zcv = zc[pt];
                    float az;
                    if (cd == 1u) {
                        az = A.k.c0 * zcv + A.k.x1 * (zw[pt] + ze[pt]) + A.k.y1 * (zc[pt - W] + zc[pt + W]) +
                             A.k.z1 * (zc[pt - 1] + zc[pt + 1]);
                    } else {
                        CoefF a = A.at(Pk * g.si + j * g.sj + kg);
                        az = a.c * zcv;
                        if (Pk > 0) az += a.w * zw[pt];
                        if (Pk < g.nx - 1) az += a.e * ze[pt];
                        if (j > 0) az += a.s * zc[pt - W];
                        if (j < g.ny - 1) az += a.n * zc[pt + W];
                        if (kg > 0) az += a.b * zc[pt - 1];
                        if (kg < g.nz - 1) az += a.t * zc[pt + 1];
                    }
                    const float rv = rpl[pt];
                    const float pck = fmaf(cf.b[lv - 1], pcp[pt], rv - az);
                    const float zk = fmaf(cf.a[lv - 1], pck, zcv);
                    if (lv < S) {
                        zo[pt] = zk;
                        po[pt] = pck;
                    } else if (out_lane && row >= S && row < S + TJ) {
                        z_out[Pk * g.si + j * g.sj + kg] = zk;
                        acc_prod(arz, rv, zk);
                    }
                }
            }
            __syncthreads();
        }
    }
    double v[2] = {acc_value(arr), acc_value(arz)};
    if (last_block_sum<2>(v, partials, counter, sm)) {
        if (threadIdx.x == 0) {
            if (FIRST) {
                st->rho = v[1];
            } else {
                const double err = sqrt(v[0]);
                const int kk = st->k + 1;
                st->k = kk;
                st->err = err;
                const int total = outer->iters + 1;
                outer->iters = total;
                if (err < st->tol) { st->done = 1; st->status = LES_OK; }
                else if (!isfinite(err)) { st->done = 1; st->status = LES_NONFINITE; }
                else if (kk >= st->max_iter || total >= total_cap) { st->done = 1; st->status = LES_NOT_CONVERGED; }
                st->beta = v[1] / st->rho;
                st->rho = v[1];
            }
        }
    }
}

template <int S>
const void* pass_b_fn(bool first)
{
    return first ? (const void*)k_pass_b<S, true> : (const void*)k_pass_b<S, false>;
}

template <int S>
const void* pass_b_tma_fn(bool first)
{
    return first ? (const void*)k_pass_b_tma<S, true> : (const void*)k_pass_b_tma<S, false>;
}

template <int S>
les_status launch_b(les_ctx* c, bool first, int CI, ViewF A, const ChebF& cf, const float* rin, float* rout,
                    const float* q, const float* p, float* e, float* z, SolverState* in, SolverState* out, int cap)
{
    const Geo& g = c->g;
    const size_t bytes = BGeom<S>::BYTES;
    const dim3 gr((g.nz + BGeom<S>::TK - 1) / BGeom<S>::TK, (g.ny + BGeom<S>::TJ - 1) / BGeom<S>::TJ,
                  (g.nx + CI - 1) / CI);
    auto kf = first ? k_pass_b<S, true> : k_pass_b<S, false>;
    cudaEvent_t e1 = nullptr;
    if (c->prof_on) prof_begin(c, PROF_IN_CHEB, &e1);
    kf<<<gr, NT, bytes, c->stream>>>(g, A, CI, cf, rin, rout, q, p, e, z, c->partials, c->counters + 14, in, out,
                                      cap);
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return LES_OK;
}

// Chunk length along i so that a pass fills about one wave of resident
// blocks (longer chunks amortise the i-halo of the march).
int chunk_len(les_ctx* c, const void* fn, size_t smem, int tiles, int min_ci)
{
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, NT, smem);
    int chunks = (occ < 1 ? 1 : occ) * c->sms / (tiles < 1 ? 1 : tiles);
    if (chunks < 1) chunks = 1;
    int ci = (c->g.nx + chunks - 1) / chunks;
    return ci < min_ci ? min_ci : ci;
}

}  // namespace

namespace les {

bool tma_encode_3d(CUtensorMap* map, CUtensorMapDataType dtype, size_t esize, void* base, int nx, int ny, int nz,
                   unsigned bx, unsigned by)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    }
    if (!encode) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nz, (cuuint64_t)ny, (cuuint64_t)nx};
    cuuint64_t strides[2] = {(cuuint64_t)nz * esize, (cuuint64_t)ny * nz * esize};
    cuuint32_t box[3] = {bx, by, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return encode(map, dtype, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps over the inner-solve vectors, built once per context and
// Chebyshev degree (the boxes of pass B depend on the halo).
struct TmaCache {
    int S = -1;
    bool ok = false;
    CUtensorMap a_z, a_p[2], a_c;                 // pass A: z, p_old (ping-pong), codes
    CUtensorMap b_r[2], b_q, b_c, b_e, b_p[2];    // pass B
};

void tma_cache_free(TmaCache* t) { delete t; }

static bool build_tma(les_ctx* c, int S)
{
    if (!c->tma) c->tma = new TmaCache();
    TmaCache& t = *c->tma;
    if (t.S == S) return t.ok;
    const Geo& g = c->g;
    const unsigned H = 16 + 2 * S;
    const auto F = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const auto U8 = CU_TENSOR_MAP_DATA_TYPE_UINT8;
    bool ok = g.nz % 16 == 0 && c->code != nullptr;
    ok = ok && tma_encode_3d(&t.a_z, F, 4, c->f[1], g.nx, g.ny, g.nz, TMA_BX, A_H);
    ok = ok && tma_encode_3d(&t.a_p[0], F, 4, c->f[2], g.nx, g.ny, g.nz, TMA_BX, A_H);
    ok = ok && tma_encode_3d(&t.a_p[1], F, 4, c->f[3], g.nx, g.ny, g.nz, TMA_BX, A_H);
    ok = ok && tma_encode_3d(&t.a_c, U8, 1, c->code, g.nx, g.ny, g.nz, TMA_CBX, A_H);
    ok = ok && tma_encode_3d(&t.b_r[0], F, 4, c->f[0], g.nx, g.ny, g.nz, TMA_BX, H);
    ok = ok && tma_encode_3d(&t.b_r[1], F, 4, c->f[6], g.nx, g.ny, g.nz, TMA_BX, H);
    ok = ok && tma_encode_3d(&t.b_q, F, 4, c->f[4], g.nx, g.ny, g.nz, TMA_BX, H);
    ok = ok && tma_encode_3d(&t.b_c, U8, 1, c->code, g.nx, g.ny, g.nz, TMA_CBX, H);
    ok = ok && tma_encode_3d(&t.b_e, F, 4, c->f[5], g.nx, g.ny, g.nz, W, 16);
    ok = ok && tma_encode_3d(&t.b_p[0], F, 4, c->f[2], g.nx, g.ny, g.nz, W, 16);
    ok = ok && tma_encode_3d(&t.b_p[1], F, 4, c->f[3], g.nx, g.ny, g.nz, W, 16);
    t.S = S;
    t.ok = ok;
    return ok;
}

ChebF cheb_coefs(const les_pcg_opts* o)
{
    ChebF cf{};
    const int S = o->precond == LES_PC_CHEBYSHEV ? o->degree - 1 : 0;
    if (S > 0) {
        const double d = (o->lambda_max + o->lambda_min) / 2.0;
        const double cc = (o->lambda_max - o->lambda_min) / 2.0;
        double alpha = 2.0 / d;
        cf.a0 = (float)alpha;
        for (int k = 1; k <= S && k <= 8; ++k) {
            const double beta = (cc * alpha / 2.0) * (cc * alpha / 2.0);
            alpha = 1.0 / (d - beta);
            cf.a[k - 1] = (float)alpha;
            cf.b[k - 1] = (float)beta;
        }
    }
    return cf;
}

bool fused_supported(const les_pcg_opts* o)
{
    if (o->precond == LES_PC_JACOBI) return true;
    return o->precond == LES_PC_CHEBYSHEV && o->degree >= 2 && o->degree <= 7;
}

// One inner FP32 solve A e = r (e from 0) with the fused passes.  f[0] holds
// the right-hand side on entry and is used as scratch.
// Everything a launch of the fused passes needs, fixed for one solve (and
// baked into a captured graph).
struct FusedPlan {
    bool col = false;   // register-column passes (les_col.cu) instead of the tiles below
    ColPlan cp;
    int S = 0;
    ChebF cf{};
    bool tma = false;
    size_t smem_b = 0;
    const void* fb[2] = {};
    int CIA = 8, CIB = 8;
    dim3 ga, gb;
    ViewF A{};
    SolverState* in = nullptr;
    SolverState* out = nullptr;
    int cap = 0;
};

les_status fused_plan(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out, FusedPlan& P)
{
    const Geo& g = c->g;
    const int S = o->precond == LES_PC_JACOBI ? 0 : o->degree - 1;
    if (col_supported(c, o)) {
        P.col = true;
        return col_plan(c, o, A, in, out, P.cp);
    }
    P.S = S;
    P.A = A;
    P.in = in;
    P.out = out;
    P.cap = o->max_iter;
    P.cf = cheb_coefs(o);
    const bool tma = c->opt_tma && build_tma(c, S);
    P.tma = tma;
    size_t smem_b = 0;
    int tk_b = W, tj_b = 16;
    const void** fb = P.fb;
    switch (S) {
#define LES_CASE(s)                                                                              \
    case s:                                                                                      \
        smem_b = tma ? BTma<s>::BYTES : BGeom<s>::BYTES;                                        \
        tk_b = BGeom<s>::TK; tj_b = BGeom<s>::TJ;                                               \
        fb[0] = tma ? pass_b_tma_fn<s>(true) : pass_b_fn<s>(true);                               \
        fb[1] = tma ? pass_b_tma_fn<s>(false) : pass_b_fn<s>(false);                             \
        break;
        LES_CASE(0) LES_CASE(1) LES_CASE(2) LES_CASE(3) LES_CASE(4) LES_CASE(5)
    default: LES_CASE(6)
#undef LES_CASE
    }
    P.smem_b = smem_b;
    if (smem_b > 48 * 1024)
        for (int q = 0; q < 2; ++q) {
            les_status st = check_cuda(
                c, cudaFuncSetAttribute(fb[q], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b), "smem attribute");
            if (st) return st;
        }
    const int tiles_a = ((g.nz + A_TK - 1) / A_TK) * ((g.ny + A_TJ - 1) / A_TJ);
    const int tiles_b = ((g.nz + tk_b - 1) / tk_b) * ((g.ny + tj_b - 1) / tj_b);
    const void* fa = tma ? (const void*)k_pass_a_tma<false> : (const void*)k_pass_a<false>;
    P.CIA = c->tune_cia > 0 ? c->tune_cia : chunk_len(c, fa, 0, tiles_a, 8);
    P.CIB = (c->tune_cib > 0 && c->tune_s == S) ? c->tune_cib : chunk_len(c, fb[1], smem_b, tiles_b, 4 * S > 8 ? 4 * S : 8);
    P.ga = dim3((g.nz + A_TK - 1) / A_TK, (g.ny + A_TJ - 1) / A_TJ, (g.nx + P.CIA - 1) / P.CIA);
    P.gb = dim3((g.nz + tk_b - 1) / tk_b, (g.ny + tj_b - 1) / tj_b, (g.nx + P.CIB - 1) / P.CIB);
    return LES_OK;
}

// Pass A: p_new = pb[pc^1] from z and p_old = pb[pc].
les_status emit_pass_a(les_ctx* c, const FusedPlan& P, bool first, int pc)
{
    if (P.col) return col_pass_a(c, P.cp, first, pc);
    float *z = c->f[1], *pb[2] = {c->f[2], c->f[3]}, *q = c->f[4];
    if (P.tma) {
        const TmaCache& t = *c->tma;
        auto ka = first ? k_pass_a_tma<true> : k_pass_a_tma<false>;
        launch_p(c, PROF_IN_SPMV, ka, P.ga, dim3(NT), c->g, P.A, P.CIA, t.a_z, t.a_p[pc], t.a_c, pb[pc ^ 1], q,
                 c->partials, c->counters + 15, P.in);
    } else {
        auto ka = first ? k_pass_a<true> : k_pass_a<false>;
        launch_p(c, PROF_IN_SPMV, ka, P.ga, dim3(NT), c->g, P.A, P.CIA, (const float*)z, (const float*)pb[pc],
                 pb[pc ^ 1], q, c->partials, c->counters + 15, P.in);
    }
    return check_launch(c, "pass A");
}

// Pass B: r[rin] -> r[rin^1], p = pb[pcur].
les_status emit_pass_b(les_ctx* c, const FusedPlan& P, bool first, int rin, int pcur)
{
    if (P.col) return col_pass_b(c, P.cp, first, rin);
    float* r[2] = {c->f[0], c->f[6]};
    float *z = c->f[1], *pb[2] = {c->f[2], c->f[3]}, *q = c->f[4], *e = c->f[5];
    if (!P.tma) {
        switch (P.S) {
        case 0: return launch_b<0>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        case 1: return launch_b<1>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        case 2: return launch_b<2>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        case 3: return launch_b<3>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        case 4: return launch_b<4>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        case 5: return launch_b<5>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        default: return launch_b<6>(c, first, P.CIB, P.A, P.cf, r[rin], r[rin ^ 1], q, pb[pcur], e, z, P.in, P.out, P.cap);
        }
    }
    const TmaCache& t = *c->tma;
    cudaEvent_t e1 = nullptr;
    if (c->prof_on) prof_begin(c, PROF_IN_CHEB, &e1);
    const void* fn = P.fb[first ? 0 : 1];
    float* rout = r[rin ^ 1];
    double* parts = c->partials;
    unsigned* cnt = c->counters + 14;
    int CI = P.CIB, cap = P.cap;
    Geo gg = c->g;
    ViewF AA = P.A;
    ChebF cff = P.cf;
    SolverState *in = P.in, *out = P.out;
    void* args[] = {&gg, &AA, &CI, &cff, (void*)&t.b_r[rin], (void*)&t.b_q, (void*)&t.b_c, (void*)&t.b_e,
                    (void*)&t.b_p[pcur], &rout, &e, &z, &parts, &cnt, &in, &out, &cap};
    les_status st = check_cuda(c, cudaLaunchKernel(fn, P.gb, dim3(NT), args, P.smem_b, c->stream), "pass B (TMA)");
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return st;
}

les_status inner_solve_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out,
                             int inner_cap)
{
    FusedPlan P;
    les_status st = fused_plan(c, o, A, in, out, P);
    if (st) return st;
    st = emit_pass_b(c, P, true, 0, 0);   // z = M^-1 r, rho, e = 0
    if (st) return st;
    int rc = 1, pc = 0, launched = 0, batch = 4;
    for (;;) {
        for (int it = 0; it < batch; ++it) {
            if ((st = emit_pass_a(c, P, launched + it == 0, pc))) return st;
            pc ^= 1;
            if ((st = emit_pass_b(c, P, false, rc, pc))) return st;
            rc ^= 1;
        }
        launched += batch;
        st = read_state(c);
        if (st) return st;
        if (c->h_state[1].done || launched >= inner_cap) break;
        batch = batch < 32 ? batch * 2 : 32;
    }
    if (c->h_state[1].status == LES_TIMEOUT) return fail(c, LES_TIMEOUT, "a TMA wait in the inner solve timed out");
    return LES_OK;
}

// ---- the whole mixed solve as a CUDA graph -----------------------------------
// Both loops run on the device: each is a conditional `while` node whose body
// ends with a one-thread kernel that sets the loop's condition from the
// solver state.  The inner body holds 2 * INNER_BODY_PAIRS iterations (an
// even number, so that the ping-pong buffers are in the same roles every time
// it repeats; kernels of an iteration that starts after convergence exit at
// once).

__global__ void k_cond_inner(const SolverState* in, cudaGraphConditionalHandle h, int cap)
{
    cudaGraphSetConditional(h, (!in->done && in->k < cap) ? 1u : 0u);
}

__global__ void k_cond_outer(const SolverState* out, cudaGraphConditionalHandle h, int max_outer, int cap)
{
    cudaGraphSetConditional(h, (!out->done && out->k < max_outer && out->iters < cap) ? 1u : 0u);
}

// Adds a `while` loop at the current capture point of c->stream: creates the
// loop's condition handle, captures `entry(h)` (a kernel that sets the
// condition from the solver state, so the loop can be skipped and is
// re-armed each time an enclosing loop comes back to it), adds the
// conditional node, captures its body with `body(h)` (which must end by
// setting the condition again), and resumes the capture after the node.
template <class Entry, class Body>
static les_status capture_while(les_ctx* c, Entry entry, Body body)
{
    return capture_while_on(&c->stream, [c](cudaError_t r, const char* what) { return check_cuda(c, r, what); },
                            entry, body);
}

// Emits the mixed solve of les_mixed.cu (outer FP64 defect correction, inner
// fused FP32 PCG) into the capture in progress on c->stream.
les_status capture_mixed_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, int keep_tol)
{
    SolverState* out = c->state;
    SolverState* in = c->state + 1;
    const int inner_cap = o->inner_max_iter > 0 ? o->inner_max_iter : o->max_iter;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 50;
    FusedPlan P;
    les_status st = fused_plan(c, o, A, in, out, P);
    if (st) return st;
    if ((st = emit_outer_start(c, o, keep_tol))) return st;   // tol, r = b - A x, ||r||
    auto set_outer = [&](cudaGraphConditionalHandle h) -> les_status {
        launch(c, k_cond_outer, 1, 1, (const SolverState*)out, h, max_outer, o->max_iter);
        return check_launch(c, "outer condition");
    };
    auto set_inner = [&](cudaGraphConditionalHandle h) -> les_status {
        launch(c, k_cond_inner, 1, 1, (const SolverState*)in, h, inner_cap);
        return check_launch(c, "inner condition");
    };
    return capture_while(c, set_outer, [&](cudaGraphConditionalHandle ho) -> les_status {
        les_status s2;
        if ((s2 = emit_inner_start(c, o, inner_cap))) return s2;     // inner state from the outer residual
        if ((s2 = emit_pass_b(c, P, true, 0, 0))) return s2;          // z = M^-1 r, rho, e = 0
        if ((s2 = emit_pass_a(c, P, true, 0))) return s2;             // iteration 1: p1 = z
        if ((s2 = emit_pass_b(c, P, false, 1, 1))) return s2;         //   r1 -> r0
        s2 = capture_while(c, set_inner, [&](cudaGraphConditionalHandle hi) -> les_status {
            les_status s3;
            for (int q = 0; q < INNER_BODY_PAIRS; ++q) {
                if ((s3 = emit_pass_a(c, P, false, 1))) return s3;    // p1 -> p0
                if ((s3 = emit_pass_b(c, P, false, 0, 0))) return s3; // r0 -> r1
                if ((s3 = emit_pass_a(c, P, false, 0))) return s3;    // p0 -> p1
                if ((s3 = emit_pass_b(c, P, false, 1, 1))) return s3; // r1 -> r0
            }
            return set_inner(hi);
        });
        if (s2) return s2;
        if ((s2 = emit_outer_update(c, P.col))) return s2;                   // x += e, r = b - A x, ||r||
        return set_outer(ho);
    });
}

}  // namespace les
