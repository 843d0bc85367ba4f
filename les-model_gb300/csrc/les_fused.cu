// les_fused.cu -- the FP32 inner PCG iteration of the mixed-precision solve in
// two fused passes over the grid (Jacobi or Chebyshev preconditioner).
//
// Pass A (k_pass_a): p = z + beta p_old, q = A p, p.q -> alpha.
// Pass B (k_pass_b): r' = r - alpha q, e' = e + alpha p, ||r'||^2, then the
//   whole preconditioner z = M^-1 r' (Chebyshev: S = degree-1 stencil levels,
//   the recurrence of les-model src/pressure.cpp:871-905; Jacobi: r'/A_c),
//   and r'.z -> beta, rho.  Convergence is tested on ||r'||.
//
// Both passes march along i (the slowest axis) over a 32(k) x 8(j) tile and a
// chunk of planes.  Pass A keeps a ring of three (tile + 1 halo) planes of p in
// shared memory.  Pass B is temporally blocked: at march step I it computes
// level 0 (r') at plane I and Chebyshev level k at plane I-k, each level over
// the tile grown by S-k halo cells, from rings of planes of the level below
// held in shared memory; only r, q, p, e are read and r', e', z written, once
// per cell.  That is 17 + 29 bytes per cell per inner iteration instead of the
// 104 of five unfused kernels.
//
// Inner products are accumulated per thread in compensated FP32 (TwoProd +
// TwoSum, i.e. double-float, ~48-bit significand) and summed across threads
// and blocks in FP64; GB300's FP64 pipe is ~70x slower than its FP32 pipe, so
// a per-cell FP64 add tree would dominate these memory-bound kernels.
#include <cmath>

#include "les_internal.cuh"
#include "les_mixed.cuh"

using namespace les;

namespace {

constexpr int TK = 32, TJ = 8, NT = TK * TJ;

// double-float accumulator: the sum is hi + lo
struct Acc {
    float hi = 0.f, lo = 0.f;
};

__device__ __forceinline__ void acc_add(Acc& a, float x)
{
    float s = __fadd_rn(a.hi, x);
    float bp = __fsub_rn(s, a.hi);
    float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, err);
}

__device__ __forceinline__ void acc_prod(Acc& a, float x, float y)
{
    float p = __fmul_rn(x, y);
    float pe = __fmaf_rn(x, y, -p);   // exact low part of x*y
    acc_add(a, p);
    a.lo = __fadd_rn(a.lo, pe);
}

__device__ __forceinline__ double acc_value(const Acc& a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }

template <bool FIRST>
__global__ void __launch_bounds__(NT) k_pass_a(Geo g, ViewF A, int CI, const float* __restrict__ z,
                                                const float* __restrict__ pold, float* __restrict__ pnew,
                                                float* __restrict__ q, double* partials, unsigned* counter,
                                                SolverState* st)
{
    constexpr int W = TK + 2, H = TJ + 2, PL = W * H;
    __shared__ float sp[3][PL];
    __shared__ double sm[32];
    if (st->done) return;
    const float beta = FIRST ? 0.f : (float)st->beta;
    const int tk = threadIdx.x, tj = threadIdx.y, tid = tk + TK * tj;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    const int gj = j0 + tj, gk = k0 + tk;
    const bool own = gj < g.ny && gk < g.nz;
    const int opt = (tj + 1) * W + (tk + 1);
    Acc acc;
    for (int P = i0 - 1; P <= i1; ++P) {
        if (P >= 0 && P < g.nx) {
            float* buf = sp[P % 3];
            for (int pt = tid; pt < PL; pt += NT) {
                const int jj = pt / W, kk = pt - jj * W;
                const int j = j0 - 1 + jj, k = k0 - 1 + kk;
                float v = 0.f;
                if (j >= 0 && j < g.ny && k >= 0 && k < g.nz) {
                    const int id = P * g.si + j * g.sj + k;
                    v = FIRST ? z[id] : fmaf(beta, pold[id], z[id]);
                    if (jj >= 1 && jj <= TJ && kk >= 1 && kk <= TK && P >= i0 && P < i1) pnew[id] = v;
                }
                buf[pt] = v;
            }
        }
        __syncthreads();
        const int C = P - 1;
        if (own && C >= i0 && C < i1) {
            const float* cb = sp[C % 3];
            const int id = C * g.si + gj * g.sj + gk;
            const float pc = cb[opt];
            float val;
            if (A.interior(id)) {
                val = A.k.c0 * pc + A.k.x1 * (sp[(C + 2) % 3][opt] + sp[(C + 1) % 3][opt]) +
                      A.k.y1 * (cb[opt - W] + cb[opt + W]) + A.k.z1 * (cb[opt - 1] + cb[opt + 1]);
            } else {
                CoefF a = A.at(id);
                val = a.c * pc;
                if (C > 0) val += a.w * sp[(C + 2) % 3][opt];
                if (C < g.nx - 1) val += a.e * sp[(C + 1) % 3][opt];
                if (gj > 0) val += a.s * cb[opt - W];
                if (gj < g.ny - 1) val += a.n * cb[opt + W];
                if (gk > 0) val += a.b * cb[opt - 1];
                if (gk < g.nz - 1) val += a.t * cb[opt + 1];
            }
            q[id] = val;
            acc_prod(acc, pc, val);
        }
        __syncthreads();
    }
    double v[1] = {acc_value(acc)};
    if (last_block_sum<1>(v, partials, counter, sm)) {
        if (tid == 0) st->alpha = st->rho / v[0];
    }
}

struct ChebF {
    float a0;
    float a[8], b[8];
};

template <int S>
struct BSmem {
    static constexpr int W = TK + 2 * S, H = TJ + 2 * S, PL = W * H;
    // r' ring (S+1 planes), z_k rings (3 planes each, k = 0..S-1), pc_k rings
    // (2 planes each, k = 1..S-1)
    static constexpr int FLOATS = (S + 1) * PL + 3 * S * PL + 2 * (S > 1 ? S - 1 : 0) * PL;
    static constexpr size_t BYTES = sizeof(float) * (size_t)FLOATS;
};

// S = 0: Jacobi (z = r'/A_c, no stencil levels).
template <int S, bool FIRST>
__global__ void __launch_bounds__(NT) k_pass_b(Geo g, ViewF A, int CI, ChebF cf, const float* __restrict__ r_in,
                                                float* __restrict__ r_out, const float* __restrict__ q,
                                                const float* __restrict__ p, float* __restrict__ e,
                                                float* __restrict__ z_out, double* partials, unsigned* counter,
                                                SolverState* st, SolverState* outer, int total_cap)
{
    using SM = BSmem<S>;
    constexpr int W = SM::W, H = SM::H, PL = SM::PL;
    extern __shared__ float dsm[];
    __shared__ double sm[64];
    if (st->done) return;
    float* rp = dsm;                               // [(S+1)][PL]
    float* zr = rp + (S + 1) * PL;                 // [S][3][PL]
    float* pcr = zr + 3 * S * PL;                  // [S-1][2][PL]
    const float alpha = FIRST ? 0.f : (float)st->alpha;
    const int tid = threadIdx.x + TK * threadIdx.y;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int i0 = blockIdx.z * CI, i1 = imin(g.nx, i0 + CI);
    Acc arr, arz;
    for (int I = i0 - S; I < i1 + S; ++I) {
        // ---- level 0 at plane I: r' = r - alpha q over tile + S halo
        if (I >= 0 && I < g.nx && I < i1 + S) {
            float* rpl = rp + (I % (S + 1)) * PL;
            for (int pt = tid; pt < PL; pt += NT) {
                const int jj = pt / W, kk = pt - jj * W;
                const int j = j0 - S + jj, k = k0 - S + kk;
                if (j < 0 || j >= g.ny || k < 0 || k >= g.nz) continue;
                const int id = I * g.si + j * g.sj + k;
                const float rold = r_in[id];
                const float rv = FIRST ? rold : fmaf(-alpha, q[id], rold);
                rpl[pt] = rv;
                const bool center = jj >= S && jj < S + TJ && kk >= S && kk < S + TK && I >= i0 && I < i1;
                if (S > 0) zr[(I % 3) * PL + pt] = cf.a0 * rv;
                if (center) {
                    r_out[id] = rv;
                    e[id] = FIRST ? 0.f : fmaf(alpha, p[id], e[id]);
                    acc_prod(arr, rv, rv);
                    if (S == 0) {
                        const float zv = rv * A.inv_diag(id);
                        z_out[id] = zv;
                        acc_prod(arz, rv, zv);
                    }
                }
            }
        }
        __syncthreads();
        // ---- Chebyshev levels k = 1..S at plane I-k
#pragma unroll
        for (int lv = 1; lv <= S; ++lv) {
            const int Pk = I - lv;
            if (Pk >= imax(0, i0 - S + lv) && Pk < imin(g.nx, i1 + S - lv)) {
                const int Wk = W - 2 * lv, Hk = H - 2 * lv, PLk = Wk * Hk;
                const float* zc = zr + ((lv - 1) * 3 + Pk % 3) * PL;
                const float* zw = zr + ((lv - 1) * 3 + (Pk + 2) % 3) * PL;
                const float* ze = zr + ((lv - 1) * 3 + (Pk + 1) % 3) * PL;
                const float* rpl = rp + (Pk % (S + 1)) * PL;
                const float* pcp = lv >= 2 ? pcr + ((lv - 2) * 2 + Pk % 2) * PL : rpl;
                for (int qq = tid; qq < PLk; qq += NT) {
                    const int jj = lv + qq / Wk, kk = lv + qq % Wk;
                    const int j = j0 - S + jj, k = k0 - S + kk;
                    if (j < 0 || j >= g.ny || k < 0 || k >= g.nz) continue;
                    const int pt = jj * W + kk;
                    const int id = Pk * g.si + j * g.sj + k;
                    const float zcv = zc[pt];
                    float az;
                    if (A.interior(id)) {   // all six neighbours present, base coefficients
                        az = A.k.c0 * zcv + A.k.x1 * (zw[pt] + ze[pt]) + A.k.y1 * (zc[pt - W] + zc[pt + W]) +
                             A.k.z1 * (zc[pt - 1] + zc[pt + 1]);
                    } else {
                        CoefF a = A.at(id);
                        az = a.c * zcv;
                        if (Pk > 0) az += a.w * zw[pt];
                        if (Pk < g.nx - 1) az += a.e * ze[pt];
                        if (j > 0) az += a.s * zc[pt - W];
                        if (j < g.ny - 1) az += a.n * zc[pt + W];
                        if (k > 0) az += a.b * zc[pt - 1];
                        if (k < g.nz - 1) az += a.t * zc[pt + 1];
                    }
                    const float rv = rpl[pt];
                    const float res = rv - az;
                    const float pck = fmaf(cf.b[lv - 1], pcp[pt], res);
                    const float zk = fmaf(cf.a[lv - 1], pck, zcv);
                    if (lv < S) {
                        zr[(lv * 3 + Pk % 3) * PL + pt] = zk;
                        pcr[((lv - 1) * 2 + Pk % 2) * PL + pt] = pck;
                    } else if (jj >= S && jj < S + TJ && kk >= S && kk < S + TK && Pk >= i0 && Pk < i1) {
                        z_out[id] = zk;
                        acc_prod(arz, rv, zk);
                    }
                }
            }
            __syncthreads();
        }
    }
    double v[2] = {acc_value(arr), acc_value(arz)};
    if (last_block_sum<2>(v, partials, counter, sm)) {
        if (tid == 0) {
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
les_status launch_b(les_ctx* c, bool first, dim3 gr, ViewF A, int CI, const ChebF& cf, const float* rin,
                    float* rout, const float* q, const float* p, float* e, float* z, SolverState* in,
                    SolverState* out, int cap)
{
    const size_t bytes = BSmem<S>::BYTES;
    auto kf = first ? k_pass_b<S, true> : k_pass_b<S, false>;
    if (bytes > 48 * 1024) {
        les_status st = check_cuda(c, cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                                   "smem attribute");
        if (st) return st;
    }
    cudaEvent_t e1 = nullptr;
    if (c->prof_on) prof_begin(c, PROF_IN_CHEB, &e1);
    kf<<<gr, dim3(TK, TJ), bytes, c->stream>>>(c->g, A, CI, cf, rin, rout, q, p, e, z, c->partials, c->counters + 14,
                                               in, out, cap);
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return LES_OK;
}

}  // namespace

namespace les {

bool fused_supported(const les_pcg_opts* o)
{
    if (o->precond == LES_PC_JACOBI) return true;
    return o->precond == LES_PC_CHEBYSHEV && o->degree >= 2 && o->degree <= 7;
}

// One inner FP32 solve A e = r (e from 0) with the fused passes.  r0 holds
// the right-hand side on entry and is used as scratch.
les_status inner_solve_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out,
                             int inner_cap)
{
    const Geo& g = c->g;
    const int S = o->precond == LES_PC_JACOBI ? 0 : o->degree - 1;
    ChebF cf{};
    if (S > 0) {
        const double d = (o->lambda_max + o->lambda_min) / 2.0;
        const double cc = (o->lambda_max - o->lambda_min) / 2.0;
        double alpha = 2.0 / d;
        cf.a0 = (float)alpha;
        for (int k = 1; k <= S; ++k) {
            const double beta = (cc * alpha / 2.0) * (cc * alpha / 2.0);
            alpha = 1.0 / (d - beta);
            cf.a[k - 1] = (float)alpha;
            cf.b[k - 1] = (float)beta;
        }
    }
    float* r[2] = {c->f[0], c->f[6]};
    float *z = c->f[1], *pb[2] = {c->f[2], c->f[3]}, *q = c->f[4], *e = c->f[5];
    // chunk lengths along i chosen so that each pass fills about one wave of
    // resident blocks (longer chunks amortise the i-halo of the march)
    const int tiles = ((g.nz + TK - 1) / TK) * ((g.ny + TJ - 1) / TJ);
    auto chunk = [&](const void* fn, size_t smem, int min_ci) {
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, NT, smem);
        int chunks = (occ < 1 ? 1 : occ) * c->sms / tiles;
        if (chunks < 1) chunks = 1;
        int ci = (g.nx + chunks - 1) / chunks;
        return ci < min_ci ? min_ci : ci;
    };
    size_t smem_b = 0;
    const void* fb = nullptr;
    switch (S) {
    case 0: smem_b = BSmem<0>::BYTES; fb = (const void*)k_pass_b<0, false>; break;
    case 1: smem_b = BSmem<1>::BYTES; fb = (const void*)k_pass_b<1, false>; break;
    case 2: smem_b = BSmem<2>::BYTES; fb = (const void*)k_pass_b<2, false>; break;
    case 3: smem_b = BSmem<3>::BYTES; fb = (const void*)k_pass_b<3, false>; break;
    case 4: smem_b = BSmem<4>::BYTES; fb = (const void*)k_pass_b<4, false>; break;
    case 5: smem_b = BSmem<5>::BYTES; fb = (const void*)k_pass_b<5, false>; break;
    default: smem_b = BSmem<6>::BYTES; fb = (const void*)k_pass_b<6, false>; break;
    }
    if (smem_b > 48 * 1024)
        cudaFuncSetAttribute(fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
    const int CIA = chunk((const void*)k_pass_a<false>, 0, 8);
    const int CIB = chunk(fb, smem_b, 4 * S > 8 ? 4 * S : 8);
    const dim3 ga((g.nz + TK - 1) / TK, (g.ny + TJ - 1) / TJ, (g.nx + CIA - 1) / CIA);
    const dim3 gb((g.nz + TK - 1) / TK, (g.ny + TJ - 1) / TJ, (g.nx + CIB - 1) / CIB);
    auto pass_b = [&](bool first, const float* rin, float* rout, const float* p) -> les_status {
        switch (S) {
        case 0: return launch_b<0>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        case 1: return launch_b<1>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        case 2: return launch_b<2>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        case 3: return launch_b<3>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        case 4: return launch_b<4>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        case 5: return launch_b<5>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        default: return launch_b<6>(c, first, gb, A, CIB, cf, rin, rout, q, p, e, z, in, out, o->max_iter);
        }
    };
    int rc = 0;
    les_status st = pass_b(true, r[0], r[1], pb[0]);   // z = M^-1 r, rho, e = 0
    if (st) return st;
    rc = 1;
    int pc = 0, launched = 0, batch = 4;
    for (;;) {
        for (int it = 0; it < batch; ++it) {
            auto ka = (launched + it == 0) ? k_pass_a<true> : k_pass_a<false>;
            launch_p(c, PROF_IN_SPMV, ka, ga, dim3(TK, TJ), g, A, CIA, (const float*)z, (const float*)pb[pc],
                     pb[pc ^ 1], q, c->partials, c->counters + 15, in);
            pc ^= 1;
            st = pass_b(false, r[rc], r[rc ^ 1], pb[pc]);
            if (st) return st;
            rc ^= 1;
        }
        launched += batch;
        st = check_launch(c, "fused inner iteration");
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        if (c->h_state[1].done || launched >= inner_cap) break;
        batch = batch < 32 ? batch * 2 : 32;
    }
    return LES_OK;
}

}  // namespace les
