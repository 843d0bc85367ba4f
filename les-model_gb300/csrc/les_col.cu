// les_col.cu -- the FP32 inner PCG iteration of the mixed-precision solve as
// two register-resident column marches (Jacobi or Chebyshev preconditioner).
//
// Each warp owns a strip of the grid, 32 consecutive cells along k (one per
// lane) by H rows along j, and marches along i over a chunk of planes.  A lane
// keeps its own column of values in registers for the planes a stencil needs:
// the i and j neighbours of a cell are registers of the same thread and the k
// neighbours come from the adjacent lanes by warp shuffle.  There is no shared
// memory and no block barrier inside the march; every warp runs on its own.
//
// Pass A (k_col_a), halo 1:
//     convergence test on ||r'||, beta, rho   (from pass B's sums)
//     p = z + beta p_old          (strip + halo)
//     e += alpha_prev p_old       (the previous iteration's update of the inner
//                                  solution, deferred to here so that pass B
//                                  reads neither p nor e)
//     q = A p, p.q                (left for pass B)
// Pass B (k_col_b), halo S:
//     alpha                       (from pass A's sum)
//     r' = r - alpha q, ||r'||^2
//     z = M^-1 r': Chebyshev with S = degree-1 stencil levels (the polynomial
//       of les-model src/pressure.cpp:871-905 in three-term form, ColCheb),
//       temporally blocked along i -- at march step I level k works on plane
//       I-k over the strip grown by S-k cells; Jacobi (S = 0): z = r' / A_c
//     r'.z                        (left for pass A)
// The grid sums of one pass are formed by the next (the deferred form below;
// the batched ensemble kernels reduce at the end of their own pass).  The
// last p and alpha of a solve are left for col_x_update (x += e + alpha p).
//
// Compulsory bytes per cell and iteration: pass A reads z, p_old, e and writes
// p, q, e (24 B); pass B reads r, q and writes r', z (16 B).
//
// The matrix.  These passes serve the device-built matrix of a solid-free mask
// (the reference builds the pressure matrix before it applies the obstacle,
// src/main.cpp:66-81), whose coefficients depend only on the position
// (src/pressure.cpp:613-696): the base 7-point Laplacian; at the inlet plane
// (i = 0) and at the j and k walls the missing neighbour's coefficient is
// moved onto the opposite one (a Neumann mirror); the plane before the outlet
// (i = nx-2) has no east coefficient; the outlet plane (i = nx-1) is an
// identity row.  The march realises the mirrors by loading reflected
// neighbours into the halo (row -m reads row m, plane -m reads plane m, and so
// on): the reflected field stays mirror-symmetric through every Chebyshev
// level, so each cell uses the interior formula and only the two outlet
// planes need plane-uniform coefficients.  Halo cells of a strip are
// recomputed by every strip that needs them (values of lanes and rows past
// the shrinking halo are never used).
#include "les_col_march.cuh"

namespace {

// x += e + alpha p_last (FP64 solution, FP32 correction)
__global__ void k_x_update(Geo g, double* __restrict__ x, const float* __restrict__ e, const float* __restrict__ p0,
                           const float* __restrict__ p1, const SolverState* in)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    const float a = (float)in->alpha;
    const float* p = in->buf ? p1 : p0;
    x[t] = __dadd_rn(x[t], (double)fmaf(a, p[t], e[t]));
}

// ---- batched over the cases of an ensemble ------------------------------------
// Each block finds its case from the prefix of block starts and runs the
// single-case body on that case's block range; blocks of a case whose inner
// solve is done leave at once.  (Pass A runs 3 blocks per SM here: the case's
// fields take registers that the single-case kernel reads from its
// parameters, and 4 blocks would spill.)
template <int TJ, bool FIRST>
__global__ void __launch_bounds__(CTB, TJ == 8 ? 3 : 2) k_col_a_batch(const BatchCase* __restrict__ cs,
                                                                   const int* __restrict__ pre, int n, int pc)
{
    const int c = batch_case(pre, n, blockIdx.x);
    const BatchCase& C = cs[c];
    const int b0 = __ldg(pre + c), nb = __ldg(pre + c + 1) - b0;
    col_a<0, TJ, FIRST, false, false>(C.g, C.ma, Coef{C.c0, C.x1, C.y1, C.z1}, C.z, pc ? C.p1 : C.p0, pc ? C.p0 : C.p1, C.q,
                            C.e, C.partials, C.counters + 15, C.in, pc ^ 1, blockIdx.x - b0, nb, Defer{}, C.out,
                            C.cap);
}

template <int S, int TJ, bool FIRST>
__global__ void __launch_bounds__(CTB, blocks4_b(S, TJ)) k_col_b_batch(const BatchCase* __restrict__ cs,
                                                                               const int* __restrict__ pre, int n,
                                                                               int rin)
{
    const int c = batch_case(pre, n, blockIdx.x);
    const BatchCase& C = cs[c];
    const int b0 = __ldg(pre + c), nb = __ldg(pre + c + 1) - b0;
    col_b<0, S, TJ, FIRST, false, false>(C.g, C.mb, C.c3, C.inv_c0, rin ? C.r1 : C.r0, rin ? C.r0 : C.r1, C.q, C.z, C.partials,
                               C.counters + 14, C.in, C.out, C.cap, blockIdx.x - b0, nb, Defer{});
}

// x += e + alpha p_last for the cases in their correction round
__global__ void k_x_update_batch(const BatchCase* __restrict__ cs, const int* __restrict__ pre, int n)
{
    const int c = batch_case(pre, n, blockIdx.x);
    const BatchCase& C = cs[c];
    if (!C.act) return;
    const int t = (blockIdx.x - __ldg(pre + c)) * blockDim.x + threadIdx.x;
    if (t >= C.g.n) return;
    const float a = (float)C.in->alpha;
    const float* p = C.in->buf ? C.p1 : C.p0;
    C.x[t] = __dadd_rn(C.x[t], (double)fmaf(a, p[t], C.e[t]));
}

// ---- launch plumbing ----------------------------------------------------------
// the kernels for row stride sj (0: the runtime-stride instance)
KA pick_a(int sj, int tj, bool first)
{
    switch (sj) {
    case 32: return col_pick_a_sj32(tj, first);
    case 64: return col_pick_a_sj64(tj, first);
    case 128: return col_pick_a_sj128(tj, first);
    case 256: return col_pick_a_sj256(tj, first);
    default: return pick_a_t<0>(tj, first);
    }
}

KB pick_b(int sj, int S, int tj, bool first)
{
    switch (sj) {
    case 32: return col_pick_b_sj32(S, tj, first);
    case 64: return col_pick_b_sj64(S, tj, first);
    case 128: return col_pick_b_sj128(S, tj, first);
    case 256: return col_pick_b_sj256(S, tj, first);
    default: return pick_b_t<0>(S, tj, first);
    }
}

int stride_of(const les_ctx* c) { return c->col_stride ? c->g.sj : 0; }

int default_tj_b(int S) { return S == 0 ? 16 : (S <= 3 ? 8 : 4); }

bool valid_tj_b(int S, int tj)
{
    if (S == 0) return tj == 16;
    if (S <= 3) return tj == 4 || tj == 8;
    return tj == 4;
}

int threads_a(int tj) { return col_threads(blocks4_a(tj)); }
int threads_b(int S, int tj) { return col_threads(blocks4_b(S, tj)); }

// Strips x chunks for one pass: as many chunks along i as fit in one wave of
// resident warps (a partial second wave would double the pass time); a
// chunk re-reads 2 x halo planes.
ColMap col_map(les_ctx* c, const void* fn, int threads, int halo, int tj, int ci_force)
{
    const Geo& g = c->g;
    ColMap m{};
    m.tk = 32 - 2 * halo;
    m.tj = tj;
    m.tiles_k = (g.nz + m.tk - 1) / m.tk;
    m.tiles_j = (g.ny + tj - 1) / tj;
    const int tiles = m.tiles_k * m.tiles_j;
    int ci = ci_force;
    if (ci <= 0) {
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, 0);
        const double share = c->share > 0 && c->share <= 1 ? c->share : 1.0;
        const long long warps = (long long)((occ < 1 ? 1 : occ) * (threads / 32) * c->sms * share);
        long long chunks = warps / tiles;
        if (chunks < 1) chunks = 1;
        ci = (int)((g.nx + chunks - 1) / chunks);
        const int min_ci = 2 * halo > 4 ? 2 * halo : 4;
        if (ci < min_ci) ci = min_ci;
    }
    if (ci > g.nx) ci = g.nx;
    m.ci = ci;
    m.items = tiles * ((g.nx + ci - 1) / ci);
    return m;
}

}  // namespace

namespace les {

ColCheb col_cheb(const les_pcg_opts* o, float c0f, float x1f, float y1f, float z1f)
{
    ColCheb t{};
    const int S = o->precond == LES_PC_CHEBYSHEV ? o->degree - 1 : 0;
    if (S <= 0) return t;
    // a_k, b_k as the reference's recurrence forms them (src/pressure.cpp:878-899)
    const double d = (o->lambda_max + o->lambda_min) / 2.0, cw = (o->lambda_max - o->lambda_min) / 2.0;
    const double c0 = c0f, x1 = x1f, y1 = y1f, z1 = z1f, a0 = 2.0 / d;
    double ap = a0;   // a_{k-1}
    for (int k = 1; k <= S && k <= 6; ++k) {
        const double b = (cw * ap / 2.0) * (cw * ap / 2.0);
        const double a = 1.0 / (d - b);
        const double gk = a * b / ap;
        const double sc = k == 1 ? a0 : 1.0;   // level 1 applies its stencil to r'
        double cc = sc * (1.0 + gk) - a * sc * c0, ci = sc * (1.0 + gk) - a * sc;
        double rr = a, gg = -gk;
        if (k == 1) { cc += a; ci += a; rr = 0.0; gg = 0.0; }   // r' is the centre value
        if (k == 2) { rr = a - gk * a0; gg = 0.0; }            // z_0 = a0 r' at the centre
        t.cc[k - 1] = (float)cc;
        t.ci[k - 1] = (float)ci;
        t.cx[k - 1] = (float)(-a * sc * x1);
        t.cy[k - 1] = (float)(-a * sc * y1);
        t.cz[k - 1] = (float)(-a * sc * z1);
        t.rr[k - 1] = (float)rr;
        t.gg[k - 1] = (float)gg;
        ap = a;
    }
    return t;
}

bool col_supported(const les_ctx* c, const les_pcg_opts* o)
{
    if (!(c->fused == 1 && !c->opt_tma && c->stencil_mode == 1 && c->code_plain && fused_supported(o))) return false;
    // the reflections need the mirrored rows, columns and planes inside the grid
    const int S = o->precond == LES_PC_JACOBI ? 1 : (o->degree - 1 > 1 ? o->degree - 1 : 1);
    const Geo& g = c->g;
    return g.nx >= 2 * S + 4 && g.ny >= 2 * S + 2 && g.nz >= 2 * S + 2;
}

les_status col_plan(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out, ColPlan& P)
{
    P.S = o->precond == LES_PC_JACOBI ? 0 : o->degree - 1;
    P.c3 = col_cheb(o, A.k.c0, A.k.x1, A.k.y1, A.k.z1);
    P.inv_c0 = 1.f / A.k.c0;
    P.A = A;
    P.in = in;
    P.out = out;
    P.cap = o->max_iter;
    const int tja = (c->tune_tja == 8 || c->tune_tja == 16) ? c->tune_tja : 8;
    const int tjb = valid_tj_b(P.S, c->tune_tjb) ? c->tune_tjb : default_tj_b(P.S);
    const int wa = threads_a(tja) / 32, wb = threads_b(P.S, tjb) / 32;
    const int sj = stride_of(c);
    P.ma = col_map(c, (const void*)pick_a(sj, tja, false), threads_a(tja), 1, tja, c->tune_cia);
    P.mb = col_map(c, (const void*)pick_b(sj, P.S, tjb, false), threads_b(P.S, tjb), P.S, tjb, c->tune_cib);
    P.blocks_a = (P.ma.items + wa - 1) / wa;
    P.blocks_b = (P.mb.items + wb - 1) / wb;
    // pass B's partials (2 per block) then pass A's, both live across a pass
    if ((size_t)2 * P.blocks_b + (size_t)P.blocks_a > c->partials_len)
        return fail(c, LES_BAD_ARG, "column pass grid exceeds the reduction scratch");
    return LES_OK;
}

static Coef coef_of(const ColPlan& P) { return Coef{P.A.k.c0, P.A.k.x1, P.A.k.y1, P.A.k.z1}; }

les_status col_pass_a(les_ctx* c, const ColPlan& P, bool first, int pc)
{
    float *z = c->f[1], *pb[2] = {c->f[2], c->f[3]}, *q = c->f[4], *e = c->f[5];
    float2* const part = reinterpret_cast<float2*>(c->partials);   // pass B's pairs, then pass A's
    const Defer df{part, P.blocks_b, part + 2 * (size_t)P.blocks_b};
    launch_pdl(c, PROF_IN_SPMV, pick_a(stride_of(c), P.ma.tj, first), P.blocks_a, threads_a(P.ma.tj), c->g, P.ma, coef_of(P), (const float*)z,
             (const float*)pb[pc], pb[pc ^ 1], q, e, c->partials, c->counters + 15, P.in, pc ^ 1, df, P.out, P.cap);
    return check_launch(c, "column pass A");
}

les_status col_pass_b(les_ctx* c, const ColPlan& P, bool first, int rin)
{
    float* r[2] = {c->f[0], c->f[6]};
    float *z = c->f[1], *q = c->f[4];
    float2* const part = reinterpret_cast<float2*>(c->partials);
    const Defer df{part + 2 * (size_t)P.blocks_b, P.blocks_a, part};
    launch_pdl(c, PROF_IN_CHEB, pick_b(stride_of(c), P.S, P.mb.tj, first), P.blocks_b, threads_b(P.S, P.mb.tj), c->g, P.mb, P.c3, P.inv_c0,
             (const float*)r[rin], r[rin ^ 1], (const float*)q, z, c->partials, c->counters + 14, P.in, P.out, P.cap,
             df);
    return check_launch(c, "column pass B");
}

// ---- batched passes ------------------------------------------------------------
using KAB = void (*)(const BatchCase*, const int*, int, int);

static KAB pick_a_batch(bool first) { return first ? k_col_a_batch<8, true> : k_col_a_batch<8, false>; }

static KAB pick_b_batch(int S, bool first)
{
#define LES_BB(s, t) return first ? k_col_b_batch<s, t, true> : k_col_b_batch<s, t, false>
    switch (S) {
    case 0: LES_BB(0, 16);
    case 1: LES_BB(1, 8);
    case 2: LES_BB(2, 8);
    case 3: LES_BB(3, 8);
    case 4: LES_BB(4, 4);
    case 5: LES_BB(5, 4);
    default: LES_BB(6, 4);
    }
#undef LES_BB
}

int col_batch_tj_b(int S) { return default_tj_b(S); }

int col_batch_warps_per_block() { return CWPB_B; }

ColMap col_batch_map(les_ctx* c, int pass, int S, int chunk_planes)
{
    if (pass == 0) return col_map(c, (const void*)pick_a_batch(false), CTB, 1, 8, chunk_planes);
    return col_map(c, (const void*)pick_b_batch(S, false), CTB, S, default_tj_b(S), chunk_planes);
}

int col_batch_resident_warps(int pass, int S)
{
    int occ = 1, dev = 0, sms = 1;
    const void* fn = pass == 0 ? (const void*)pick_a_batch(false) : (const void*)pick_b_batch(S, false);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, CTB, 0);
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (occ < 1 ? 1 : occ) * CWPB_B * sms;
}

les_status col_batch_pass_a(cudaStream_t s, bool first, int pc, const BatchCase* cs, const int* pre, int n,
                            int blocks)
{
    pick_a_batch(first)<<<blocks, CTB, 0, s>>>(cs, pre, n, pc);
    return cudaPeekAtLastError() == cudaSuccess ? LES_OK : LES_CUDA_ERROR;
}

les_status col_batch_pass_b(cudaStream_t s, int S, bool first, int rin, const BatchCase* cs, const int* pre, int n,
                            int blocks)
{
    pick_b_batch(S, first)<<<blocks, CTB, 0, s>>>(cs, pre, n, rin);
    return cudaPeekAtLastError() == cudaSuccess ? LES_OK : LES_CUDA_ERROR;
}

les_status col_batch_x_update(cudaStream_t s, const BatchCase* cs, const int* pre, int n, int blocks)
{
    k_x_update_batch<<<blocks, 256, 0, s>>>(cs, pre, n);
    return cudaPeekAtLastError() == cudaSuccess ? LES_OK : LES_CUDA_ERROR;
}

les_status col_x_update(les_ctx* c)
{
    const Geo& g = c->g;
    launch(c, k_x_update, (g.n + 255) / 256, 256, g, c->slot[LES_P], (const float*)c->f[5], (const float*)c->f[2],
           (const float*)c->f[3], (const SolverState*)(c->state + 1));
    return check_launch(c, "solution update");
}

}  // namespace les
