// les_col_march.cuh -- device code of the register-column marches (the FP32
// inner PCG iteration, les_col.cu), templated on the row stride.
//
// The row offsets of a strip are multiples of the row stride (nz cells).
// With the stride a compile-time constant they become immediate offsets of
// the loads and stores, which takes most of the address arithmetic out of
// the marches (256x128x128 mixed step: 148.7 -> 169.0 Mcell-steps/s); the
// kernels are therefore compiled for the common strides 32, 64, 128 and 256,
// one translation unit each (les_col_sjN.cu), and once for a stride read at
// run time (SJF = 0, les_col.cu).  Every instance does the same arithmetic in
// the same order: the results do not depend on which one runs.
#pragma once
#include <cmath>
#include <type_traits>

#include "les_internal.cuh"
#include "les_mixed.cuh"

namespace les {

struct Coef {
    float c0, x1, y1, z1;
};

struct Defer {
    const float2* pin;   // the previous pass's block partials, (hi, lo) pairs
    int nb_in;           // blocks of the previous pass
    float2* pout;        // this pass's block partials
};

using KA = void (*)(Geo, ColMap, Coef, const float*, const float*, float*, float*, float*, double*, unsigned*,
                    SolverState*, int, Defer, SolverState*, int);
using KB = void (*)(Geo, ColMap, ColCheb, float, const float*, float*, const float*, float*, double*, unsigned*,
                    SolverState*, SolverState*, int, Defer);

// the kernels of the compiled strides (tj rows per strip, S levels)
KA col_pick_a_sj32(int tj, bool first);
KA col_pick_a_sj64(int tj, bool first);
KA col_pick_a_sj128(int tj, bool first);
KA col_pick_a_sj256(int tj, bool first);
KB col_pick_b_sj32(int S, int tj, bool first);
KB col_pick_b_sj64(int S, int tj, bool first);
KB col_pick_b_sj128(int S, int tj, bool first);
KB col_pick_b_sj256(int S, int tj, bool first);

}  // namespace les

using namespace les;

namespace {

// Block shapes.  A pass's deferred head sums every block partial of the
// pass before it, so fewer, larger blocks make the head cheaper: a
// single-case kernel that fits 4-warp blocks on an SM in a multiple of four
// runs 16-warp blocks, in a multiple of two 8-warp blocks (256x128x128:
// 146.3 Mcell-steps/s with 4-warp blocks, 149.1 with 8; pass A in 16-warp
// blocks: 167.7 -> 168.5; 512x256x256 unchanged within 0.7 %).  The batched
// kernels sum their partials in a separate kernel and keep 4 warps.
constexpr int col_threads(int blocks4) { return blocks4 % 4 == 0 ? 512 : (blocks4 % 2 == 0 ? 256 : 128); }
constexpr int col_blocks(int blocks4) { return blocks4 % 4 == 0 ? blocks4 / 4 : (blocks4 % 2 == 0 ? blocks4 / 2 : blocks4); }
constexpr int blocks4_a(int TJ) { return TJ == 8 ? 4 : 2; }               // 4-warp blocks per SM
constexpr int blocks4_b(int S, int TJ) { return (TJ == 4 && S <= 3) ? 3 : 2; }
constexpr int CTB = 128;          // batched kernels: threads per block
constexpr int CWPB_B = CTB / 32;
constexpr unsigned FULL = 0xffffffffu;


struct StripPos {
    int j0;        // j of row 0
    int i0, i1;    // owned planes [i0, i1)
    int kl;        // this lane's k after reflection at the walls
    unsigned own;  // bit r: cell of row r owned by this lane
    int rows;      // row pattern (RowsMode) of the strip
    bool kown;     // this lane's k is owned
    bool allrows;  // every owned row of the strip is inside the grid: ownership is kown
};

// How the rows of a strip map onto grid rows.  Row r of a strip lies at
// j = j0 + r, reflected into [0, ny) about the wall rows.  The interior
// strips need no reflection; the first strip (j0 = -HALO) reflects about its
// row HALO and, when ny is a multiple of the strip's owned rows, the last
// strip about its row H - HALO - 1: both patterns are known at compile time,
// so these strips fetch as cheaply as the interior ones.  Any other strip
// (a grid only a few strips wide, a ragged last strip) reflects per row.
enum RowsMode { ROWS_PLAIN = 0, ROWS_FIRST = 1, ROWS_LAST = 2, ROWS_ANY = 3 };

// reflected grid row of strip row r, minus j0
template <int MODE, int HALO, int H>
__device__ __forceinline__ int row_rel(int r, int j0, int ny)
{
    if (MODE == ROWS_PLAIN) return r;
    if (MODE == ROWS_FIRST) return (r < HALO ? HALO - r : r - HALO) + HALO;
    if (MODE == ROWS_LAST) {
        constexpr int e = H - HALO - 1;
        return r <= e ? r : 2 * e - r;
    }
    int j = j0 + r;
    j = j < 0 ? -j : j;
    j = min(j, 2 * (ny - 1) - j);
    return max(j, 0) - j0;   // rows beyond one reflection are never used: any row in the grid
}

// calls f(integral_constant<int, mode>) for the strip's row pattern
template <class F>
__device__ __forceinline__ void with_rows(int mode, F&& f)
{
    if (mode == ROWS_PLAIN) f(std::integral_constant<int, ROWS_PLAIN>{});
    else if (mode == ROWS_FIRST) f(std::integral_constant<int, ROWS_FIRST>{});
    else if (mode == ROWS_LAST) f(std::integral_constant<int, ROWS_LAST>{});
    else f(std::integral_constant<int, ROWS_ANY>{});
}

// reflection of index x into [0, n) about the end cells (-1 if still outside)
__device__ __forceinline__ int reflect(int x, int n)
{
    x = x < 0 ? -x : x;
    x = x > n - 1 ? 2 * (n - 1) - x : x;
    return x >= 0 ? x : -1;
}

template <int HALO, int TJ>
__device__ __forceinline__ StripPos strip_pos(const Geo& g, const ColMap& m, int item, int lane)
{
    StripPos s;
    const int kt = item % m.tiles_k, rest = item / m.tiles_k;
    const int jt = rest % m.tiles_j, ch = rest / m.tiles_j;
    const int kg = kt * m.tk - HALO + lane;
    s.j0 = jt * TJ - HALO;
    constexpr int H = TJ + 2 * HALO;
    if (s.j0 >= 0 && s.j0 + H <= g.ny) s.rows = ROWS_PLAIN;
    else if (s.j0 == -HALO && H - HALO <= g.ny) s.rows = ROWS_FIRST;
    else if (s.j0 >= 0 && s.j0 + H == g.ny + HALO) s.rows = ROWS_LAST;
    else s.rows = ROWS_ANY;
    s.i0 = ch * m.ci;
    s.i1 = min(g.nx, s.i0 + m.ci);
    // lanes past one reflection are never used; they read any cell of the grid
    s.kl = max(reflect(kg, g.nz), 0);
    const bool kown = kg >= 0 && kg < g.nz && lane >= HALO && lane < HALO + m.tk;
    s.kown = kown;
    s.allrows = s.j0 + HALO + TJ <= g.ny;
    s.own = 0u;
#pragma unroll
    for (int r = HALO; r < HALO + TJ; ++r)
        if (kown && s.j0 + r < g.ny) s.own |= 1u << r;
    return s;
}

// ---- the grid sums between the passes ------------------------------------------
// Two protocols.  Last block (DEFER = false, the batched ensemble kernels):
// every block leaves its partial sums, and the block that arrives last
// (fence + atomic counter) adds them up and updates the solver state before
// the kernel ends.  Deferred (DEFER = true, the single-case kernels): a pass
// only leaves its block partials; every block of the NEXT pass adds them up
// itself, in the same fixed order, right after its dependency wait, and its
// block 0 writes the state.  The deferred form takes the fence, the atomic
// and the serial final sum off the end of every pass (3.8 us of pass A's and
// 6.6 us of pass B's 57 us iteration at 256x128x128), at the price of a
// parallel sum at the start of the next one.  The decisions stay those of
// the last-block form: pass A of iteration k+1 makes the convergence test on
// ||r_k||, forms beta and rho from pass B's partials and, if the solve ends,
// stores the final state; pass B forms alpha from pass A's partials and
// commits the iteration count and rho.  A block only writes state fields
// that no block of its own kernel reads (rho_next is the rho handed from
// pass A to pass B), so the kernels need no ordering among their blocks.
// Which hand-offs of the single-case kernels are deferred: pass A -> pass B
// (alpha) and pass B -> pass A (beta, the convergence test).
#ifndef COL_DEFER_AB
#define COL_DEFER_AB 1
#endif
#ifndef COL_DEFER_BA
#define COL_DEFER_BA 1
#endif

// Double-float sums on the FP32 pipe (GB300 runs FP64 arithmetic at a small
// fraction of its FP32 rate, and FP64 block sums in every block of a pass
// cost microseconds): the sum of two (hi, lo) pairs by TwoSum of the high
// parts, renormalised; about 48 significant bits, as the per-thread
// accumulators keep.
__device__ __forceinline__ Acc df_add(const Acc& a, const Acc& b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bp = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
    const float lo = __fadd_rn(__fadd_rn(a.lo, b.lo), err);
    Acc r;
    r.hi = __fadd_rn(s, lo);
    r.lo = __fsub_rn(lo, __fsub_rn(r.hi, s));
    return r;
}

// Block sum of NV pairs in a fixed order; the totals in thread 0.
// sm: NV * 32 float2.
template <int NV>
__device__ __forceinline__ void block_sum_df(Acc (&v)[NV], float2* sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            Acc t;
            t.hi = __shfl_down_sync(0xffffffffu, v[q].hi, o);
            t.lo = __shfl_down_sync(0xffffffffu, v[q].lo, o);
            v[q] = df_add(v[q], t);
        }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sm[q * 32 + warp] = make_float2(v[q].hi, v[q].lo);
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const float2 t = lane < nw ? sm[q * 32 + lane] : make_float2(0.f, 0.f);
            v[q].hi = t.x;
            v[q].lo = t.y;
        }
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                Acc t;
                t.hi = __shfl_down_sync(0xffffffffu, v[q].hi, o);
                t.lo = __shfl_down_sync(0xffffffffu, v[q].lo, o);
                v[q] = df_add(v[q], t);
            }
    }
}

// A pass's block partials: block_sum_df, then (hi, lo) at [q * nb + blk].
template <int NV>
__device__ __forceinline__ void put_partials(Acc (&v)[NV], float2* sm, float2* pout, int blk, int nb)
{
    block_sum_df<NV>(v, sm);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) pout[q * nb + blk] = make_float2(v[q].hi, v[q].lo);
}

// Sums NV vectors of nb block partials (thread-strided, then the block
// tree: a fixed order); the totals as doubles in thread 0.
template <int NV>
__device__ __forceinline__ void sum_partials(const float2* __restrict__ part, int nb, double (&v)[NV], float2* sm)
{
    Acc acc[NV];
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const float2 t = __ldcg(part + q * nb + b);
            Acc x;
            x.hi = t.x;
            x.lo = t.y;
            acc[q] = df_add(acc[q], x);
        }
    block_sum_df<NV>(acc, sm);
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = (double)acc[q].hi + (double)acc[q].lo;
}

// The last-block form with the same double-float sums: every block leaves
// its (hi, lo) partials, and the block that arrives last (fence + atomic
// counter) adds them up; true in every thread of that block, the totals in
// its thread 0.
template <int NV>
__device__ bool last_block_sum_df(Acc (&v)[NV], float2* part, unsigned* counter, float2* sm, int bid, int nb,
                                  double (&out)[NV])
{
    __shared__ int am_last;
    block_sum_df<NV>(v, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) part[q * nb + bid] = make_float2(v[q].hi, v[q].lo);
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        am_last = t == (unsigned)nb - 1u;
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    sum_partials<NV>(part, nb, out, sm);
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// The deferred heads of the two passes, kept out of line: inlined, their
// FP64 scalars and barriers changed how the march around them was compiled
// (pass A's march ran 20 % slower).  Both return `end` (leave the kernel:
// the solve is done) in every thread of the block.
struct HeadOut {
    int end;
    float coef;   // pass A: beta; pass B: alpha
};

// Pass A: pass B's sums ||r'||^2, r'.z; the convergence test and the state
// in thread 0 (FP64), block 0 writing.
template <bool FIRST>
__device__ __noinline__ HeadOut head_a(const float2* __restrict__ pin, int nb_in, SolverState* st,
                                       SolverState* outer, int total_cap, int pslot, int blk)
{
    __shared__ double sm[64];
    __shared__ HeadOut so;
    double v[2];
    if (threadIdx.x == 0) so.end = st->done;
    __syncthreads();
    if (so.end) return so;
    __syncthreads();
    sum_partials<2>(pin, nb_in, v, reinterpret_cast<float2*>(sm));
    if (threadIdx.x == 0) {
        const bool w0 = blk == 0;
        int status = -1;
        if (FIRST) {
            if (w0) st->rho_next = v[1];
            so.coef = 0.f;
        } else {
            const double err = sqrt(v[0]), rho_old = st->rho;
            const int kk = st->k, total = outer->iters;   // committed by pass B
            if (err < st->tol) status = LES_OK;
            else if (!isfinite(err)) status = LES_NONFINITE;
            else if (kk >= st->max_iter || total >= total_cap) status = LES_NOT_CONVERGED;
            const bool frozen = st->frozen;
            if (frozen) status = -1;
            const double b = frozen ? 0.0 : v[1] / rho_old;
            so.coef = (float)b;
            if (w0) {
                st->err = err;
                st->beta = b;
                if (status >= 0) {   // the solve ends at iteration kk: the final state
                    st->rho = v[1];
                    st->status = status;
                    st->done = 1;
                } else {
                    st->rho_next = v[1];
                }
            }
        }
        if (w0 && status < 0) st->buf = pslot;   // buffer holding this iteration's p
        so.end = status >= 0;                    // no work after the last iteration
    }
    __syncthreads();
    return so;
}

// Pass B: pass A's sum p.q -> alpha (thread 0, FP64); with pass B's own sums
// deferred too, pass A hands rho over in rho_next and this pass commits the
// iteration, otherwise rho is current and this pass's last block does the
// state at its end.
template <bool BOUT>
__device__ __noinline__ HeadOut head_b(const float2* __restrict__ pin, int nb_in, SolverState* st,
                                       SolverState* outer, int blk)
{
    __shared__ double sm[64];
    __shared__ HeadOut so;
    double v[1];
    if (threadIdx.x == 0) so.end = st->done;
    __syncthreads();
    if (so.end) return so;
    __syncthreads();
    sum_partials<1>(pin, nb_in, v, reinterpret_cast<float2*>(sm));
    if (threadIdx.x == 0) {
        const double rho = BOUT ? st->rho_next : st->rho, a = st->frozen ? 0.0 : rho / v[0];
        so.coef = (float)a;
        if (blk == 0) {
            st->alpha = a;
            if (BOUT) {
                st->rho = rho;
                st->k = st->k + 1;
                outer->iters = outer->iters + 1;
            }
        }
    }
    __syncthreads();
    return so;
}

// ---- pass A -----------------------------------------------------------------
// blk / nblk: this block among the blocks of the pass (one case's blocks in
// a batched launch)
template <int SJF, int TJ, bool FIRST, bool AIN, bool AOUT>
__device__ __forceinline__ void col_a(const Geo& g, const ColMap& m, const Coef& k, const float* __restrict__ z,
                                      const float* __restrict__ pold, float* __restrict__ pnew, float* __restrict__ q,
                                      float* __restrict__ e, double* partials, unsigned* counter, SolverState* st,
                                      int pslot, int blk, int nblk, const Defer& df, SolverState* outer, int total_cap)
{
    constexpr int H = TJ + 2;
    __shared__ double sm[64];
    const int lane = threadIdx.x & 31;
    const int item = blk * (int)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const StripPos s = strip_pos<1, TJ>(g, m, item, lane);   // from the arguments only
    const int SJ = SJF ? SJF : g.sj, SI = g.si;   // row and plane strides
    dep_wait();
    float beta = 0.f;
    if (AIN) {   // pass B's sums, the decision and the state
        const HeadOut h = head_a<FIRST>(df.pin, df.nb_in, st, outer, total_cap, pslot, blk);
        if (h.end) return;
        beta = h.coef;
    } else {
        if (st->done) return;
        if (!FIRST) beta = (float)st->beta;
    }
    const float aprev = FIRST ? 0.f : (float)st->alpha;
    if (!AIN && AOUT && blk == 0 && threadIdx.x == 0) st->buf = pslot;   // buffer holding this iteration's p
    Acc acc;
    if (item < m.items) {
        float p0[H], p1[H], p2[H];   // p at planes P, P-1, P-2
        float vz[H], vp[H], ve[TJ];  // z, p_old, e of the plane being fetched
#pragma unroll
        for (int r = 0; r < H; ++r) p0[r] = p1[r] = p2[r] = 0.f;
        auto fetch = [&](int P) {
            const bool pown = P >= s.i0 && P < s.i1;
            const int pl = P < 0 ? -P : P;   // plane -m reads plane m
            if (pl >= g.nx) {                // planes past the outlet are not read
#pragma unroll
                for (int r = 0; r < H; ++r) vz[r] = vp[r] = 0.f;
                return;
            }
            // e only on owned planes (its values on cells this lane does not
            // own are never used)
            const int base = pl * SI + s.j0 * SJ + s.kl;
            if (s.rows == ROWS_PLAIN) {
                int id = base;
#pragma unroll
                for (int r = 0; r < H; ++r, id += SJ) {
                    vz[r] = z[id];
                    vp[r] = FIRST ? 0.f : pold[id];
                    if (r >= 1 && r <= TJ) ve[r - 1] = (!FIRST && pown) ? e[id] : 0.f;
                }
                return;
            }
            with_rows(s.rows, [&](auto md) {
                constexpr int MD = decltype(md)::value;
#pragma unroll
                for (int r = 0; r < H; ++r) {
                    const int id = base + row_rel<MD, 1, H>(r, s.j0, g.ny) * SJ;
                    vz[r] = z[id];
                    vp[r] = FIRST ? 0.f : pold[id];
                    if (r >= 1 && r <= TJ) ve[r - 1] = (!FIRST && pown) ? e[id] : 0.f;
                }
            });
        };
        fetch(s.i0 - 1);
        for (int P = s.i0 - 1; P <= s.i1; ++P) {
#pragma unroll
            for (int r = 0; r < H; ++r) p0[r] = FIRST ? vz[r] : fmaf(beta, vp[r], vz[r]);
            if (P >= s.i0 && P < s.i1) {
                const int base = P * SI + s.j0 * SJ + s.kl;   // owned cells: no reflection
                auto outp = [&](auto all) {
                    constexpr bool AL = decltype(all)::value;
#pragma unroll
                    for (int r = 1; r <= TJ; ++r) {
                        if (AL ? s.kown : ((s.own >> r) & 1u)) {
                            const int id = base + r * SJ;
                            pnew[id] = p0[r];
                            e[id] = FIRST ? 0.f : fmaf(aprev, vp[r], ve[r - 1]);
                        }
                    }
                };
                if (s.allrows) outp(std::true_type{});
                else outp(std::false_type{});
            }
            if (P < s.i1) fetch(P + 1);
            // q = A p at plane C = P - 1
            const int C = P - 1;
            if (C >= s.i0) {
                const int cb = C * SI + s.j0 * SJ + s.kl;
                // plane-uniform coefficients: the outlet plane is an identity
                // row, the plane before it has no east coefficient
                const bool ident = C == g.nx - 1;
                const float cc = ident ? 1.f : k.c0, cx = ident ? 0.f : k.x1;
                const float ce = (ident || C == g.nx - 2) ? 0.f : k.x1;
                const float cy = ident ? 0.f : k.y1, cz = ident ? 0.f : k.z1;
                float sq = 0.f, qv[TJ + 1];
                // all rows' products first (one basic block), then the owned stores
#pragma unroll
                for (int r = 1; r <= TJ; ++r) {
                    const float pc = p1[r];
                    const float pb = __shfl_up_sync(FULL, pc, 1);
                    const float pt = __shfl_down_sync(FULL, pc, 1);
                    qv[r] = cc * pc + cx * p2[r] + ce * p0[r] + cy * (p1[r - 1] + p1[r + 1]) + cz * (pb + pt);
                }
                auto outq = [&](auto all) {
                    constexpr bool AL = decltype(all)::value;
#pragma unroll
                    for (int r = 1; r <= TJ; ++r) {
                        const bool o = AL ? s.kown : ((s.own >> r) & 1u);
                        if (o) q[cb + r * SJ] = qv[r];
                        sq = fmaf(AL || o ? p1[r] : 0.f, qv[r], sq);
                    }
                    if (AL && !s.kown) sq = 0.f;
                };
                if (s.allrows) outq(std::true_type{});
                else outq(std::false_type{});
                acc_add(acc, sq);
            }
#pragma unroll
            for (int r = 0; r < H; ++r) {
                p2[r] = p1[r];
                p1[r] = p0[r];
            }
        }
    }
    dep_signal();
    if (AOUT) {
        Acc v[1] = {acc};
        put_partials<1>(v, reinterpret_cast<float2*>(sm), df.pout, blk, nblk);
        return;
    }
    Acc va[1] = {acc};
    double v[1];
    if (last_block_sum_df<1>(va, reinterpret_cast<float2*>(partials), counter, reinterpret_cast<float2*>(sm), blk,
                             nblk, v)) {
        if (threadIdx.x == 0) {
            st->alpha = st->frozen ? 0.0 : st->rho / v[0];
            st->buf = pslot;   // buffer holding this iteration's p
        }
    }
}

template <int SJF, int TJ, bool FIRST>
__global__ void __launch_bounds__(col_threads(blocks4_a(TJ)), col_blocks(blocks4_a(TJ))) k_col_a(Geo g, ColMap m, Coef k, const float* __restrict__ z,
                                                             const float* __restrict__ pold, float* __restrict__ pnew,
                                                             float* __restrict__ q, float* __restrict__ e,
                                                             double* partials, unsigned* counter, SolverState* st,
                                                             int pslot, Defer df, SolverState* outer, int total_cap)
{
    col_a<SJF, TJ, FIRST, COL_DEFER_BA, COL_DEFER_AB>(g, m, k, z, pold, pnew, q, e, partials, counter, st, pslot,
                                                  blockIdx.x, gridDim.x, df, outer, total_cap);
}

// ---- pass B -----------------------------------------------------------------
// Grid sums of ||r'||^2 and r'.z; the last block updates the inner state:
// the first pass sets rho, later ones the convergence test, beta and rho.
template <bool FIRST>
__device__ __forceinline__ void pass_b_finish(const Acc& arr, const Acc& arz, double* partials, unsigned* counter,
                                              double* sm, SolverState* st, SolverState* outer, int total_cap,
                                              int blk, int nblk)
{
    Acc va[2] = {arr, arz};
    double v[2];
    if (last_block_sum_df<2>(va, reinterpret_cast<float2*>(partials), counter, reinterpret_cast<float2*>(sm), blk,
                             nblk, v)) {
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
                if (st->frozen) { st->beta = 0.0; return; }   // the autotuner's timing rounds
                if (err < st->tol) { st->done = 1; st->status = LES_OK; }
                else if (!isfinite(err)) { st->done = 1; st->status = LES_NONFINITE; }
                else if (kk >= st->max_iter || total >= total_cap) { st->done = 1; st->status = LES_NOT_CONVERGED; }
                st->beta = v[1] / st->rho;
                st->rho = v[1];
            }
        }
    }
}

template <int SJF, int S, int TJ, bool FIRST, bool BIN, bool BOUT>
__device__ __forceinline__ void col_b(const Geo& g, const ColMap& m, const ColCheb& c3, float inv_c0,
                                      const float* __restrict__ r_in, float* __restrict__ r_out,
                                      const float* __restrict__ q, float* __restrict__ z_out, double* partials,
                                      unsigned* counter, SolverState* st, SolverState* outer, int total_cap, int blk,
                                      int nblk, const Defer& df)
{
    constexpr int H = TJ + 2 * S;
    constexpr int NL = S > 1 ? S - 1 : 1;   // stored levels z_1 .. z_{S-1}
    __shared__ double sm[64];
    const int lane = threadIdx.x & 31;
    const int item = blk * (int)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const StripPos s = strip_pos<S, TJ>(g, m, item, lane);   // from the arguments only
    const int SJ = SJF ? SJF : g.sj, SI = g.si;   // row and plane strides
    dep_wait();
    float alpha = 0.f;
    if (BIN && !FIRST) {   // pass A's sum, alpha (and the commit of the iteration)
        const HeadOut h = head_b<BOUT>(df.pin, df.nb_in, st, outer, blk);
        if (h.end) return;
        alpha = h.coef;
    } else {
        if (st->done) return;
        if (!FIRST) alpha = (float)st->alpha;
    }
    Acc arr, arz;
    if (item < m.items) {
        // r' at planes I - d: level 1 reads planes I .. I-2 and level L >= 2
        // plane I-L, so S + 1 planes, and 3 for a single level
        constexpr int NP = S == 0 ? 1 : (S < 2 ? 3 : S + 1);
        float rp[NP][H];
        float zr[NL][3][H];      // z_L at planes I - L - d (L = 1 .. S-1 at [L-1])
        float vr[H], vq[H];      // r, q of the plane being fetched
        float zS[H];             // the last level's z at its plane, before the stores
#pragma unroll
        for (int d = 0; d < NP; ++d)
#pragma unroll
            for (int r = 0; r < H; ++r) rp[d][r] = 0.f;
#pragma unroll
        for (int L = 0; L < NL; ++L)
#pragma unroll
            for (int r = 0; r < H; ++r) zr[L][0][r] = zr[L][1][r] = zr[L][2][r] = 0.f;
        auto fetch = [&](int P) {
            // plane -m reads plane m; planes past the outlet are not read (a
            // select, not a branch: the loads stay in the plane's basic block)
            const int pl = P < 0 ? -P : P;
            const bool ok = pl < g.nx;
            const int base = pl * SI + s.j0 * SJ + s.kl;
            with_rows(s.rows, [&](auto md) {
                constexpr int MD = decltype(md)::value;
#pragma unroll
                for (int r = 0; r < H; ++r) {
                    const int id = base + row_rel<MD, S, H>(r, s.j0, g.ny) * SJ;
                    vr[r] = ok ? r_in[id] : 0.f;
                    vq[r] = (!FIRST && ok) ? q[id] : 0.f;
                }
            });
        };
        fetch(s.i0 - S);
        // three steps per loop pass: the three-plane z rings rotate by
        // register renaming instead of moves (up to 4 levels; deeper ones
        // would spill)
        constexpr int UNROLL = S <= 4 ? 3 : 1;
#pragma unroll UNROLL
        for (int I = s.i0 - S; I < s.i1 + S; ++I) {
            // ---- level 0 at plane I
            {
                const bool pown = I >= s.i0 && I < s.i1;
                const int base = I * SI + s.j0 * SJ + s.kl;
                const float dinv = I == g.nx - 1 ? 1.f : inv_c0;   // Jacobi: identity row at the outlet
                float srr = 0.f, srz = 0.f;
                // the arithmetic of all rows first (one basic block), then
                // the stores and sums of the owned cells
#pragma unroll
                for (int r = 0; r < H; ++r) rp[0][r] = FIRST ? vr[r] : fmaf(-alpha, vq[r], vr[r]);
                // owned cells: every row of the strip or the rows inside the
                // grid (sums over all rows, then the lane's share)
                auto out0 = [&](auto all) {
                    constexpr bool AL = decltype(all)::value;
#pragma unroll
                    for (int r = S; r < S + TJ; ++r) {
                        const float rv = rp[0][r];
                        const bool o = AL ? s.kown : ((s.own >> r) & 1u);
                        const int id = base + r * SJ;
                        if (o) r_out[id] = rv;
                        srr = fmaf(AL || o ? rv : 0.f, rv, srr);
                        if (S == 0) {
                            const float zv = rv * dinv;
                            if (o) z_out[id] = zv;
                            srz = fmaf(AL || o ? rv : 0.f, zv, srz);
                        }
                    }
                    if (AL && !s.kown) srr = srz = 0.f;
                };
                if (pown) {
                    if (s.allrows) out0(std::true_type{});
                    else out0(std::false_type{});
                    acc_add(arr, srr);
                    if (S == 0) acc_add(arz, srz);
                }
            }
            if (I + 1 < s.i1 + S) fetch(I + 1);
            // ---- Chebyshev levels 1..S at planes I-1 .. I-S
#pragma unroll
            for (int LV = 1; LV <= S; ++LV) {
                const int Pk = I - LV;
                // plane-uniform level weights: the outlet plane is an identity
                // row, the plane before it has no east coefficient
                const bool ident = Pk == g.nx - 1;
                const float cc = ident ? c3.ci[LV - 1] : c3.cc[LV - 1], cx = ident ? 0.f : c3.cx[LV - 1];
                const float ce = (ident || Pk == g.nx - 2) ? 0.f : c3.cx[LV - 1];
                const float cy = ident ? 0.f : c3.cy[LV - 1], cz = ident ? 0.f : c3.cz[LV - 1];
                const float cr = c3.rr[LV - 1], cg = c3.gg[LV - 1];
                const bool out_plane = LV == S && Pk >= s.i0 && Pk < s.i1;
                const int pbase = Pk * SI + s.j0 * SJ + s.kl;
                float s2 = 0.f;
#pragma unroll
                for (int r = LV; r < H - LV; ++r) {
                    float zc, zw, ze, zs, zn;
                    if (LV == 1) {   // the stencil of z_0 = a0 r' (a0 is in the weights)
                        zc = rp[1][r]; zw = rp[2][r]; ze = rp[0][r];
                        zs = rp[1][r - 1]; zn = rp[1][r + 1];
                    } else {
                        zc = zr[LV - 2][1][r]; zw = zr[LV - 2][2][r]; ze = zr[LV - 2][0][r];
                        zs = zr[LV - 2][1][r - 1]; zn = zr[LV - 2][1][r + 1];
                    }
                    const float zb = __shfl_up_sync(FULL, zc, 1);
                    const float zt = __shfl_down_sync(FULL, zc, 1);
                    float zk = cc * zc + cx * zw + ce * ze + cy * (zs + zn) + cz * (zb + zt);
                    if (LV == 2) zk = fmaf(cr, rp[2][r], zk);   // r' and z_0 = a0 r'
                    if (LV >= 3) zk = fmaf(cr, rp[LV][r], fmaf(cg, zr[LV - 3][2][r], zk));
                    if (LV < S) zr[LV - 1][0][r] = zk;
                    else zS[r] = zk;
                }
                if (LV == S && out_plane) {   // stores and r'.z of the owned cells
                    auto outS = [&](auto all) {
                        constexpr bool AL = decltype(all)::value;
#pragma unroll
                        for (int r = S; r < S + TJ; ++r) {
                            const bool o = AL ? s.kown : ((s.own >> r) & 1u);
                            if (o) z_out[pbase + r * SJ] = zS[r];
                            s2 = fmaf(AL || o ? rp[S][r] : 0.f, zS[r], s2);
                        }
                        if (AL && !s.kown) s2 = 0.f;
                    };
                    if (s.allrows) outS(std::true_type{});
                    else outS(std::false_type{});
                    acc_add(arz, s2);
                }
            }
            // ---- rotate the rings by one plane
#pragma unroll
            for (int d = NP - 1; d >= 1; --d)
#pragma unroll
                for (int r = 0; r < H; ++r) rp[d][r] = rp[d - 1][r];
#pragma unroll
            for (int L = 0; L < S - 1; ++L)
#pragma unroll
                for (int r = 0; r < H; ++r) {
                    zr[L][2][r] = zr[L][1][r];
                    zr[L][1][r] = zr[L][0][r];
                }
        }
    }
    dep_signal();
    if (BOUT) {
        Acc v[2] = {arr, arz};
        put_partials<2>(v, reinterpret_cast<float2*>(sm), df.pout, blk, nblk);
        return;
    }
    pass_b_finish<FIRST>(arr, arz, partials, counter, sm, st, outer, total_cap, blk, nblk);
}

template <int SJF, int S, int TJ, bool FIRST>
__global__ void __launch_bounds__(col_threads(blocks4_b(S, TJ)), col_blocks(blocks4_b(S, TJ))) k_col_b(Geo g, ColMap m, ColCheb c3, float inv_c0,
                                               const float* __restrict__ r_in, float* __restrict__ r_out,
                                               const float* __restrict__ q, float* __restrict__ z_out,
                                               double* partials, unsigned* counter, SolverState* st,
                                               SolverState* outer, int total_cap, Defer df)
{
    col_b<SJF, S, TJ, FIRST, COL_DEFER_AB, COL_DEFER_BA>(g, m, c3, inv_c0, r_in, r_out, q, z_out, partials, counter, st,
                                                     outer, total_cap, blockIdx.x, gridDim.x, df);
}

// The single-case kernels for row stride SJF (0: the grid's, at run time).
template <int SJF>
KA pick_a_t(int tj, bool first)
{
    if (tj == 8) return first ? k_col_a<SJF, 8, true> : k_col_a<SJF, 8, false>;
    return first ? k_col_a<SJF, 16, true> : k_col_a<SJF, 16, false>;
}

// (levels, rows) instantiated: Jacobi 16 rows; 1..3 levels 4 or 8 rows;
// 4..6 levels 4 rows
template <int SJF>
KB pick_b_t(int S, int tj, bool first)
{
#define LES_B(s, t) return first ? k_col_b<SJF, s, t, true> : k_col_b<SJF, s, t, false>
    switch (S) {
    case 0: LES_B(0, 16);
    case 1: if (tj == 4) LES_B(1, 4); LES_B(1, 8);
    case 2: if (tj == 4) LES_B(2, 4); LES_B(2, 8);
    case 3: if (tj == 4) LES_B(3, 4); LES_B(3, 8);
    case 4: LES_B(4, 4);
    case 5: LES_B(5, 4);
    default: LES_B(6, 4);
    }
#undef LES_B
}

}  // namespace

// One translation unit per compiled row stride N defines the pickers of its
// kernels (les_col_sjN.cu).
#define LES_COL_STRIDE_UNIT(N)                                                                       \
    namespace les {                                                                                  \
    KA col_pick_a_sj##N(int tj, bool first) { return pick_a_t<N>(tj, first); }                       \
    KB col_pick_b_sj##N(int S, int tj, bool first) { return pick_b_t<N>(S, tj, first); }             \
    }

