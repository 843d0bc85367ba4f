// les_mixed.cuh -- shared pieces of the mixed-precision solve: the FP32 view
// of the pressure matrix, the Chebyshev coefficients and inner-product
// accumulators of the fused passes, the register-column pass plans
// (les_col.cu), the case table of the batched ensemble solve
// (les_ensemble.cu) and the capture of conditional solver loops.
#pragma once

#include "les_internal.cuh"

namespace les {

struct CoefF {
    float c, w, e, s, n, b, t;
};

__device__ __forceinline__ float self(unsigned m, float v1, float v2) { return m == 0u ? 0.f : (m == 1u ? v1 : v2); }

// The seven diagonals in FP32: decoded from the stencil codes (coefficients
// rounded once from the exact FP64 values) or read from FP32 copies of a
// stored matrix.
struct ViewF {
    const uint8_t* code;
    StencilCoefF k;
    const float* d[7];   // stored mode: c, n, s, e, w, t, b
    // Code 1 = all three axes in state 0: a fluid cell whose six neighbours
    // all exist and are fluid, with the base coefficients.
    __device__ __forceinline__ bool interior(int id) const { return code && code[id] == 1u; }
    __device__ __forceinline__ CoefF base() const
    {
        CoefF a;
        a.c = k.c0; a.w = a.e = k.x1; a.s = a.n = k.y1; a.b = a.t = k.z1;
        return a;
    }
    // coefficients of stencil code cd (device-built matrix)
    __device__ __forceinline__ CoefF from_code(unsigned cd) const
    {
        CoefF a;
        if (cd == 1u) return base();
        if (cd == 0u) {
            a.c = 1.f; a.w = a.e = a.s = a.n = a.b = a.t = 0.f;
            return a;
        }
        unsigned c = cd - 1u, xs = c % 5u, r = c / 5u, ys = r & 3u, zs = r >> 2;
        a.c = k.c0;
        a.w = self((XW_PACK >> (2 * xs)) & 3u, k.x1, k.x2);
        a.e = self((XE_PACK >> (2 * xs)) & 3u, k.x1, k.x2);
        a.s = self((YL_PACK >> (2 * ys)) & 3u, k.y1, k.y2);
        a.n = self((YH_PACK >> (2 * ys)) & 3u, k.y1, k.y2);
        a.b = self((YL_PACK >> (2 * zs)) & 3u, k.z1, k.z2);
        a.t = self((YH_PACK >> (2 * zs)) & 3u, k.z1, k.z2);
        return a;
    }
    __device__ __forceinline__ CoefF at(int id) const
    {
        if (code) return from_code(code[id]);
        CoefF a;
        a.c = d[0][id]; a.n = d[1][id]; a.s = d[2][id]; a.e = d[3][id];
        a.w = d[4][id]; a.t = d[5][id]; a.b = d[6][id];
        return a;
    }
    __device__ __forceinline__ float inv_diag(int id) const
    {
        if (code) return code[id] == 0 ? 1.f : 1.f / k.c0;
        return 1.f / d[0][id];
    }
};

// Chebyshev recurrence coefficients in FP32 (les-model src/pressure.cpp:871-905):
// z_0 = a0 r; level k: pc_k = b[k-1] pc_{k-1} + (r - A z_{k-1}), z_k = z_{k-1} + a[k-1] pc_k.
struct ChebF {
    float a0;
    float a[8], b[8];
};

// The same polynomial in three-term form, as the column passes apply it.
// With pc_{k-1} = (z_{k-1} - z_{k-2}) / a_{k-1} (z_{-1} = 0, so pc_0 = r),
// level k is  z_k = (1 + g_k) z_{k-1} - g_k z_{k-2} + a_k (r - A z_{k-1}),
// g_k = a_k b_k / a_{k-1}.  A's plane-uniform coefficients are folded into
// per-level weights, so a level is one 7-point stencil plus the r and z_{k-2}
// terms.  Level 1 reads r' directly (z_0 = a0 r', its r term joins the
// centre weight); level 2's z_{k-2} = z_0 term joins its r term.
struct ColCheb {
    float cc[6], ci[6];          // centre weight; on the outlet plane's identity rows
    float cx[6], cy[6], cz[6];   // neighbour weights along i, j, k
    float rr[6], gg[6];          // weights of r' and of z_{k-2} at the centre
};
ColCheb col_cheb(const les_pcg_opts* o, float c0, float x1, float y1, float z1);

// Inner products of the fused passes: per-thread double-float (TwoSum /
// TwoProd, ~48-bit significand) accumulation, summed across threads and
// blocks in FP64.  GB300's FP64 pipe is ~70x slower than its FP32 pipe.
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

// The inner FP32 solve of a correction stops at max(inner_rtol ||r||,
// tol / LAST_MARGIN): the last correction is not solved further than the
// outer FP64 test needs, less a margin for the FP32 rounding of the update
// (the FP64 test still decides, at worst after one more correction).
// Measured on GB300 (inner iterations per step, 256x128x128 / 512x256x256 /
// 64-case batch): margin 3: 564 / 986 / 207, 2: 557 / 969 / 202, 1.5: 553 /
// 962 / 198.
constexpr double LAST_MARGIN = 1.5;

ChebF cheb_coefs(const les_pcg_opts* o);
bool fused_supported(const les_pcg_opts* o);

// ---- register-column passes (les_col.cu) ----------------------------------
// Work split of one pass: warp `item` owns k-strip item % tiles_k, row strip
// (item / tiles_k) % tiles_j and plane chunk item / (tiles_k * tiles_j).
struct ColMap {
    int tk;        // output cells of a strip along k (32 minus twice the halo)
    int tj;        // output rows of a strip along j
    int tiles_k, tiles_j;
    int ci;        // planes per chunk
    int items;     // strips x chunks = warps with work
};

struct ColPlan {
    int S = 0;             // Chebyshev levels (degree - 1); 0 = Jacobi
    ColCheb c3{};
    float inv_c0 = 1.f;
    ColMap ma{}, mb{};
    int blocks_a = 0, blocks_b = 0;
    ViewF A{};
    SolverState* in = nullptr;
    SolverState* out = nullptr;
    int cap = 0;
};

// the column passes serve this solve (device-built matrix, Jacobi or
// Chebyshev degree 2..7, option LES_OPT_FUSED = 1 without TMA)
bool col_supported(const les_ctx* c, const les_pcg_opts* o);
les_status col_plan(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out, ColPlan& P);
// pass A: p_new = pb[pc ^ 1] from z and p_old = pb[pc]; pass B: r[rin] -> r[rin ^ 1]
les_status col_pass_a(les_ctx* c, const ColPlan& P, bool first, int pc);
les_status col_pass_b(les_ctx* c, const ColPlan& P, bool first, int rin);
// x += e + alpha p_last: the update the column passes defer to the end of the solve
les_status col_x_update(les_ctx* c);
les_status inner_solve_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out,
                             int inner_cap);
// ---- batched ensemble solve (les_ensemble.cu) ------------------------------
// One case of a mixed-precision solve that advances together with the other
// cases of an ensemble: each batched kernel covers every case, its blocks
// split into consecutive per-case ranges (prefix arrays of block starts), and
// each block works on its own case only.  Lives in device memory.
// Iteration pairs per pass of the inner loop body of a captured mixed solve:
// each pass of a conditional loop costs about 6 us at 256x128x128 (the
// condition kernel and the body's relaunch), each iteration that starts
// after convergence a few us of early exits.  Measured, 20 steps of
// 256x128x128: 1 pair 140.4, 2 pairs 144.0, 3 pairs 145.5, 4 pairs 146.1
// Mcell-steps/s; 512x256x256 unchanged.  With the later, faster passes:
// 4 pairs 170.0, 6 pairs 170.7, 8 pairs 171.1.
#ifndef INNER_BODY_PAIRS
#define INNER_BODY_PAIRS 8
#endif

struct BatchCase {
    Geo g;
    ColMap ma, mb;                 // column-pass work splits
    float c0, x1, y1, z1;          // plane-uniform FP32 coefficients
    ColCheb c3;                    // pass B's Chebyshev level weights
    float inv_c0;
    float *r0, *r1, *z, *p0, *p1, *q, *e;   // FP32 inner vectors
    double* x;                     // FP64 solution (the pressure slot)
    const double* b;               // FP64 right-hand side
    StencilView A;                 // FP64 matrix for the defect
    double* partials;
    unsigned* counters;
    SolverState* out;
    SolverState* in;
    double inner_rtol;
    int cap, inner_cap, max_outer; // total inner iterations, per correction, corrections
    int act;                       // the current correction round runs for this case
};

// block -> case of a batched grid (pre: n + 1 block starts, ascending)
__device__ __forceinline__ int batch_case(const int* pre, int n, int block)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// column passes over all cases (S levels; rows as in the single-case default)
int col_batch_tj_b(int S);
les_status tune_prep(les_ctx* c);   // the autotuner's inputs and frozen state (les_tune.cu)
// les_ensemble_autotune for a batched ensemble: times its work splits
// (*handled = 0 when the ensemble does not run batched)
les_status ensemble_tune_batched(les_ensemble* e, const les_pcg_opts* o, double* best_us, int* handled);
int col_batch_warps_per_block();   // warps of a batched column-pass block (one item each)
ColMap col_batch_map(les_ctx* c, int pass, int S, int chunk_planes);   // pass 0: A, 1: B
int col_batch_resident_warps(int pass, int S);
les_status col_batch_pass_a(cudaStream_t s, bool first, int pc, const BatchCase* cs, const int* pre, int n,
                            int blocks);
les_status col_batch_pass_b(cudaStream_t s, int S, bool first, int rin, const BatchCase* cs, const int* pre, int n,
                            int blocks);
les_status col_batch_x_update(cudaStream_t s, const BatchCase* cs, const int* pre, int n, int blocks);
// the FP64 defect of every case still in its correction round (les_mixed.cu)
les_status batch_outer_resid(cudaStream_t s, const BatchCase* cs, const int* pre, int n, int blocks);
int batch_resid_blocks(const Geo& g);
StencilView stencil_view_of(les_ctx* c);

// Adds a `while` loop at the current capture point of *stream: creates the
// loop's condition handle, captures `entry(h)` (a kernel that sets the
// condition from the solver state, so the loop can be skipped and is
// re-armed each time an enclosing loop comes back to it), adds the
// conditional node, captures its body with `body(h)` -- *stream points to the
// body's capture stream meanwhile -- which must end by setting the condition
// again, and resumes the capture after the node.  check(err, what) turns a
// CUDA error into a status.
template <class Check, class Entry, class Body>
les_status capture_while_on(cudaStream_t* stream, Check check, Entry entry, Body body)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    les_status st = check(cudaStreamGetCaptureInfo(*stream, &cs, nullptr, &g, &deps, nullptr, &ndeps), "capture info");
    if (st) return st;
    if (cs != cudaStreamCaptureStatusActive) return LES_BAD_ARG;
    cudaGraphConditionalHandle h;
    if ((st = check(cudaGraphConditionalHandleCreate(&h, g, 0, 0), "conditional handle"))) return st;
    if ((st = entry(h))) return st;
    if ((st = check(cudaStreamGetCaptureInfo(*stream, &cs, nullptr, &g, &deps, nullptr, &ndeps), "capture info")))
        return st;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if ((st = check(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np), "conditional node"))) return st;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    cudaStream_t outer = *stream, inner = nullptr;
    if ((st = check(cudaStreamCreateWithFlags(&inner, cudaStreamNonBlocking), "body stream"))) return st;
    st = check(cudaStreamBeginCaptureToGraph(inner, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
               "body capture");
    if (!st) {
        *stream = inner;
        st = body(h);
        *stream = outer;
        cudaGraph_t got = nullptr;
        les_status st2 = check(cudaStreamEndCapture(inner, &got), "end body capture");
        if (!st) st = st2;
    }
    cudaStreamDestroy(inner);
    if (st) return st;
    return check(cudaStreamUpdateCaptureDependencies(outer, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                 "resume capture");
}

// graph capture of the whole mixed solve (fused inner iteration)
les_status emit_outer_start(les_ctx* c, const les_pcg_opts* o, int keep_tol);
les_status emit_inner_start(les_ctx* c, const les_pcg_opts* o, int inner_cap);
les_status emit_outer_update(les_ctx* c, bool deferred);
les_status capture_mixed_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, int keep_tol);
ViewF view32_of(les_ctx* c);

}  // namespace les
