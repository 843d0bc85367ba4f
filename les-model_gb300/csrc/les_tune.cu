// les_tune.cu -- autotuner for the register-column inner passes (les_col.cu):
// rows per strip and planes per march chunk, chosen by timing.
//
// A pass's strip shape trades halo recomputation (fewer rows: more halo rows
// per owned row) against registers and so occupancy; its chunk length trades
// the i-halo of each chunk against the number of independent warps.  Both
// optima depend on the grid, on the Chebyshev degree and on how much of the
// GPU the case gets (alone, or beside other cases of an ensemble), so they are
// measured: each candidate runs a few launches of the pass on the context's
// own matrix and work vectors, timed with CUDA events, cases of an ensemble
// concurrently as in a step.
#include <algorithm>
#include <vector>

#include "les_internal.cuh"
#include "les_mixed.cuh"

using namespace les;

struct les_ensemble;
extern "C" les_ctx* les_ensemble_case(les_ensemble* e, int i);
extern "C" int les_ensemble_size(const les_ensemble* e);

namespace {

constexpr int KT = 8;   // timed launches per candidate

// Inputs that keep the passes busy without converging: r = 1, z = 1/2,
// p = q = e = 0, alpha = beta = 0, tolerance -1 (never met).
__global__ void k_tune_prep(int n, float* r, float* z, float* p0, float* p1, float* q, float* e, float* r1)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    r[t] = 1.f;
    z[t] = 0.5f;
    p0[t] = p1[t] = q[t] = e[t] = r1[t] = 0.f;
}

// Finite block partials, so that a pass timed on its own (not after the
// other one) forms finite alpha, beta and residual norms from them.
__global__ void k_tune_partials(double* p, size_t n)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = 1.0;
}

// frozen: the passes' heads form their sums but use alpha = beta = 0 and
// never end the solve, so the vectors stay bounded however long it runs
__global__ void k_tune_state(SolverState* in, SolverState* out)
{
    in->frozen = 1;
    in->done = 0;
    in->k = 0;
    in->tol = -1.0;
    in->max_iter = 1 << 30;
    in->alpha = 0.0;
    in->beta = 0.0;
    in->rho = 1e300;       // beta = r'.z / rho rounds to 0 in FP32: p stays bounded
    in->rho_next = 1.0;
    in->status = LES_OK;
    out->iters = 0;
}

struct Case {
    les_ctx* c;
    les_pcg_opts o;
    int S;
    std::vector<int> ca, cb;   // chunk-length candidates of pass A, B
};

les_status prep(les_ctx* c)
{
    les_status st = ensure_work(c);
    if (!st) st = ensure_work32(c);
    if (st) return st;
    const int n = c->g.n;
    launch(c, k_tune_prep, (n + 255) / 256, 256, n, c->f[0], c->f[1], c->f[2], c->f[3], c->f[4], c->f[5], c->f[6]);
    launch(c, k_tune_partials, (unsigned)((c->partials_len + 255) / 256), 256, c->partials, c->partials_len);
    launch(c, k_tune_state, 1, 1, c->state + 1, c->state);
    return check_launch(c, "tune prep");
}

// chunk lengths the occupancy rule picks for shares 1, 1/2, 1/4, ... down to
// base/4 (distinct): from chunks that fill the GPU with this case alone to
// chunks that leave the GPU to the other cases
std::vector<int> chunk_candidates(les_ctx* c, const les_pcg_opts* o, double base, bool pass_b, int rows)
{
    std::vector<int> out;
    const double saved = c->share;
    const int sa = c->tune_cia, sb = c->tune_cib, ta = c->tune_tja, tb = c->tune_tjb;
    for (double sh = 1.0; sh >= base / 4.0 - 1e-12; sh /= 2.0) {
        c->share = sh;
        c->tune_cia = c->tune_cib = 0;
        if (pass_b) c->tune_tjb = rows; else c->tune_tja = rows;
        ColPlan P;
        if (col_plan(c, o, view32_of(c), c->state + 1, c->state, P)) continue;
        const int ci = pass_b ? P.mb.ci : P.ma.ci;
        if (std::find(out.begin(), out.end(), ci) == out.end()) out.push_back(ci);
    }
    c->share = saved;
    c->tune_cia = sa; c->tune_cib = sb; c->tune_tja = ta; c->tune_tjb = tb;
    return out;
}

// Runs KT inner iterations (pass A, then pass B) on every case concurrently
// (each case on its own stream, forked from and joined to `main`); returns
// microseconds per iteration round.
les_status time_round(std::vector<Case>& cs, cudaStream_t main, double* us)
{
    les_ctx* c0 = cs[0].c;
    cudaEvent_t e0, e1, fork;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    std::vector<cudaEvent_t> joins(cs.size());
    for (auto& j : joins) cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    std::vector<ColPlan> plans(cs.size());
    les_status st = LES_OK;
    for (size_t i = 0; i < cs.size() && !st; ++i) {
        st = prep(cs[i].c);
        if (!st) st = col_plan(cs[i].c, &cs[i].o, view32_of(cs[i].c), cs[i].c->state + 1, cs[i].c->state, plans[i]);
    }
    for (int rep = 0; rep < 2 && !st; ++rep) {   // rep 0 warms up
        cudaEventRecord(fork, main);
        if (rep == 1) cudaEventRecord(e0, main);
        for (size_t i = 0; i < cs.size() && !st; ++i) {
            les_ctx* c = cs[i].c;
            if (c->stream != main) cudaStreamWaitEvent(c->stream, fork, 0);
            for (int k = 0; k < KT && !st; ++k) {
                st = col_pass_a(c, plans[i], false, k & 1);
                if (!st) st = col_pass_b(c, plans[i], false, k & 1);
            }
            if (c->stream != main) {
                cudaEventRecord(joins[i], c->stream);
                cudaStreamWaitEvent(main, joins[i], 0);
            }
        }
        if (rep == 1) cudaEventRecord(e1, main);
    }
    if (!st) st = check_cuda(c0, cudaEventSynchronize(e1), "tune timing");
    float ms = 0.f;
    if (!st) st = check_cuda(c0, cudaEventElapsedTime(&ms, e0, e1), "tune timing");
    *us = 1e3 * ms / KT;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(fork);
    for (auto& j : joins) cudaEventDestroy(j);
    return st;
}

// Tries every candidate of one pass for all cases at once: rows r and the
// k-th chunk candidate of each case (its own list, clamped).  Leaves the
// fastest in the cases' tuning fields.
les_status tune_pass(std::vector<Case>& cs, cudaStream_t main, bool pass_b, double base, double* best)
{
    const int S = cs[0].S;
    std::vector<int> rows;
    if (pass_b) {
        if (S == 0) rows = {16};
        else if (S <= 3) rows = {4, 8};
        else rows = {4};
    } else {
        rows = {8, 16};
    }
    *best = 1e30;
    int br = rows[0], bk = 0;
    for (int r : rows) {
        size_t nk = 0;
        for (auto& q : cs) {
            auto& v = pass_b ? q.cb : q.ca;
            v = chunk_candidates(q.c, &q.o, base, pass_b, r);
            nk = std::max(nk, v.size());
        }
        for (size_t k = 0; k < nk; ++k) {
            for (auto& q : cs) {
                auto& v = pass_b ? q.cb : q.ca;
                const int ci = v.empty() ? 0 : v[std::min(k, v.size() - 1)];
                if (pass_b) { q.c->tune_tjb = r; q.c->tune_cib = ci; }
                else { q.c->tune_tja = r; q.c->tune_cia = ci; }
            }
            double us = 0;
            les_status st = time_round(cs, main, &us);
            if (st) return st;
            if (us < *best) {
                *best = us;
                br = r;
                bk = (int)k;
            }
        }
    }
    for (auto& q : cs) {   // apply the winner (recompute the list for its rows)
        auto v = chunk_candidates(q.c, &q.o, base, pass_b, br);
        const int ci = v.empty() ? 0 : v[std::min((size_t)bk, v.size() - 1)];
        if (pass_b) { q.c->tune_tjb = br; q.c->tune_cib = ci; }
        else { q.c->tune_tja = br; q.c->tune_cia = ci; }
        ++q.c->version;
    }
    return LES_OK;
}

les_status tune(std::vector<Case>& cs, cudaStream_t main, double base, double* best_us)
{
    double ua = 0, ub = 0;
    les_status st = tune_pass(cs, main, false, base, &ua);
    if (!st) st = tune_pass(cs, main, true, base, &ub);
    if (!st && best_us) *best_us = ub;   // an iteration with both chosen shapes
    // the next solve's own initialisation clears the frozen state
    for (auto& q : cs) q.c->share = base;
    return st;
}

}  // namespace

namespace les {
// The inputs and frozen solver state of the autotuner's timing rounds
les_status tune_prep(les_ctx* c) { return prep(c); }
}  // namespace les

extern "C" {

les_status les_autotune(les_ctx* c, const les_pcg_opts* o, double share, double* best_us)
{
    if (!c || !o || !(share > 0) || share > 1) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    if (!col_supported(c, o))
        return fail(c, LES_BAD_ARG, "autotune: the solve does not use the register-column passes");
    std::vector<Case> cs(1);
    cs[0].c = c;
    cs[0].o = *o;
    cs[0].o.max_iter = 1 << 30;
    cs[0].S = o->precond == LES_PC_JACOBI ? 0 : o->degree - 1;
    return tune(cs, c->stream, share, best_us);
}

les_status les_ensemble_autotune(les_ensemble* e, const les_pcg_opts* o, double* best_us)
{
    const int n = les_ensemble_size(e);
    if (!e || !o || n < 1) return LES_BAD_ARG;
    int handled = 0;   // the batched form tunes its work split
    les_status bst = les::ensemble_tune_batched(e, o, best_us, &handled);
    if (handled || bst) return bst;
    std::vector<Case> cs(n);
    for (int i = 0; i < n; ++i) {
        les_ctx* c = les_ensemble_case(e, i);
        cudaSetDevice(c->device);
        if (!col_supported(c, o))
            return fail(c, LES_BAD_ARG, "autotune: a case does not use the register-column passes");
        cs[i].c = c;
        cs[i].o = *o;
        cs[i].o.max_iter = 1 << 30;
        cs[i].S = o->precond == LES_PC_JACOBI ? 0 : o->degree - 1;
    }
    // time on case 0's stream as the fork point; every case's own stream runs its branch
    cudaStream_t main = nullptr;
    les_status st = check_cuda(cs[0].c, cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking), "tune stream");
    if (st) return st;
    for (auto& q : cs) {   // after the cases' pending work
        cudaEvent_t ev;
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        cudaEventRecord(ev, q.c->stream);
        cudaStreamWaitEvent(main, ev, 0);
        cudaEventDestroy(ev);
    }
    st = tune(cs, main, 1.0 / n, best_us);
    cudaStreamSynchronize(main);
    cudaStreamDestroy(main);
    return st;
}

}  // extern "C"
