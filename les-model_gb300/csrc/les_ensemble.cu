// les_ensemble.cu -- many independent cases of uneven grid sizes advanced by
// one CUDA graph launch per time step.
//
// Each case is an ordinary context (its own fields, matrix, solver state and
// work vectors).  A step of the ensemble is captured once per velocity-buffer
// parity and replayed with one launch.  Two forms:
//
// Batched (default, when every case runs the register-column passes with the
// same preconditioner): the capture forks into every case's stream for the
// step up to the pressure solve's first FP64 defect, joins, runs the mixed
// solves of all cases together -- each inner pass, defect and update is ONE
// kernel over all cases (blocks in per-case ranges), the inner and outer
// loops are conditional nodes that run while any case still iterates, and a
// case that has converged leaves each kernel at once -- then forks again for
// the projection.  The GPU sees a few large launches per iteration instead of
// two small ones per case.
//
// Branches: one independent branch per case holding that case's whole step
// (both solver loops as its own conditional nodes); the cases' kernels
// overlap on the GPU, and a case that converges early ends its branch early.
//
// The cases are independent units: across GPUs they would be partitioned with
// no exchange.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "les_internal.cuh"
#include "les_mixed.cuh"

using namespace les;

struct les_ensemble {
    int device = 0;
    std::vector<les_ctx*> cs;
    cudaStream_t main = nullptr;
    cudaEvent_t ev = nullptr;       // fork / join / ordering
    int batched = 1;                // les_ensemble_set_batched
    int split = 4;                  // batched passes: items per pass up to split x the resident warps
    unsigned long long* d_count = nullptr;   // batched kernels run (added by the loop conditions)
    struct Graph {
        std::vector<les_step_params> prm;
        std::vector<double*> slots;       // LES_NSLOTS per case
        std::vector<double*> tau;
        std::vector<unsigned long long> version, captured;
        cudaGraphExec_t exec = nullptr;
        int req = -1;                         // e->batched when captured
        int split = 0;                        // e->split when captured
        bool batched = false;                 // the form captured (branches if the cases cannot batch)
        les::BatchCase* d_cases = nullptr;    // batched form: case table, grid order
        int* d_pre = nullptr;                 // block starts: A, B, defect, update (4 x (n + 1))
    } g[2];
    int last = 0;
    std::string err;
};

namespace {

les_status efail(les_ensemble* e, les_status st, const std::string& msg)
{
    e->err = msg;
    return st;
}

les_status ecuda(les_ensemble* e, cudaError_t r, const char* what)
{
    if (r == cudaSuccess) return LES_OK;
    cudaGetLastError();
    return efail(e, LES_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(r));
}

void graph_clear(les_ensemble::Graph& g)
{
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.d_cases) cudaFree(g.d_cases);
    if (g.d_pre) cudaFree(g.d_pre);
    g = les_ensemble::Graph{};
}

bool graph_matches(const les_ensemble* e, const les_ensemble::Graph& g, const les_step_params* prm)
{
    if (!g.exec || g.req != e->batched || g.split != e->split) return false;
    for (size_t i = 0; i < e->cs.size(); ++i) {
        const les_ctx* c = e->cs[i];
        if (g.version[i] != c->version || g.tau[i] != c->tau ||
            std::memcmp(&g.prm[i], &prm[i], sizeof(les_step_params)) != 0 ||
            std::memcmp(&g.slots[i * LES_NSLOTS], c->slot, sizeof(double*) * LES_NSLOTS) != 0)
            return false;
    }
    return true;
}

bool same_params(const les_ensemble* e, const les_ensemble::Graph& g, const les_step_params* prm)
{
    if (!g.exec || g.req != e->batched || g.split != e->split) return false;
    for (size_t i = 0; i < e->cs.size(); ++i)
        if (g.version[i] != e->cs[i]->version || std::memcmp(&g.prm[i], &prm[i], sizeof(les_step_params)) != 0)
            return false;
    return true;
}

// ---- batched form --------------------------------------------------------------
// A correction round starts for every case that still iterates: its inner
// state is set up as for one case (les_mixed.cu k_inner_init); the others get
// a finished inner state so that their blocks leave every kernel at once.
__global__ void k_round_begin(BatchCase* cs, int n)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        BatchCase& C = cs[c];
        SolverState* out = C.out;
        SolverState* in = C.in;
        const int act = !out->done && out->k < C.max_outer && out->iters < C.cap;
        C.act = act;
        if (act) {
            in->tol = fmax(C.inner_rtol * out->err, out->tol / LAST_MARGIN);
            in->max_iter = C.inner_cap;
            in->k = 0;
            in->done = 0;
            in->frozen = 0;
            in->iters = 0;
            in->status = LES_OK;
            in->beta = 0.0;
        } else {
            in->done = 1;
        }
    }
}

// Loop conditions: any case still in its inner solve / its corrections; add
// counts the batched kernels of the loop pass that ends here.
__global__ void k_cond_any_inner(const BatchCase* cs, int n, cudaGraphConditionalHandle h, unsigned long long* count,
                                 int add)
{
    int any = 0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const SolverState* in = cs[c].in;
        any |= (!in->done && in->k < cs[c].inner_cap) ? 1 : 0;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, any ? 1u : 0u);
        *count += add;
    }
}

__global__ void k_cond_any_outer(const BatchCase* cs, int n, cudaGraphConditionalHandle h, unsigned long long* count,
                                 int add)
{
    int any = 0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const SolverState* out = cs[c].out;
        any |= (!out->done && out->k < cs[c].max_outer && out->iters < cs[c].cap) ? 1 : 0;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, any ? 1u : 0u);
        *count += add;
    }
}

struct BatchLayout {
    int S = 0;
    int blocks[4] = {};          // A, B, defect, update
    std::vector<int> order;      // grid position -> case
};

// Can the cases' solves run batched: all mixed-precision fused PCG on the
// register-column passes with one preconditioner (Jacobi, or Chebyshev of one
// degree).
bool batchable(les_ensemble* e, const les_step_params* prm)
{
    for (size_t i = 0; i < e->cs.size(); ++i) {
        const les_pcg_opts& o = prm[i].pcg;
        if (!col_supported(e->cs[i], &o) || o.precond != prm[0].pcg.precond ||
            (o.precond == LES_PC_CHEBYSHEV && o.degree != prm[0].pcg.degree))
            return false;
    }
    return true;
}

// Work splits of the batched column passes: each case starts with one chunk
// per strip (whole-length marches); while all cases' items are fewer than
// e->split times the GPU's resident warps, the case with the longest march
// gets one chunk more.  Many short, similar items let the block scheduler
// balance the ragged cases (64-case batch, GB300: 1x resident 162, 2x 194,
// 3x 207, 4x 210, 6x 203 Mcell-steps/s); the default is 4 and
// les_ensemble_autotune times 2, 3, 4 and 6.  Grid order: longest marches
// first.
les_status batch_plan(les_ensemble* e, const les_step_params* prm, les_ensemble::Graph& g, BatchLayout& L)
{
    const int n = (int)e->cs.size();
    const les_pcg_opts& o0 = prm[0].pcg;
    L.S = o0.precond == LES_PC_JACOBI ? 0 : o0.degree - 1;
    std::vector<ColMap> ma(n), mb(n);
    for (int pass = 0; pass < 2; ++pass) {
        const int halo = pass == 0 ? 1 : L.S;
        const int resident = col_batch_resident_warps(pass, L.S);
        std::vector<int> chunks(n, 1);
        std::vector<ColMap>& m = pass == 0 ? ma : mb;
        long long total = 0;
        for (int i = 0; i < n; ++i) {
            m[i] = col_batch_map(e->cs[i], pass, L.S, e->cs[i]->g.nx);
            total += m[i].items;
        }
        const int min_ci = 2 * halo > 4 ? 2 * halo : 4;
        while (total < (long long)e->split * resident) {
            int best = -1;
            for (int i = 0; i < n; ++i)
                if (m[i].ci / 2 >= min_ci && (best < 0 || m[i].ci > m[best].ci)) best = i;
            if (best < 0) break;
            total -= m[best].items;
            ++chunks[best];
            const int nx = e->cs[best]->g.nx;
            m[best] = col_batch_map(e->cs[best], pass, L.S, (nx + chunks[best] - 1) / chunks[best]);
            total += m[best].items;
        }
    }
    L.order.resize(n);
    std::iota(L.order.begin(), L.order.end(), 0);
    std::stable_sort(L.order.begin(), L.order.end(), [&](int a, int b) { return mb[a].ci > mb[b].ci; });
    std::vector<BatchCase> hc(n);
    std::vector<int> pre(4 * (n + 1), 0);
    for (int q = 0; q < n; ++q) {
        const int i = L.order[q];
        les_ctx* c = e->cs[i];
        const les_pcg_opts& o = prm[i].pcg;
        const ViewF A32 = view32_of(c);
        BatchCase& C = hc[q];
        C.g = c->g;
        C.ma = ma[i];
        C.mb = mb[i];
        C.c0 = A32.k.c0;
        C.x1 = A32.k.x1;
        C.y1 = A32.k.y1;
        C.z1 = A32.k.z1;
        C.c3 = col_cheb(&o, A32.k.c0, A32.k.x1, A32.k.y1, A32.k.z1);
        C.inv_c0 = 1.f / A32.k.c0;
        C.r0 = c->f[0]; C.r1 = c->f[6]; C.z = c->f[1]; C.p0 = c->f[2]; C.p1 = c->f[3]; C.q = c->f[4]; C.e = c->f[5];
        C.x = c->slot[LES_P];
        C.b = c->slot[LES_B];
        C.A = stencil_view_of(c);
        C.partials = c->partials;
        C.counters = c->counters;
        C.out = c->state;
        C.in = c->state + 1;
        C.inner_rtol = o.inner_rtol;
        C.cap = o.max_iter;
        C.inner_cap = o.inner_max_iter > 0 ? o.inner_max_iter : o.max_iter;
        C.max_outer = o.max_outer > 0 ? o.max_outer : 50;
        C.act = 0;
        const int wpb = col_batch_warps_per_block();
        const int nb[4] = {(ma[i].items + wpb - 1) / wpb, (mb[i].items + wpb - 1) / wpb, batch_resid_blocks(c->g),
                           (c->g.n + 255) / 256};
        if ((size_t)2 * nb[0] > c->partials_len || (size_t)2 * nb[1] > c->partials_len ||
            (size_t)nb[2] > c->partials_len)
            return efail(e, LES_BAD_ARG, "case " + std::to_string(i) + ": batched grid exceeds the reduction scratch");
        for (int k = 0; k < 4; ++k) pre[k * (n + 1) + q + 1] = pre[k * (n + 1) + q] + nb[k];
    }
    for (int k = 0; k < 4; ++k) L.blocks[k] = pre[k * (n + 1) + n];
    les_status st = ecuda(e, cudaMalloc(&g.d_cases, sizeof(BatchCase) * n), "batch table");
    if (!st) st = ecuda(e, cudaMalloc(&g.d_pre, sizeof(int) * pre.size()), "batch blocks");
    if (!st) st = ecuda(e, cudaMemcpy(g.d_cases, hc.data(), sizeof(BatchCase) * n, cudaMemcpyHostToDevice), "batch table");
    if (!st) st = ecuda(e, cudaMemcpy(g.d_pre, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice), "batch blocks");
    return st;
}

// The mixed solves of all cases, batched, into the capture on e->main
les_status emit_batched_solve(les_ensemble* e, les_ensemble::Graph& g, const BatchLayout& L)
{
    const int n = (int)e->cs.size();
    BatchCase* cs = g.d_cases;
    const int *pa = g.d_pre, *pb = g.d_pre + (n + 1), *pr = g.d_pre + 2 * (n + 1), *px = g.d_pre + 3 * (n + 1);
    unsigned long long* cnt = e->d_count;
    cudaStream_t s = e->main;
    auto chk = [e](cudaError_t r, const char* what) { return ecuda(e, r, what); };
    auto launched = [&](const char* what) { return ecuda(e, cudaPeekAtLastError(), what); };
    les_status st = capture_while_on(
        &s, chk,
        [&](cudaGraphConditionalHandle h) {
            k_cond_any_outer<<<1, 256, 0, s>>>(cs, n, h, cnt, 1);
            return launched("outer condition");
        },
        [&](cudaGraphConditionalHandle ho) -> les_status {
            les_status s2;
            k_round_begin<<<(n + 127) / 128, 128, 0, s>>>(cs, n);
            if ((s2 = launched("round start"))) return s2;
            // z = M^-1 r, rho; iteration 1 (p1 = z, e = 0); r1 -> r0
            if ((s2 = col_batch_pass_b(s, L.S, true, 0, cs, pb, n, L.blocks[1]))) return launched("batched pass B");
            if ((s2 = col_batch_pass_a(s, true, 0, cs, pa, n, L.blocks[0]))) return launched("batched pass A");
            if ((s2 = col_batch_pass_b(s, L.S, false, 1, cs, pb, n, L.blocks[1]))) return launched("batched pass B");
            s2 = capture_while_on(
                &s, chk,
                [&](cudaGraphConditionalHandle h) {
                    k_cond_any_inner<<<1, 256, 0, s>>>(cs, n, h, cnt, 0);
                    return launched("inner condition");
                },
                [&](cudaGraphConditionalHandle hi) -> les_status {
                    if (col_batch_pass_a(s, false, 1, cs, pa, n, L.blocks[0])) return launched("batched pass A");
                    if (col_batch_pass_b(s, L.S, false, 0, cs, pb, n, L.blocks[1])) return launched("batched pass B");
                    if (col_batch_pass_a(s, false, 0, cs, pa, n, L.blocks[0])) return launched("batched pass A");
                    if (col_batch_pass_b(s, L.S, false, 1, cs, pb, n, L.blocks[1])) return launched("batched pass B");
                    k_cond_any_inner<<<1, 256, 0, s>>>(cs, n, hi, cnt, 5);
                    return launched("inner condition");
                });
            if (s2) return s2;
            // x += e + alpha p_last, r = b - A x, ||r|| for the cases of the round
            if ((s2 = col_batch_x_update(s, cs, px, n, L.blocks[3]))) return launched("batched update");
            if ((s2 = batch_outer_resid(s, cs, pr, n, L.blocks[2]))) return launched("batched defect");
            k_cond_any_outer<<<1, 256, 0, s>>>(cs, n, ho, cnt, 8);
            return launched("outer condition");
        });
    return st;
}

les_status capture_batched(les_ensemble* e, const les_step_params* prm, les_ensemble::Graph& g)
{
    const size_t n = e->cs.size();
    g.prm.assign(prm, prm + n);
    g.slots.resize(n * LES_NSLOTS);
    g.tau.resize(n);
    g.version.resize(n);
    g.captured.resize(n);
    g.batched = true;
    std::vector<double*> before(n * LES_NSLOTS);
    for (size_t i = 0; i < n; ++i) {
        les_ctx* c = e->cs[i];
        les_status st = ensure_work(c);
        if (!st) st = ensure_work32(c);
        if (st) return efail(e, st, "case " + std::to_string(i) + ": " + c->err);
        std::memcpy(&before[i * LES_NSLOTS], c->slot, sizeof(double*) * LES_NSLOTS);
        g.version[i] = c->version;
        g.tau[i] = c->tau;
    }
    if (!e->d_count) {
        les_status st = ecuda(e, cudaMalloc(&e->d_count, sizeof(unsigned long long)), "launch counter");
        if (!st) st = ecuda(e, cudaMemset(e->d_count, 0, sizeof(unsigned long long)), "launch counter");
        if (st) return st;
    }
    BatchLayout L;
    les_status st = batch_plan(e, prm, g, L);
    if (st) return st;
    std::memcpy(g.slots.data(), before.data(), sizeof(double*) * n * LES_NSLOTS);
    st = ecuda(e, cudaStreamBeginCapture(e->main, cudaStreamCaptureModeRelaxed), "begin ensemble capture");
    if (st) return st;
    std::vector<cudaEvent_t> evs;
    auto fork_join = [&](auto per_case) -> les_status {
        cudaEvent_t f = nullptr;
        les_status s1 = ecuda(e, cudaEventCreateWithFlags(&f, cudaEventDisableTiming), "fork event");
        if (s1) return s1;
        evs.push_back(f);
        if ((s1 = ecuda(e, cudaEventRecord(f, e->main), "fork"))) return s1;
        for (size_t i = 0; i < n; ++i) {
            les_ctx* c = e->cs[i];
            if ((s1 = ecuda(e, cudaStreamWaitEvent(c->stream, f, 0), "fork wait"))) return s1;
            const unsigned long long l0 = c->launches;
            les_status s2 = per_case(i, c);
            g.captured[i] += c->launches - l0;
            c->launches = l0;
            if (s2) return efail(e, s2, "case " + std::to_string(i) + ": " + c->err);
            cudaEvent_t j = nullptr;
            if ((s1 = ecuda(e, cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "join event"))) return s1;
            evs.push_back(j);
            if ((s1 = ecuda(e, cudaEventRecord(j, c->stream), "join"))) return s1;
            if ((s1 = ecuda(e, cudaStreamWaitEvent(e->main, j, 0), "join wait"))) return s1;
        }
        return LES_OK;
    };
    std::fill(g.captured.begin(), g.captured.end(), 0ull);
    st = fork_join([&](size_t i, les_ctx* c) { return emit_step_pre(c, &prm[i], true); });
    if (!st) st = emit_batched_solve(e, g, L);
    if (!st) st = fork_join([&](size_t i, les_ctx* c) { return emit_step_post(c, &prm[i]); });
    cudaGraph_t graph = nullptr;
    les_status s3 = ecuda(e, cudaStreamEndCapture(e->main, &graph), "end ensemble capture");
    for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
    if (!st) st = s3;
    if (!st) st = ecuda(e, cudaGraphInstantiate(&g.exec, graph, 0), "instantiate ensemble graph");
    if (graph) cudaGraphDestroy(graph);
    if (st) {   // nothing ran: undo the captured buffer swaps
        for (size_t i = 0; i < n; ++i) std::memcpy(e->cs[i]->slot, &before[i * LES_NSLOTS], sizeof(double*) * LES_NSLOTS);
        graph_clear(g);
    }
    return st;
}

les_status capture_branches(les_ensemble* e, const les_step_params* prm, les_ensemble::Graph& g)
{
    const size_t n = e->cs.size();
    g.prm.assign(prm, prm + n);
    g.slots.resize(n * LES_NSLOTS);
    g.tau.resize(n);
    g.version.resize(n);
    g.captured.resize(n);
    std::vector<double*> before(n * LES_NSLOTS);
    for (size_t i = 0; i < n; ++i) {
        les_ctx* c = e->cs[i];
        les_status st = ensure_work(c);
        if (!st) st = ensure_work32(c);
        if (st) return efail(e, st, "case " + std::to_string(i) + ": " + c->err);
        std::memcpy(&g.slots[i * LES_NSLOTS], c->slot, sizeof(double*) * LES_NSLOTS);
        std::memcpy(&before[i * LES_NSLOTS], c->slot, sizeof(double*) * LES_NSLOTS);
        g.version[i] = c->version;
    }
    les_status st = ecuda(e, cudaStreamBeginCapture(e->main, cudaStreamCaptureModeRelaxed), "begin ensemble capture");
    if (st) return st;
    st = ecuda(e, cudaEventRecord(e->ev, e->main), "fork");
    size_t done = 0;
    std::vector<cudaEvent_t> joins;
    for (size_t i = 0; i < n && !st; ++i) {
        les_ctx* c = e->cs[i];
        st = ecuda(e, cudaStreamWaitEvent(c->stream, e->ev, 0), "fork wait");
        if (st) break;
        const unsigned long long l0 = c->launches;
        les_status s2 = emit_step(c, &prm[i]);
        g.captured[i] = c->launches - l0;
        c->launches = l0;
        g.tau[i] = c->tau;
        done = i + 1;
        if (s2) {
            st = efail(e, s2, "case " + std::to_string(i) + ": " + c->err);
            break;
        }
        // join: the ensemble stream waits for this case's branch
        cudaEvent_t j = nullptr;
        st = ecuda(e, cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "join event");
        if (st) break;
        joins.push_back(j);
        st = ecuda(e, cudaEventRecord(j, c->stream), "join");
        if (!st) st = ecuda(e, cudaStreamWaitEvent(e->main, j, 0), "join wait");
    }
    cudaGraph_t graph = nullptr;
    les_status s3 = ecuda(e, cudaStreamEndCapture(e->main, &graph), "end ensemble capture");
    for (cudaEvent_t j : joins) cudaEventDestroy(j);
    if (!st) st = s3;
    if (!st) st = ecuda(e, cudaGraphInstantiate(&g.exec, graph, 0), "instantiate ensemble graph");
    if (graph) cudaGraphDestroy(graph);
    if (st) {   // nothing ran: undo the captured buffer swaps
        for (size_t i = 0; i < done; ++i)
            std::memcpy(e->cs[i]->slot, &before[i * LES_NSLOTS], sizeof(double*) * LES_NSLOTS);
        graph_clear(g);
    }
    return st;
}

les_status capture(les_ensemble* e, const les_step_params* prm, les_ensemble::Graph& g)
{
    les_status st = (e->batched && batchable(e, prm)) ? capture_batched(e, prm, g) : capture_branches(e, prm, g);
    if (!st) {
        g.req = e->batched;
        g.split = e->split;
    }
    return st;
}

}  // namespace

// les_ensemble_autotune's batched form: for each candidate work split, the
// case table of the batched plan and KT timing rounds of the batched passes
// A and B over all cases (inputs and frozen states of the single-case
// tuner); keeps the fastest split.
les_status les::ensemble_tune_batched(les_ensemble* e, const les_pcg_opts* o, double* best_us, int* handled)
{
    *handled = 0;
    const int n = (int)e->cs.size();
    std::vector<les_step_params> prm(n);
    for (auto& p : prm) {
        p = les_step_params{};
        p.solver = LES_SOLVER_PCG;
        p.pcg = *o;
        p.pcg.precision = LES_MIXED;
    }
    if (!e->batched || !batchable(e, prm.data())) return LES_OK;
    *handled = 1;
    cudaSetDevice(e->device);
    les_status st = ecuda(e, cudaStreamSynchronize(e->main), "tune sync");
    for (int i = 0; i < n && !st; ++i) {
        les_ctx* c = e->cs[i];
        st = tune_prep(c);
        if (!st) st = ecuda(e, cudaStreamSynchronize(c->stream), "tune prep");
        if (st == LES_CUDA_ERROR || st == LES_BAD_ARG) st = efail(e, st, "case " + std::to_string(i) + ": " + c->err);
    }
    if (st) return st;
    constexpr int KT = 6;
    const int cand[4] = {2, 3, 4, 6};
    const int saved = e->split;
    double best = 1e30;
    int pick = saved;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = ecuda(e, cudaEventCreate(&e0), "tune event");
    if (!st) st = ecuda(e, cudaEventCreate(&e1), "tune event");
    for (int q = 0; q < 4 && !st; ++q) {
        e->split = cand[q];
        les_ensemble::Graph tg;   // the case table and block starts only
        BatchLayout L;
        st = batch_plan(e, prm.data(), tg, L);
        const int* pa = tg.d_pre;
        const int* pb = tg.d_pre + (n + 1);
        for (int rep = 0; rep < 2 && !st; ++rep) {   // rep 0 warms up
            st = ecuda(e, cudaEventRecord(e0, e->main), "tune event");
            for (int k = 0; k < KT && !st; ++k) {
                st = col_batch_pass_a(e->main, false, k & 1, tg.d_cases, pa, n, L.blocks[0]);
                if (!st) st = col_batch_pass_b(e->main, L.S, false, k & 1, tg.d_cases, pb, n, L.blocks[1]);
                if (st) st = ecuda(e, cudaGetLastError(), "tune pass");
            }
            if (!st) st = ecuda(e, cudaEventRecord(e1, e->main), "tune event");
        }
        float ms = 0.f;
        if (!st) st = ecuda(e, cudaEventSynchronize(e1), "tune timing");
        if (!st) st = ecuda(e, cudaEventElapsedTime(&ms, e0, e1), "tune timing");
        graph_clear(tg);
        if (!st && 1e3 * ms / KT < best) {
            best = 1e3 * ms / KT;
            pick = cand[q];
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    e->split = st ? saved : pick;
    if (!st && best_us) *best_us = best;
    return st;
}

extern "C" {

les_status les_ensemble_create(const les_mesh* meshes, int count, int device, les_ensemble** out)
{
    if (!meshes || count < 1 || !out) return LES_BAD_ARG;
    *out = nullptr;
    les_ensemble* e = new les_ensemble();
    e->device = device;
    les_status st = LES_OK;
    for (int i = 0; i < count && !st; ++i) {
        les_ctx* c = nullptr;
        st = les_create(&meshes[i], device, &c);
        if (!st) {
            // cases run side by side on their own streams: a dependent launch
            // would hold SM slots waiting for its predecessor that other
            // cases' kernels could use (measured: 16-38 % slower steps)
            c->pdl = 0;
            e->cs.push_back(c);
        }
    }
    if (!st) {
        cudaSetDevice(device);
        st = ecuda(e, cudaStreamCreateWithFlags(&e->main, cudaStreamNonBlocking), "ensemble stream");
        if (!st) st = ecuda(e, cudaEventCreateWithFlags(&e->ev, cudaEventDisableTiming), "ensemble event");
    }
    if (st) {
        les_ensemble_destroy(e);
        return st;
    }
    *out = e;
    return LES_OK;
}

void les_ensemble_destroy(les_ensemble* e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->main) cudaStreamSynchronize(e->main);
    graph_clear(e->g[0]);
    graph_clear(e->g[1]);
    for (les_ctx* c : e->cs) les_destroy(c);
    if (e->d_count) cudaFree(e->d_count);
    if (e->ev) cudaEventDestroy(e->ev);
    if (e->main) cudaStreamDestroy(e->main);
    delete e;
}

int les_ensemble_size(const les_ensemble* e) { return e ? (int)e->cs.size() : 0; }

les_ctx* les_ensemble_case(les_ensemble* e, int i)
{
    if (!e || i < 0 || i >= (int)e->cs.size()) return nullptr;
    return e->cs[i];
}

const char* les_ensemble_last_error(const les_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

les_status les_ensemble_step(les_ensemble* e, const les_step_params* prm, les_step_stats* stats)
{
    if (!e || !prm) return LES_BAD_ARG;
    cudaSetDevice(e->device);
    const size_t n = e->cs.size();
    for (size_t i = 0; i < n; ++i) {
        if (prm[i].solver < LES_SOLVER_PCG || prm[i].solver > LES_SOLVER_GS_SOR) return LES_BAD_ARG;
        if (!graph_eligible(e->cs[i], &prm[i]))
            return efail(e, LES_BAD_ARG, "case " + std::to_string(i) +
                                             ": an ensemble step needs the mixed-precision fused PCG (Jacobi or "
                                             "Chebyshev) on a device-built matrix, with profiling off");
    }
    // order after any per-case work already queued on the cases' streams
    les_status st;
    for (les_ctx* c : e->cs) {
        if ((st = ecuda(e, cudaEventRecord(e->ev, c->stream), "order"))) return st;
        if ((st = ecuda(e, cudaStreamWaitEvent(e->main, e->ev, 0), "order wait"))) return st;
    }
    les_ensemble::Graph* g = graph_matches(e, e->g[0], prm) ? &e->g[0] : (graph_matches(e, e->g[1], prm) ? &e->g[1] : nullptr);
    bool fresh = false;
    if (!g) {
        int k = !same_params(e, e->g[0], prm) ? 0 : (!same_params(e, e->g[1], prm) ? 1 : e->last ^ 1);
        graph_clear(e->g[k]);
        if ((st = capture(e, prm, e->g[k]))) return st;
        g = &e->g[k];
        fresh = true;
    }
    if ((st = ecuda(e, cudaGraphLaunch(g->exec, e->main), "launch ensemble graph"))) return st;
    e->last = g == &e->g[0] ? 0 : 1;
    // later per-case calls on the cases' own streams come after the step
    if ((st = ecuda(e, cudaEventRecord(e->ev, e->main), "step done"))) return st;
    for (les_ctx* c : e->cs) {
        if ((st = ecuda(e, cudaStreamWaitEvent(c->stream, e->ev, 0), "step done wait"))) return st;
        if (!fresh) swap_velocity(c);
    }
    if (!stats) {
        for (size_t i = 0; i < n; ++i) e->cs[i]->launches += g->captured[i];
        return LES_OK;
    }
    // every case's solver state with one synchronisation (pinned mirrors)
    for (size_t i = 0; i < n && !st; ++i)
        st = ecuda(e, cudaMemcpyAsync(e->cs[i]->h_state, e->cs[i]->state, 2 * sizeof(SolverState),
                                      cudaMemcpyDeviceToHost, e->main),
                   "read states");
    if (st) return st;
    if ((st = ecuda(e, cudaStreamSynchronize(e->main), "ensemble step"))) return st;
    for (size_t i = 0; i < n; ++i) {
        les_ctx* c = e->cs[i];
        const unsigned long long run = graph_step_stats(c, &prm[i], g->captured[i], &stats[i]);
        c->launches += g->batched ? g->captured[i] : run;
    }
    if (g->batched && e->d_count) {   // the batched kernels, counted on the device, go to case 0
        unsigned long long k = 0;
        if ((st = ecuda(e, cudaMemcpy(&k, e->d_count, sizeof k, cudaMemcpyDeviceToHost), "launch count"))) return st;
        if ((st = ecuda(e, cudaMemset(e->d_count, 0, sizeof k), "launch count"))) return st;
        e->cs[0]->launches += k;
    }
    return LES_OK;
}

int les_ensemble_batch_split(const les_ensemble* e) { return e ? e->split : 0; }

les_status les_ensemble_set_batched(les_ensemble* e, int on)
{
    if (!e) return LES_BAD_ARG;
    e->batched = on ? 1 : 0;   // the step graphs are captured again in the new form
    return LES_OK;
}

les_status les_ensemble_sync(les_ensemble* e)
{
    if (!e) return LES_BAD_ARG;
    cudaSetDevice(e->device);
    return ecuda(e, cudaStreamSynchronize(e->main), "ensemble sync");
}

}  // extern "C"
