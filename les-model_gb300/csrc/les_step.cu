// les_step.cu -- one time step of les-model's loop body (src/main.cpp:115-144)
// on the device: dt, SGS + nu_t BCs, momentum (+ swap), velocity BCs,
// pressure solve, projection, velocity BCs.  Statistics and VTK output
// (:152-164) stay with the caller.
#include <cmath>
#include <cstring>
#include <utility>

#include "les_internal.cuh"
#include "les_mixed.cuh"

using namespace les;

namespace les {
les_status velocity_bcs_dev(les_ctx* c);
les_status sgs_nut_dev(les_ctx* c, double cs, int want_tau);
les_status momentum_dev(les_ctx* c, double dt, double nu, const double* dtp);
les_status sgs_nut32_dev(les_ctx* c, double cs);
les_status momentum32_dev(les_ctx* c, double dt, double nu, const double* dtp);
les_status correct_dev(les_ctx* c, double dt, double rho, const double* dtp);
les_status adaptive_dt_dev(les_ctx* c, double nu, double cfl_conv, double cfl_visc, double dt_max);
les_status div_b_dev(les_ctx* c, double dt, double rho, double rel_tol, const double* dtp);
les_status pcg_fp64(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status pcg_mixed_impl(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status solve_jacobi_dev(les_ctx* c, double dt, double rho, int max_iter, double tol, int* sweeps);
les_status solve_gs_dev(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps);
}

// ---- the time step as a CUDA graph -------------------------------------------
// With the mixed-precision fused PCG every decision of a step can be taken on
// the device: dt comes from the CFL reduction through a device pointer, and
// both solver loops are conditional graph nodes (les_fused.cu).  The whole
// step is captured once per velocity-buffer parity (the momentum update swaps
// u and u_new, and a graph holds fixed pointers) and replayed with one launch.
namespace les {

struct StepGraph {
    les_step_params prm{};
    double* slots[LES_NSLOTS] = {};
    double* tau = nullptr;
    int phys32 = 0;
    unsigned long long version = 0;
    cudaGraphExec_t exec = nullptr;
    unsigned long long captured = 0;   // kernel nodes outside and inside one pass of each loop
};

void step_graph_free(StepGraph* s)
{
    if (!s) return;
    if (s->exec) cudaGraphExecDestroy(s->exec);
    delete s;
}

bool graph_eligible(const les_ctx* c, const les_step_params* prm)
{
    return !c->prof_on && prm->solver == LES_SOLVER_PCG && prm->pcg.precision == LES_MIXED &&
           c->stencil_mode == 1 && c->fused && fused_supported(&prm->pcg) && prm->pcg.max_iter > 0;
}

// FP32 physics (les_physics32.cu) for a step of the mixed-precision solve
bool phys32_on(const les_ctx* c, const les_step_params* prm)
{
    return c->phys32 && prm->solver == LES_SOLVER_PCG && prm->pcg.precision == LES_MIXED && !prm->want_tau;
}

// nu_t (with its boundary values) and the momentum update of one step
les_status physics_dev(les_ctx* c, const les_step_params* prm, double dt, const double* dtp)
{
    les_status st;
    if (phys32_on(c, prm)) {
        if ((st = sgs_nut32_dev(c, prm->cs))) return st;
        return momentum32_dev(c, dt, prm->nu, dtp);
    }
    if ((st = sgs_nut_dev(c, prm->cs, prm->want_tau))) return st;
    return momentum_dev(c, dt, prm->nu, dtp);
}

void swap_velocity(les_ctx* c)
{
    std::swap(c->slot[LES_U], c->slot[LES_U_NEW]);
    std::swap(c->slot[LES_V], c->slot[LES_V_NEW]);
    std::swap(c->slot[LES_W], c->slot[LES_W_NEW]);
}

// Statistics of the step a graph ran, from the device state (after a sync);
// returns the number of kernels that ran (captured = the kernels captured:
// those outside the loops and one pass of each loop body).
unsigned long long graph_step_stats(les_ctx* c, const les_step_params* prm, unsigned long long captured,
                                    les_step_stats* stats)
{
    const SolverState& o = c->h_state[0];
    les_step_stats s{};
    s.dt = prm->dt_fixed > 0 ? prm->dt_fixed : o.scal[0];
    s.iters = o.iters;
    s.outer = o.k;
    s.residual = o.err;
    s.b_norm = o.bnorm;
    s.status = o.done ? (les_status)o.status : LES_NOT_CONVERGED;
    if (stats) *stats = s;
    // less one pass of each loop body, plus 8 kernels per outer correction
    // and 4 * INNER_BODY_PAIRS + 1 per pass of the inner body (passes counted
    // approximately: a correction's first iteration is outside the loop)
    const long long per = 4LL * INNER_BODY_PAIRS + 1, len = 2LL * INNER_BODY_PAIRS;
    const long long body = (o.iters - o.k + (len / 2) * o.k) / len;
    const long long run = (long long)captured - (8 + per) + 8LL * o.k + per * (body > 0 ? body : 0);
    return run > 0 ? (unsigned long long)run : captured;
}

}  // namespace les

static bool graph_matches(const les_ctx* c, const StepGraph* s, const les_step_params* prm)
{
    return s && s->exec && s->version == c->version && s->tau == c->tau && s->phys32 == c->phys32 &&
           std::memcmp(&s->prm, prm, sizeof *prm) == 0 && std::memcmp(s->slots, c->slot, sizeof s->slots) == 0;
}

// dt of a captured step: fixed, or read by the kernels from the CFL reduction
static double step_dt(les_ctx* c, const les_step_params* prm, const double** dtp)
{
    *dtp = prm->dt_fixed > 0 ? nullptr : &c->state[0].scal[0];   // nothing else in the step writes it
    return prm->dt_fixed > 0 ? prm->dt_fixed : 1.0;                // (1.0 unused: the kernels read *dtp)
}

// One step (src/main.cpp:115-144) into the capture in progress on c->stream,
// in three parts: up to the pressure solve's first defect, the solve, and
// the projection (an ensemble solves its cases together between the parts).
les_status les::emit_step_pre(les_ctx* c, const les_step_params* prm, bool outer_start)
{
    les_status st;
    const double* dtp;
    const double dt = step_dt(c, prm, &dtp);
    if (dtp && (st = adaptive_dt_dev(c, prm->nu, prm->cfl_conv, prm->cfl_visc, prm->dt_max))) return st;
    if ((st = physics_dev(c, prm, dt, dtp))) return st;
    if ((st = velocity_bcs_dev(c))) return st;
    if ((st = div_b_dev(c, dt, prm->rho, prm->rel_tol, dtp))) return st;
    return outer_start ? emit_outer_start(c, &prm->pcg, prm->rel_tol > 0 ? 1 : 0) : LES_OK;
}

les_status les::emit_step_post(les_ctx* c, const les_step_params* prm)
{
    les_status st;
    const double* dtp;
    const double dt = step_dt(c, prm, &dtp);
    if ((st = correct_dev(c, dt, prm->rho, dtp))) return st;
    return velocity_bcs_dev(c);
}

les_status les::emit_step(les_ctx* c, const les_step_params* prm)
{
    les_status st;
    if ((st = emit_step_pre(c, prm, false))) return st;
    // the fields final before the solve may leave now (les_step_io)
    if (c->ev_pre && (st = check_cuda(c, cudaEventRecordWithFlags(c->ev_pre, c->stream, cudaEventRecordExternal),
                                      "step event")))
        return st;
    if ((st = capture_mixed_fused(c, &prm->pcg, view32_of(c), prm->rel_tol > 0 ? 1 : 0))) return st;
    return emit_step_post(c, prm);
}

// les_step_io's early downloads: after the event that follows the step's
// physics, on the context's copy stream, from the slots as they are mapped
// after the step (the velocity buffers swapped)
static les_status early_downloads(les_ctx* c)
{
    if (!c->n_early) return LES_OK;
    const size_t bytes = sizeof(double) * (size_t)c->g.n;
    les_status st = check_cuda(c, cudaStreamWaitEvent(c->io_stream, c->ev_pre, 0), "early download wait");
    for (int q = 0; q < c->n_early && !st; ++q)
        st = check_cuda(c, cudaMemcpyAsync(c->early_host[q], c->slot[c->early_slot[q]], bytes, cudaMemcpyDeviceToHost,
                                           c->io_stream),
                        "early download");
    return st;
}

static les_status step_graph(les_ctx* c, const les_step_params* prm, les_step_stats* stats)
{
    les_status st = ensure_work(c);
    if (!st) st = ensure_work32(c);
    if (st) return st;
    StepGraph* g = graph_matches(c, c->sg[0], prm) ? c->sg[0] : (graph_matches(c, c->sg[1], prm) ? c->sg[1] : nullptr);
    bool fresh = false;
    if (!g) {
        // capture into an empty or stale slot, else replace the graph not used last
        int k = -1;
        for (int q = 0; q < 2 && k < 0; ++q)
            if (!c->sg[q] || c->sg[q]->version != c->version || c->sg[q]->phys32 != c->phys32 ||
                std::memcmp(&c->sg[q]->prm, prm, sizeof *prm) != 0)
                k = q;
        if (k < 0) k = c->sg_last ^ 1;
        step_graph_free(c->sg[k]);
        c->sg[k] = g = new StepGraph();
        g->prm = *prm;
        std::memcpy(g->slots, c->slot, sizeof g->slots);
        g->version = c->version;
        g->phys32 = c->phys32;
        double* before[LES_NSLOTS];
        std::memcpy(before, c->slot, sizeof before);
        const unsigned long long l0 = c->launches;
        cudaGraph_t graph = nullptr;
        st = check_cuda(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed), "begin step capture");
        if (st) return st;
        les_status st1 = emit_step(c, prm);
        les_status st2 = check_cuda(c, cudaStreamEndCapture(c->stream, &graph), "end step capture");
        g->captured = c->launches - l0;
        c->launches = l0;
        g->tau = c->tau;
        if (!st1 && !st2)
            st1 = check_cuda(c, cudaGraphInstantiate(&g->exec, graph, 0), "instantiate step graph");
        if (graph) cudaGraphDestroy(graph);
        if (st1 || st2) {
            std::memcpy(c->slot, before, sizeof before);   // nothing ran: undo the capture's buffer swap
            step_graph_free(g);
            c->sg[k] = nullptr;
            return st1 ? st1 : st2;
        }
        fresh = true;
    }
    st = check_cuda(c, cudaGraphLaunch(g->exec, c->stream), "launch step graph");
    if (st) return st;
    c->sg_last = g == c->sg[0] ? 0 : 1;
    if (!fresh) swap_velocity(c);   // the capture swapped the host pointers once; a replay must too
    if ((st = early_downloads(c))) return st;
    if (!stats) {
        c->launches += g->captured;
        return LES_OK;
    }
    if ((st = read_state(c))) return st;
    c->launches += graph_step_stats(c, prm, g->captured, stats);
    return LES_OK;
}

static les_status step_impl(les_ctx* c, const les_step_params* prm, les_step_stats* stats);

extern "C" les_status les_step(les_ctx* c, const les_step_params* prm, les_step_stats* stats)
{
    if (!c || !prm) return LES_BAD_ARG;
    c->n_early = 0;
    return step_impl(c, prm, stats);
}

// Fields final when the pressure solve starts: nu_t, the solve's right-hand
// side and the u_new buffers (after the momentum update's swap they hold the
// step's incoming velocity, which nothing later writes)
static bool final_before_solve(int slot)
{
    return slot == LES_U_NEW || slot == LES_V_NEW || slot == LES_W_NEW || slot == LES_NU_T || slot == LES_P_RHS;
}

extern "C" les_status les_step_io(les_ctx* c, const les_step_params* prm, les_step_stats* stats, int n_in,
                                  const int* in_slots, const double* const* in_hosts, int n_out,
                                  const int* out_slots, double* const* out_hosts, double* step_ms)
{
    if (!c || !prm || n_in < 0 || n_out < 0 || n_out > LES_NSLOTS || (n_out > 0 && (!out_slots || !out_hosts)))
        return LES_BAD_ARG;
    if (prm->solver < LES_SOLVER_PCG || prm->solver > LES_SOLVER_GS_SOR) return LES_BAD_ARG;   // before any copy
    for (int q = 0; q < n_out; ++q)
        if (out_slots[q] < 0 || out_slots[q] >= LES_NSLOTS || !out_hosts[q]) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    les_status st = LES_OK;
    for (int q = 0; q < 2 && !st; ++q)
        if (!c->ev_io[q]) st = check_cuda(c, cudaEventCreate(&c->ev_io[q]), "step timing event");
    if (!st && !c->io_stream)
        st = check_cuda(c, cudaStreamCreateWithFlags(&c->io_stream, cudaStreamNonBlocking), "copy stream");
    // the uploads precede the step in the context's stream: no host wait
    if (!st && n_in > 0 && (!in_slots || !in_hosts)) return LES_BAD_ARG;
    for (int q = 0; q < n_in && !st; ++q)
        if (in_slots[q] < 0 || in_slots[q] >= LES_NSLOTS || !in_hosts[q]) return LES_BAD_ARG;
    const size_t bytes = sizeof(double) * (size_t)c->g.n;
    for (int q = 0; q < n_in && !st; ++q)
        st = check_cuda(c, cudaMemcpyAsync(c->slot[in_slots[q]], in_hosts[q], bytes, cudaMemcpyHostToDevice, c->stream),
                        "field upload");
    if (st) {
        cudaStreamSynchronize(c->stream);
        return st;
    }
    // the downloads of fields final before the solve overlap it (PCG steps);
    // the others follow the step
    c->n_early = 0;
    int late_slot[LES_NSLOTS];
    double* late_host[LES_NSLOTS];
    int n_late = 0;
    for (int q = 0; q < n_out; ++q) {
        if (prm->solver == LES_SOLVER_PCG && final_before_solve(out_slots[q])) {
            c->early_slot[c->n_early] = out_slots[q];
            c->early_host[c->n_early++] = out_hosts[q];
        } else {
            late_slot[n_late] = out_slots[q];
            late_host[n_late++] = out_hosts[q];
        }
    }
    st = check_cuda(c, cudaEventRecord(c->ev_io[0], c->stream), "step timing event");
    if (!st) st = step_impl(c, prm, stats);
    c->n_early = 0;
    les_status st2 = check_cuda(c, cudaEventRecord(c->ev_io[1], c->stream), "step timing event");
    for (int q = 0; q < n_late && !st && !st2; ++q)
        st2 = check_cuda(c, cudaMemcpyAsync(late_host[q], c->slot[late_slot[q]], bytes, cudaMemcpyDeviceToHost,
                                            c->stream),
                         "field download");
    les_status s1 = check_cuda(c, cudaStreamSynchronize(c->io_stream), "copy stream sync");
    les_status s2 = check_cuda(c, cudaStreamSynchronize(c->stream), "step sync");
    if (!st && !st2 && !s1 && !s2 && step_ms) {
        float ms = 0.f;
        st2 = check_cuda(c, cudaEventElapsedTime(&ms, c->ev_io[0], c->ev_io[1]), "step time");
        *step_ms = ms;
    }
    return st ? st : (st2 ? st2 : (s1 ? s1 : s2));
}

static les_status step_impl(les_ctx* c, const les_step_params* prm, les_step_stats* stats)
{
    if (!c || !prm) return LES_BAD_ARG;
    if (prm->solver < LES_SOLVER_PCG || prm->solver > LES_SOLVER_GS_SOR) return LES_BAD_ARG;
    if (prm->solver == LES_SOLVER_PCG && !c->stencil_mode)
        return fail(c, LES_BAD_ARG, "PCG needs a matrix: call les_build_stencil first");
    cudaSetDevice(c->device);
    if (c->graph_on && graph_eligible(c, prm)) return step_graph(c, prm, stats);
    les_status st;
    double dt = prm->dt_fixed;
    if (!(dt > 0)) {
        st = adaptive_dt_dev(c, prm->nu, prm->cfl_conv, prm->cfl_visc, prm->dt_max);
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        dt = c->h_state[0].scal[0];
    }
    if ((st = physics_dev(c, prm, dt, nullptr))) return st;
    if ((st = velocity_bcs_dev(c))) return st;
    les_status solve = LES_OK;
    les_step_stats s{};
    s.dt = dt;
    if (prm->solver == LES_SOLVER_PCG) {
        if ((st = div_b_dev(c, dt, prm->rho, prm->rel_tol, nullptr))) return st;
        if (c->n_early) {
            if ((st = check_cuda(c, cudaEventRecord(c->ev_pre, c->stream), "step event"))) return st;
            if ((st = early_downloads(c))) return st;
        }
        les_pcg_result r{};
        const int keep = prm->rel_tol > 0 ? 1 : 0;
        if (prm->pcg.precision == LES_MIXED) solve = pcg_mixed_impl(c, &prm->pcg, &r, keep);
        else solve = pcg_fp64(c, &prm->pcg, &r, keep);
        if (solve != LES_OK && solve != LES_NOT_CONVERGED && solve != LES_NONFINITE) return solve;
        s.iters = r.iters;
        s.outer = r.outer;
        s.residual = r.residual;
        s.b_norm = c->h_state[0].bnorm;
    } else if (prm->solver == LES_SOLVER_JACOBI) {
        solve = solve_jacobi_dev(c, dt, prm->rho, prm->stat_max_iter, prm->stat_tol, &s.iters);
        if (solve != LES_OK) return solve;
    } else {
        solve = solve_gs_dev(c, dt, prm->rho, prm->stat_max_iter, prm->omega, prm->stat_tol, &s.iters);
        if (solve != LES_OK) return solve;
    }
    if ((st = correct_dev(c, dt, prm->rho, nullptr))) return st;
    if ((st = velocity_bcs_dev(c))) return st;
    s.status = solve;
    if (stats) *stats = s;
    return LES_OK;
}
