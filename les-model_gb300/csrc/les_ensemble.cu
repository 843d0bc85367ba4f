// les_ensemble.cu -- many independent cases of uneven grid sizes advanced by
// one CUDA graph launch per time step.
//
// Each case is an ordinary context (its own fields, matrix, solver state and
// work vectors).  A step of the ensemble is captured once per velocity-buffer
// parity: the capture forks from the ensemble's stream into every case's
// stream, emits that case's whole step there (device dt, both mixed-precision
// solver loops as conditional nodes), and joins back, so the graph holds one
// independent branch per case and the cases' kernels overlap on the GPU.
// Replays launch that one graph; a case that converges early ends its branch
// early.  The cases are independent units: across GPUs they would be
// partitioned with no exchange.
#include <cstring>
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
    struct Graph {
        std::vector<les_step_params> prm;
        std::vector<double*> slots;       // LES_NSLOTS per case
        std::vector<double*> tau;
        std::vector<unsigned long long> version, captured;
        cudaGraphExec_t exec = nullptr;
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
    g = les_ensemble::Graph{};
}

bool graph_matches(const les_ensemble* e, const les_ensemble::Graph& g, const les_step_params* prm)
{
    if (!g.exec) return false;
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
    if (!g.exec) return false;
    for (size_t i = 0; i < e->cs.size(); ++i)
        if (g.version[i] != e->cs[i]->version || std::memcmp(&g.prm[i], &prm[i], sizeof(les_step_params)) != 0)
            return false;
    return true;
}

les_status capture(les_ensemble* e, const les_step_params* prm, les_ensemble::Graph& g)
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

}  // namespace

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
    if ((st = ecuda(e, cudaStreamSynchronize(e->main), "ensemble step"))) return st;
    for (size_t i = 0; i < n; ++i) {
        les_ctx* c = e->cs[i];
        if ((st = read_state(c))) return efail(e, st, "case " + std::to_string(i) + ": " + c->err);
        c->launches += graph_step_stats(c, &prm[i], g->captured[i], &stats[i]);
    }
    return LES_OK;
}

les_status les_ensemble_sync(les_ensemble* e)
{
    if (!e) return LES_BAD_ARG;
    cudaSetDevice(e->device);
    return ecuda(e, cudaStreamSynchronize(e->main), "ensemble sync");
}

}  // extern "C"
