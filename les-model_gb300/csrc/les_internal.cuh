// les_internal.cuh -- shared device helpers and the context layout of the
// GB300 les-model hot path.  Not part of the ABI.
//
// Layout in HBM: every field is one FP64 array of N = nx*ny*nz cells in the
// reference order idx = i*ny*nz + j*nz + k (src/field.h:40), k contiguous.
// The obstacle mask is one byte per cell.  The assembled matrix is kept as one
// byte per cell (a stencil code, decoded to exact coefficients in registers)
// when it was built on the device by les_build_stencil, or as seven FP64
// diagonals when a caller installs an arbitrary matrix.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "les_gb300.h"

namespace les {

struct TmaCache;                       // tensor maps of the fused passes (les_fused.cu)
void tma_cache_free(TmaCache* t);
struct StepGraph;                      // captured time step (les_step.cu)
void step_graph_free(StepGraph* s);
struct AdjWork;                        // adjoint checkpoints and work vectors (les_adjoint.cu)
void adj_work_free(AdjWork* a);
struct IoWork;                         // statistics sums, file staging and writer thread (les_io.cu)
void io_work_free(IoWork* w);

// ---- geometry -------------------------------------------------------------
struct Geo {
    int nx, ny, nz;
    int n;        // nx*ny*nz (< 2^31)
    int si, sj;   // strides of i and j
};

// Stencil block shape for per-cell kernels: 32 k x 8 j threads, grid.z = i.
constexpr int TBK = 32;
constexpr int TBJ = 8;

inline dim3 cell_grid(const Geo& g) { return dim3((g.nz + TBK - 1) / TBK, (g.ny + TBJ - 1) / TBJ, g.nx); }
inline dim3 cell_block() { return dim3(TBK, TBJ, 1); }

// ---- stencil codes ---------------------------------------------------------
// Code 0: identity row (solid cell or outlet, src/pressure.cpp:634-642).
// Otherwise code-1 = xs + 5*(ys + 4*zs) where each state selects the
// multiplier of the base coefficient for the two neighbours of one axis after
// the ghost-doubling of src/pressure.cpp:663-696:
//   x (w,e): 0:(1,1) 1:(0,2) 2:(1,0) 3:(0,0) 4:(2,0)
//   y (s,n) and z (b,t): 0:(1,1) 1:(0,2) 2:(2,0) 3:(1,0)
// Multipliers are packed two bits per state.
constexpr unsigned XW_PACK = 1u | (0u << 2) | (1u << 4) | (0u << 6) | (2u << 8);
constexpr unsigned XE_PACK = 1u | (2u << 2) | (0u << 4) | (0u << 6) | (0u << 8);
constexpr unsigned YL_PACK = 1u | (0u << 2) | (2u << 4) | (1u << 6);  // s / b
constexpr unsigned YH_PACK = 1u | (2u << 2) | (0u << 4) | (0u << 6);  // n / t

// Exact coefficient values: c0 = 2/dx^2 + 2/dy^2 + 2/dz^2 summed in the
// reference's order, m1 = -1/h^2, m2 = m1 + m1 per axis.
struct StencilCoef {
    double c0;
    double x1, x2, y1, y2, z1, z2;
};

struct Coef7 {
    double c, w, e, s, n, b, t;
};

__device__ __forceinline__ double sel(unsigned m, double v1, double v2)
{
    return m == 0u ? 0.0 : (m == 1u ? v1 : v2);
}

__device__ __forceinline__ Coef7 decode(unsigned code, const StencilCoef& k)
{
    Coef7 a;
    if (code == 0u) {
        a.c = 1.0; a.w = a.e = a.s = a.n = a.b = a.t = 0.0;
        return a;
    }
    unsigned c = code - 1u;
    unsigned xs = c % 5u, r = c / 5u;
    unsigned ys = r & 3u, zs = r >> 2;
    a.c = k.c0;
    a.w = sel((XW_PACK >> (2 * xs)) & 3u, k.x1, k.x2);
    a.e = sel((XE_PACK >> (2 * xs)) & 3u, k.x1, k.x2);
    a.s = sel((YL_PACK >> (2 * ys)) & 3u, k.y1, k.y2);
    a.n = sel((YH_PACK >> (2 * ys)) & 3u, k.y1, k.y2);
    a.b = sel((YL_PACK >> (2 * zs)) & 3u, k.z1, k.z2);
    a.t = sel((YH_PACK >> (2 * zs)) & 3u, k.z1, k.z2);
    return a;
}

// Float twin for the FP32 inner solve (values rounded once from the FP64 ones).
struct StencilCoefF {
    float c0, x1, x2, y1, y2, z1, z2;
};

// Source of the seven diagonals: either codes (decoded) or stored arrays.
struct StencilView {
    const uint8_t* code;       // non-null: coded mode
    StencilCoef k;
    const double* d[7];        // stored mode: c, n, s, e, w, t, b
    __device__ __forceinline__ Coef7 at(int id) const
    {
        if (code) return decode(code[id], k);
        Coef7 a;
        a.c = d[0][id]; a.n = d[1][id]; a.s = d[2][id]; a.e = d[3][id];
        a.w = d[4][id]; a.t = d[5][id]; a.b = d[6][id];
        return a;
    }
    __device__ __forceinline__ double diag(int id) const
    {
        if (code) return code[id] == 0 ? 1.0 : k.c0;
        return d[0][id];
    }
};

// ---- deterministic block reductions -----------------------------------------
template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV])
{
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
}

// Sums v over the block (fixed order); the result is valid in thread 0.
// smem: NV*32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem)
{
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5, nw = (nthr + 31) >> 5;
    warp_sum<NV>(v);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) smem[q * 32 + warp] = v[q];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = lane < nw ? smem[q * 32 + lane] : 0.0;
        warp_sum<NV>(v);
    }
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int block_linear_id() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ int block_count() { return gridDim.x * gridDim.y * gridDim.z; }

// Two-stage deterministic sum: each block stores its partial; the block that
// arrives last sums all partials in block order.  Returns true in every
// thread of the last block, with the totals valid in its thread 0.
// (bid, nb): this block's index among the nb blocks that share the
// reduction -- the whole grid, or one case's blocks of a batched launch.
template <int NV>
__device__ bool last_block_sum(double (&v)[NV], double* partials, unsigned* counter, double* smem, int bid, int nb)
{
    __shared__ int am_last;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    block_sum<NV>(v, smem);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) partials[q * nb + bid] = v[q];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        am_last = (t == (unsigned)nb - 1u);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0.0;
    for (int b = tid; b < nb; b += nthr)
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] += __ldcg(partials + q * nb + b);
    block_sum<NV>(acc, smem);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = acc[q];
        *counter = 0u;
    }
    return true;
}

template <int NV>
__device__ bool last_block_sum(double (&v)[NV], double* partials, unsigned* counter, double* smem)
{
    return last_block_sum<NV>(v, partials, counter, smem, block_linear_id(), block_count());
}

// ---- device-resident solver state -----------------------------------------
struct SolverState {
    double rho, alpha, beta, err, tol, pq, rr, rz, bnorm, maxdp;
    double scal[8];   // misc scalars (dt, lambda, ...)
    int k, done, iters, max_iter, status, buf;
    int frozen;       // column passes under the autotuner: zero alpha and beta, no end
    int pad1;
    double rho_next;  // the column passes' rho, handed from pass A to pass B
};

// ---- bounded grid barrier for cooperative (co-resident) launches ------------
struct GridSync {
    unsigned* count;
    unsigned* gen;
    int* error;       // set to 1 when a wait gives up
    unsigned nblocks;
};

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false (in every thread) once any block has given up waiting; the
// caller then leaves the kernel.  A wait gives up after ~2 s.
__device__ __forceinline__ bool grid_barrier(const GridSync& gs)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        volatile unsigned* vgen = gs.gen;
        volatile int* verr = gs.error;
        unsigned my_gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(gs.count, 1u);
        int good = 1;
        if (arrived == gs.nblocks - 1u) {
            *gs.count = 0u;
            __threadfence();
            atomicAdd(gs.gen, 1u);
        } else {
            unsigned long long t0 = globaltimer_ns();
            unsigned spins = 0;
            while (*vgen == my_gen) {
                if (*verr) { good = 0; break; }
                if ((++spins & 255u) == 0u && globaltimer_ns() - t0 > 2000000000ull) {
                    atomicExch(gs.error, 1);
                    good = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (*verr) good = 0;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace les

// ---- the context -------------------------------------------------------------
struct les_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    les_mesh mesh{};
    les::Geo g{};
    double* slot[LES_NSLOTS] = {};
    uint8_t* mask = nullptr;
    int* solid_list = nullptr;    // interior solid cells (for obstacle BC passes)
    int n_solid = 0;
    // matrix
    int stencil_mode = 0;         // 0 none, 1 coded, 2 stored
    bool code_plain = false;      // coded matrix built from a solid-free mask: every code is a
                                  // function of the cell's position
    uint8_t* code = nullptr;
    double* A[7] = {};
    bool A_valid = false;         // A[] holds the current matrix (stored, or expanded codes)
    int fused = 1;                // LES_OPT_FUSED: fused FP32 inner passes
    int opt_tma = 0;              // LES_OPT_TMA: TMA-staged fused passes where the grid allows
    int tune_cia = 0, tune_cib = 0, tune_s = -1;   // autotuned march chunk lengths (0: occupancy rule)
    int tune_tja = 0, tune_tjb = 0;                // autotuned strip rows of the column passes (0: default)
    double share = 1.0;           // fraction of the GPU's resident warps the column passes size
                                  // their chunks for (1/k when k cases run together)
    struct les::TmaCache* tma = nullptr;
    les::StencilCoef coef{};
    double* L[7] = {};
    bool have_L = false;
    double* tau = nullptr;
    double* inlet = nullptr;      // inlet u profile (ny*nz) or nullptr for the reference's uniform 1
    struct les::AdjWork* adj = nullptr;   // adjoint checkpoints and work (les_adjoint.cu)
    struct les::IoWork* io = nullptr;     // statistics and file output (les_io.cu)
    // work vectors (FP64)
    double* w[8] = {};
    // FP32 work vectors for the mixed-precision inner solve, and FP32 copies
    // of a stored A / of the IC factor for it
    float* f[8] = {};
    float* A32[7] = {};
    float* L32[7] = {};
    // reductions / state
    double* partials = nullptr;
    size_t partials_len = 0;
    unsigned* counters = nullptr;  // 32 last-block counters (one per reduction site)
    les::SolverState* state = nullptr;
    les::SolverState* h_state = nullptr;  // pinned mirror
    unsigned* gsync = nullptr;            // count, gen, error
    // pipelined wavefronts (les_wavefront.cu): one progress counter per warp
    // tile, compared against a base that grows from launch to launch (reset
    // to zero when it nears the int range)
    int* wave_prog = nullptr;
    int wave_prog_len = 0;
    int wave_epoch = 0;
    std::string err;
    // accounting: kernel launches issued by this context, and optional CUDA
    // event timing of the solver's hot kernels (les_profile)
    unsigned long long launches = 0;
    int prof_on = 0;
    std::vector<cudaEvent_t> prof_ev;     // pool, two per recorded launch
    std::vector<int> prof_id;             // kernel id of each recorded pair
    std::vector<cudaEvent_t> marks;       // les_mark slots
    // CUDA-graph time steps (les_step.cu): one executable graph per velocity
    // buffer parity, rebuilt when anything baked into it changes
    int graph_on = 1;                     // LES_OPT_GRAPH
    int pdl = 1;                          // LES_OPT_PDL
    int phys32 = 1;                       // LES_OPT_PHYS32
    int test_stall = 0;                   // LES_OPT_TEST_STALL
    int col_stride = 1;                   // LES_OPT_COL_STRIDE
    cudaStream_t aux = nullptr;           // capture stream for conditional-loop bodies
    // les_step_io: an event recorded after the step's physics (before the
    // pressure solve; an external event node of the captured step), the
    // stream of the downloads it releases, and those downloads
    cudaEvent_t ev_pre = nullptr;
    cudaEvent_t ev_io[2] = {};            // the step's device time
    cudaStream_t io_stream = nullptr;
    int n_early = 0;
    int early_slot[LES_NSLOTS] = {};
    double* early_host[LES_NSLOTS] = {};
    struct les::StepGraph* sg[2] = {};
    int sg_last = 0;                      // slot of the graph launched last
    unsigned long long version = 0;       // bumped by every change a captured graph depends on
};

namespace les {

// Profiled kernel ids (les_profile_read).
enum ProfId {
    PROF_IN_CHEB = 0,   // FP32 inner Chebyshev step (mixed path)
    PROF_IN_SPMV = 1,   // FP32 inner SpMV + p update + p.q
    PROF_IN_UPDATE = 2, // FP32 inner e/r update + ||r|| (+ first preconditioner stage)
    PROF_SPMV64 = 3,    // FP64 SpMV + p.q
    PROF_UPDATE64 = 4,  // FP64 x/r update + ||r||
    PROF_CHEB64 = 5,    // FP64 Chebyshev step
    PROF_OUTER = 6,     // FP64 outer residual of the mixed path
    PROF_IC = 7,        // IC(0) wavefront apply
    PROF_N = 8
};

void prof_begin(les_ctx* c, int id, cudaEvent_t* e1);

template <typename... KArgs, typename... Args>
inline void launch(les_ctx* c, void (*k)(KArgs...), dim3 grid, dim3 block, Args... args)
{
    k<<<grid, block, 0, c->stream>>>(args...);
    ++c->launches;
}

// Same, with CUDA events around the launch while profiling is on.
template <typename... KArgs, typename... Args>
inline void launch_p(les_ctx* c, int pid, void (*k)(KArgs...), dim3 grid, dim3 block, Args... args)
{
    cudaEvent_t e1 = nullptr;
    if (c->prof_on) prof_begin(c, pid, &e1);
    k<<<grid, block, 0, c->stream>>>(args...);
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
}

// Same, as a programmatic dependent launch when c->pdl is set: the kernel may
// start while the kernel before it in the stream drains, so it must execute
// dep_wait() before its first access to device memory.
template <typename... KArgs, typename... Args>
inline void launch_pdl(les_ctx* c, int pid, void (*k)(KArgs...), dim3 grid, dim3 block, Args... args)
{
    cudaEvent_t e1 = nullptr;
    if (c->prof_on) prof_begin(c, pid, &e1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = c->pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
}

// Waits until the grids this one depends on have completed and their writes
// are visible (returns at once for a kernel launched in plain stream order).
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the dependent grid launch once every block has signalled or exited.
__device__ __forceinline__ void dep_signal() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace les

namespace les {

les_status fail(les_ctx* c, les_status st, const std::string& msg);
les_status check_cuda(les_ctx* c, cudaError_t e, const char* what);
les_status check_launch(les_ctx* c, const char* what);
StencilView stencil_view(const les_ctx* c);
les_status ensure_work(les_ctx* c);
les_status ensure_work32(les_ctx* c);

// graph-captured time steps (les_step.cu)
bool graph_eligible(const les_ctx* c, const les_step_params* prm);
les_status emit_step(les_ctx* c, const les_step_params* prm);   // into the capture on c->stream
// the step before the pressure solve (with its first FP64 defect when
// outer_start) and after it
les_status emit_step_pre(les_ctx* c, const les_step_params* prm, bool outer_start);
les_status emit_step_post(les_ctx* c, const les_step_params* prm);
void swap_velocity(les_ctx* c);
unsigned long long graph_step_stats(les_ctx* c, const les_step_params* prm, unsigned long long captured,
                                    les_step_stats* stats);
les_status read_state(les_ctx* c);
int reduction_blocks(const Geo& g);

// kernels shared across translation units (les_pressure.cu)
les_status spmv_dev(les_ctx* c, const double* in, double* out);
les_status dot_dev(les_ctx* c, const double* a, const double* b, double* out_host);

}  // namespace les
