// les_wavefront.cu -- the three lexicographically ordered loops of les-model
// src/pressure.cpp on the device: the IC(0) factorisation (:495-556), the
// IC forward/backward substitution (:442-482) and the GS-SOR sweep
// (:212-246).
//
// Each cell of these loops depends only on its (i-1), (j-1), (k-1)
// neighbours (the backward solve: on i+1, j+1, k+1), so any order that
// computes a cell after those neighbours performs exactly the same
// floating-point operations on exactly the same operand values as the serial
// lexicographic loop: the results are bit-identical to the reference.
//
// The substitution and the SOR sweep run as a pipelined wavefront with no
// grid barrier inside a sweep.  The (j, k) plane is cut into tiles of TJ rows
// by 32 columns; a block of TJ warps owns a tile and marches along i, warp w
// on the tile's row w and lane l on column l, working at block step tau on
// plane tau - l - w (lanes and warps skewed by one plane each).  So the k-1
// neighbour of a cell is the previous lane's result of the step before (a
// warp shuffle), the j-1 neighbour the previous warp's result of the step
// before (shared memory, one block barrier per step), and the i-1 neighbour
// the thread's own result of the step before.  The rows of a tile run on the
// SM's four sub-partitions at once: a single warp would push all of them
// through one sub-partition's FP64 unit.  Only a tile's first row and first
// lane need other tiles' values: the tile below in j and the tile before in
// k publish their progress (steps completed, one counter per tile, release
// store after a fence) every WB steps, and a block waits (acquire load,
// bounded by %globaltimer) for the progress its next WB steps need, then
// reads those neighbours through L2.  The backward solve mirrors every
// direction.  Tiles are handed out to the resident blocks in an order in
// which each tile's producers come first, so the waits always end.
// The IC factorisation (set-up, once) keeps the simpler form: hyperplanes
// i+j+k = s in order, one grid barrier between them.  Every wait is bounded
// (about 2 s); a wait that gives up sets an error flag, every warp leaves,
// and the host reports LES_TIMEOUT.  Compiled with -fmad=false.
#include <cmath>

#include "les_internal.cuh"

using namespace les;

namespace {

struct Plane {
    int nx, ny, nz, si, sj;
};

__device__ __forceinline__ int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int gthreads() { return gridDim.x * blockDim.x; }

// IC(0) factorisation, src/pressure.cpp:506-555, hyperplane by hyperplane.
// L arrays must be zero on entry (fresh matrix semantics).
__global__ void k_ic_build(Plane P, StencilView A, double* Lc, double* Lw, double* Ls, double* Lb,
                           GridSync gs)
{
    const double small_val = 1e-30;
    const int smax = P.nx + P.ny + P.nz - 3;
    const int njk = P.ny * P.nz;
    for (int s = 0; s <= smax; ++s) {
        for (int t = gtid(); t < njk; t += gthreads()) {
            int j = t / P.nz, k = t - j * P.nz;
            int i = s - j - k;
            if (i < 0 || i >= P.nx) continue;
            int id = i * P.si + j * P.sj + k;
            Coef7 a = A.at(id);
            double sum_sq = 0.0;
            if (i > 0) {
                double lc = __ldcg(Lc + id - P.si);
                if (fabs(lc) > small_val) { double l = a.w / lc; Lw[id] = l; sum_sq += l * l; }
            }
            if (j > 0) {
                double lc = __ldcg(Lc + id - P.sj);
                if (fabs(lc) > small_val) { double l = a.s / lc; Ls[id] = l; sum_sq += l * l; }
            }
            if (k > 0) {
                double lc = __ldcg(Lc + id - 1);
                if (fabs(lc) > small_val) { double l = a.b / lc; Lb[id] = l; sum_sq += l * l; }
            }
            double diag = a.c - sum_sq;
            Lc[id] = (diag <= small_val) ? 1.0 : sqrt(diag);
        }
        if (!grid_barrier(gs)) return;
    }
}

// ---- pipelined wavefront -----------------------------------------------------
#ifndef LES_WAVE_WB
#define LES_WAVE_WB 4
#endif
#ifndef LES_WAVE_TJ
#define LES_WAVE_TJ 4
#endif
#ifndef LES_WAVE_WD
#define LES_WAVE_WD 8
#endif
constexpr int WB = LES_WAVE_WB;        // steps between progress publications
constexpr int WAVE_TJ = LES_WAVE_TJ;   // rows per tile = warps per block (one per SM sub-partition)
constexpr int WT = 32 * WAVE_TJ;

struct Wave {
    int nx, ny, nz, si, sj;    // the swept box (interior for GS-SOR) and the strides
    int off;                   // index of the box's first cell
    int wj, wk, ntiles;        // tiles along j and k
    int steps;                 // marching steps of a tile: planes + 31 lane skews + TJ-1 row skews
    int* prog;                 // progress counter per tile
    int* err;                  // set by a wait that gives up
    int stall;                 // tile that withholds its progress (LES_OPT_TEST_STALL), or -1
};

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One thread: waits until *p has reached target (wrap-safe); false once the
// wait gave up (~2 s) or another block raised the error flag.
__device__ bool wait_progress(const int* p, int target, int* err)
{
    if (ld_acquire(p) - target >= 0) return true;
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    for (;;) {
        if (ld_acquire(p) - target >= 0) return true;
        if (*(volatile int*)err) return false;
        if ((++spins & 63u) == 0u && globaltimer_ns() - t0 > 2000000000ull) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(32);
    }
}

// Max over the warp, the same value in every lane.
__device__ __forceinline__ double warp_max_all(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Publishes `value` as the tile's progress after every thread's stores.
__device__ __forceinline__ void publish(int* p, int value)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) st_release(p, value);
}

// Tile t's producers: DIR > 0 the tiles below in j (t-1) and before in k
// (t-wj); DIR < 0 the tiles above (t+1) and after (t+wj).
struct TileDeps {
    int dj, dk;
};

template <int DIR>
__device__ __forceinline__ TileDeps tile_deps(const Wave& W, int J, int K, int t)
{
    TileDeps d;
    if (DIR > 0) {
        d.dj = J > 0 ? t - 1 : -1;
        d.dk = K > 0 ? t - W.wj : -1;
    } else {
        d.dj = J < W.wj - 1 ? t + 1 : -1;
        d.dk = K < W.wk - 1 ? t + W.wj : -1;
    }
    return d;
}

// Waits for the progress a batch of steps [tau0, tend) needs.  A tile's row
// next to this one is its row TJ-1 (skewed TJ-1 steps behind its row 0), so
// the j-producer must be TJ-1 steps ahead; the k-producer's far lane reaches
// a plane 31 steps after its near lane.  Returns false in every thread when a
// wait gave up.
__device__ __forceinline__ bool wait_batch(const Wave& W, const TileDeps& d, int base, int tend, int* flag)
{
    if (threadIdx.x == 0) {
        int ok = 1;
        if (d.dj >= 0 && !wait_progress(W.prog + d.dj, base + min(tend + WAVE_TJ - 1, W.steps), W.err)) ok = 0;
        if (ok && d.dk >= 0 && !wait_progress(W.prog + d.dk, base + min(tend + 31, W.steps), W.err)) ok = 0;
        *flag = ok;
    }
    __syncthreads();
    return *flag != 0;
}

// ---- operand staging: every step's read-only (or not yet written) operands
// are copied into shared memory WD steps ahead with cp.async, so a step
// never waits on a global load; only the cross-tile neighbours (after the
// batch's wait) are read directly.
constexpr int WD = LES_WAVE_WD;   // steps staged ahead (a power of two)

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// A tile: rows jb.. of TJ rows (the last tile in j may have fewer) by the 32
// columns K*32..; warp w works on the tile's row w (in the sweep's order) and
// lane l on column K*32 + l.  At block step tau, warp w lane l works on plane
// tau - skew(l) - w (forward planes ascend, backward descend; skew(l) is l
// forward, 31-l backward), so:
//   the i-neighbour is the thread's own result of the step before,
//   the k-neighbour the previous lane's result of the step before (shuffle),
//   the j-neighbour the previous warp's result of the step before, handed
//   over in shared memory (double-buffered by step parity, one block barrier
//   per step); row 0 takes it from the tile before in j.
template <typename T>
struct IcStage {
    T v[WD][5][WAVE_TJ][32];   // rhs (forward r, backward the cell's forward result), Lw, Ls, Lb, Lc
    T xs[2][WAVE_TJ][32];      // each row's result of the last two steps
    int flag;
};

// IC(0) substitution of one tile, src/pressure.cpp:442-482.  DIR > 0: the
// forward solve L y = r (z = y); DIR < 0: the backward solve L^T z = y.
template <typename T, int DIR>
__device__ bool ic_tile(const Wave& W, int t, int base, const T* __restrict__ Lc, const T* __restrict__ Lw,
                        const T* __restrict__ Ls, const T* __restrict__ Lb, const T* __restrict__ r, T* z,
                        IcStage<T>& sg)
{
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int J = t % W.wj, K = t / W.wj;
    const int jb = J * WAVE_TJ, rows = min(WAVE_TJ, W.ny - jb);
    const int k = K * 32 + lane;
    const bool kin = k < W.nz;
    const int kc = min(k, W.nz - 1);                          // every address stays inside the grid
    const int sk = DIR > 0 ? lane : 31 - lane;
    const TileDeps d = tile_deps<DIR>(W, J, K, t);
    const bool wact = w < rows;                               // this warp's row exists
    // this warp's grid row (rows past the grid repeat the last one; dropped)
    const int jr = DIR > 0 ? jb + min(w, rows - 1) : jb + rows - 1 - min(w, rows - 1);
    const int rb = W.off + jr * W.sj + kc;
    const bool jin = DIR > 0 ? jr > 0 : jr < W.ny - 1;        // the row has its j-neighbour
    const bool kbn = DIR > 0 ? k > 0 : k < W.nz - 1;
    // row 0's neighbour row in the tile before, the near lane's neighbour column
    const int jn = DIR > 0 ? max(jb - 1, 0) : min(jb + rows, W.ny - 1);
    const int kn = DIR > 0 ? max(K * 32 - 1, 0) : min(K * 32 + 32, W.nz - 1);
    const int near = DIR > 0 ? 0 : 31;
    auto plane = [&](int tau, int skew) { return DIR > 0 ? tau - skew - w : W.nx - 1 - (tau - skew - w); };
    auto clampi = [&](int i) { return min(max(i, 0), W.nx - 1); };
    // the operands of step tau into slot tau % WD (one commit group per step);
    // the factors of a missing neighbour are read from the cell and not used
    auto stage = [&](int tau) {
        const int i = clampi(plane(tau, sk));
        const int sl = tau & (WD - 1);
        const int id = rb + i * W.si;
        const int ie = DIR > 0 ? 0 : (i < W.nx - 1 ? W.si : 0);
        const int je = DIR > 0 ? 0 : (jin ? W.sj : 0);
        const int ke = DIR > 0 ? 0 : (kbn ? 1 : 0);
        cp_async<sizeof(T)>(&sg.v[sl][0][w][lane], (DIR > 0 ? r : z) + id);
        cp_async<sizeof(T)>(&sg.v[sl][1][w][lane], Lw + id + ie);
        cp_async<sizeof(T)>(&sg.v[sl][2][w][lane], Ls + id + je);
        cp_async<sizeof(T)>(&sg.v[sl][3][w][lane], Lb + id + ke);
        cp_async<sizeof(T)>(&sg.v[sl][4][w][lane], Lc + id);
        cp_commit();
    };
    T prev = T(0), outp = T(0);
    sg.xs[0][w][lane] = sg.xs[1][w][lane] = T(0);
#pragma unroll
    for (int q = 0; q < WD - 1; ++q) stage(q);
    for (int tau0 = 0; tau0 < W.steps; tau0 += WB) {
        const int tend = min(tau0 + WB, W.steps);
        if (!wait_batch(W, d, base, tend, &sg.flag)) {
            cp_wait<0>();
            return false;
        }
        // the batch's cross-tile neighbours through L2 (clamped loads,
        // selected): row 0's j-neighbour for every step (own column), and the
        // k-neighbours of this warp's near lane (lane q holds step tau0 + q's)
        T zj[WB];
#pragma unroll
        for (int q = 0; q < WB; ++q) {
            const T v = __ldcg(z + W.off + clampi(plane(tau0 + q, sk)) * W.si + jn * W.sj + kc);
            zj[q] = d.dj >= 0 ? v : T(0);
        }
        T zk0;
        {
            const T v = __ldcg(z + W.off + clampi(plane(tau0 + (lane & (WB - 1)), 0)) * W.si + jr * W.sj + kn);
            zk0 = d.dk >= 0 ? v : T(0);
        }
#pragma unroll
        for (int q = 0; q < WB; ++q) {
            const int tau = tau0 + q;
            if (tau >= tend) break;   // block-uniform
            stage(tau + WD - 1);      // past the last step: clamped copies, never used
            cp_wait<WD - 1>();        // step tau's operands are in
            const int i = plane(tau, sk);
            const bool act = wact && kin && i >= 0 && i < W.nx;
            const int sl = tau & (WD - 1);
            const bool ib = DIR > 0 ? i > 0 : i < W.nx - 1;
            T zk = DIR > 0 ? __shfl_up_sync(FULL, outp, 1) : __shfl_down_sync(FULL, outp, 1);
            const T v0 = __shfl_sync(FULL, zk0, q);
            zk = lane == near ? v0 : zk;
            const T zjv = w == 0 ? zj[q] : sg.xs[(tau - 1) & 1][w - 1][lane];
            // :451-463 / :469-481, the terms in the reference's order
            T sum = sg.v[sl][0][w][lane];
            T a = sum - sg.v[sl][1][w][lane] * prev;
            sum = ib ? a : sum;
            a = sum - sg.v[sl][2][w][lane] * zjv;
            sum = jin ? a : sum;
            a = sum - sg.v[sl][3][w][lane] * zk;
            sum = kbn ? a : sum;
            const T out = sum / sg.v[sl][4][w][lane];
            if (act) z[rb + i * W.si] = out;
            prev = outp = out;
            sg.xs[tau & 1][w][lane] = out;
            __syncthreads();          // the next step reads this step's rows
        }
        if (t != W.stall) publish(W.prog + t, base + tend);   // block-uniform
    }
    cp_wait<0>();
    return true;
}

// apply_ic_preconditioner, src/pressure.cpp:442-482: the forward solve over
// all tiles, one grid barrier, the backward solve.  T = double is the
// reference's arithmetic; T = float serves the FP32 inner solve of the
// mixed-precision path (st == nullptr: never skipped).
template <typename T>
__global__ void __launch_bounds__(WT) k_ic_wave(Wave W, int base, const T* __restrict__ Lc, const T* __restrict__ Lw,
                                                const T* __restrict__ Ls, const T* __restrict__ Lb,
                                                const T* __restrict__ r, T* z, GridSync gs, const SolverState* st,
                                                int skip_done)
{
    if (skip_done && st && st->done) return;   // uniform across blocks: no barrier is entered
    __shared__ IcStage<T> sg;
    const int b = blockIdx.x, nb = gridDim.x;  // one tile per block at a time
    bool ok = true;
    for (int t = b; t < W.ntiles && ok; t += nb) ok = ic_tile<T, 1>(W, t, base, Lc, Lw, Ls, Lb, r, z, sg);
    if (!grid_barrier(gs) || !ok) return;
    for (int t = b; t < W.ntiles && ok; t += nb)
        ok = ic_tile<T, -1>(W, W.ntiles - 1 - t, base + W.steps + 1, Lc, Lw, Ls, Lb, r, z, sg);
}

// One lexicographic SOR sweep of one tile over the interior, :216-234:
// p = (1-omega) p + omega coef ((p_e + p_w)/dx2 + (p_n + p_s)/dy2 + (p_t + p_b)/dz2 - rhs)
// with the west, south and bottom neighbours already updated in this sweep
// and the east, north and top ones not yet.  POW2: dx2, dy2, dz2 are powers
// of two, so x / d2 is exactly x * (1 / d2) and the divisions become
// multiplications (same results bit for bit).  Accumulates the thread's max
// |dp| into maxr.  Staged WD steps ahead: the old values a step reads -- the
// cell, its east, north and top neighbours -- and rhs.  Those cells are
// written only at later steps: the cell by this thread at its step, the east
// one a step later, the north one by the next warp a step later (or by the
// tile above, which waits for this tile's progress, published only after the
// copies that read it completed), the top one by the next lane a step later.
struct GsStage {
    double v[WD][5][WAVE_TJ][32];   // p, p_east, p_north, p_top, rhs
    double xs[2][WAVE_TJ][32];      // each row's result of the last two steps
    int flag;
};

template <bool POW2>
__device__ bool gs_tile(const Wave& W, int t, int base, double d2x, double d2y, double d2z, double one_m_omega,
                        double omega_coef, const double* __restrict__ rhs, double* p, double& maxr, GsStage& sg)
{
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int J = t % W.wj, K = t / W.wj;
    const int jb = J * WAVE_TJ, rows = min(WAVE_TJ, W.ny - jb);
    const int k = K * 32 + lane;   // interior coordinates: grid cell (i+1, j+1, k+1)
    const bool kin = k < W.nz;
    const int kc = min(k, W.nz - 1);
    const TileDeps d = tile_deps<1>(W, J, K, t);
    const bool wact = w < rows;
    const int ssi = W.si, ssj = W.sj;
    const int rb = W.off + (jb + min(w, rows - 1)) * ssj + kc;   // (i = 0, this warp's row)
    const int rs = W.off + (jb - 1) * ssj + kc;                  // the row below the tile (the wall before the first)
    auto div2 = [&](double x, double dd) { return POW2 ? x * dd : x / dd; };
    auto clampi = [&](int i) { return min(max(i, 0), W.nx - 1); };
    auto stage = [&](int tau) {
        const int id = rb + clampi(tau - lane - w) * ssi;
        const int sl = tau & (WD - 1);
        cp_async<8>(&sg.v[sl][0][w][lane], p + id);
        cp_async<8>(&sg.v[sl][1][w][lane], p + id + ssi);
        cp_async<8>(&sg.v[sl][2][w][lane], p + id + ssj);   // the row above (the wall past the last row)
        cp_async<8>(&sg.v[sl][3][w][lane], p + id + 1);
        cp_async<8>(&sg.v[sl][4][w][lane], rhs + id);
        cp_commit();
    };
    double prev = 0.0, outp = 0.0;
    sg.xs[0][w][lane] = sg.xs[1][w][lane] = 0.0;
#pragma unroll
    for (int q = 0; q < WD - 1; ++q) stage(q);
    for (int tau0 = 0; tau0 < W.steps; tau0 += WB) {
        const int tend = min(tau0 + WB, W.steps);
        if (!wait_batch(W, d, base, tend, &sg.flag)) {
            cp_wait<0>();
            return false;
        }
        // the row below the tile (updated by the tile below, or the wall row
        // j = 0) for every step of warp 0, and the column before the near
        // lane's (the tile before in k, or the wall column k = 0): clamped loads
        double ps0[WB];
#pragma unroll
        for (int q = 0; q < WB; ++q) ps0[q] = __ldcg(p + rs + clampi(tau0 + q - lane) * ssi);
        const double pb0 = __ldcg(p + rb - kc + K * 32 - 1 + clampi(tau0 + (lane & (WB - 1)) - w) * ssi);
#pragma unroll
        for (int q = 0; q < WB; ++q) {
            const int tau = tau0 + q;
            if (tau >= tend) break;   // block-uniform
            stage(tau + WD - 1);
            cp_wait<WD - 1>();        // step tau's old values are in
            const int i = tau - lane - w;
            const bool act = wact && kin && i >= 0 && i < W.nx;
            const int sl = tau & (WD - 1);
            // plane i = 0: the west neighbour is the inlet face
            const double pw = i == 0 ? __ldcg(p + rb - ssi) : prev;
            double pb = __shfl_up_sync(FULL, outp, 1);
            const double v0 = __shfl_sync(FULL, pb0, q);
            pb = lane == 0 ? v0 : pb;
            const double ps = w == 0 ? ps0[q] : sg.xs[(tau - 1) & 1][w - 1][lane];
            const double po = sg.v[sl][0][w][lane];
            const double v = one_m_omega * po +
                             omega_coef * ((div2(sg.v[sl][1][w][lane] + pw, d2x) + div2(sg.v[sl][2][w][lane] + ps, d2y)) +
                                           div2(sg.v[sl][3][w][lane] + pb, d2z) - sg.v[sl][4][w][lane]);
            if (act) p[rb + i * ssi] = v;
            const double res = fabs(v - po);
            maxr = (act && res > maxr) ? res : maxr;
            prev = outp = v;
            sg.xs[tau & 1][w][lane] = v;
            __syncthreads();          // the next step reads this step's rows
        }
        if (t != W.stall) publish(W.prog + t, base + tend);   // block-uniform
    }
    cp_wait<0>();
    return true;
}

// solve_pressure_GS, src/pressure.cpp:212-246: up to max_iter SOR sweeps over
// the interior, each a pipelined wavefront followed by apply_pressure_BCs
// (face closed form, then the obstacle copy) and the max|dp| < tol test.
template <bool POW2>
__global__ void __launch_bounds__(WT) k_gs_wave(Wave W, int base, double d2x, double d2y, double d2z, double omega,
                                                double coef, double tol, int max_iter,
                                                const double* __restrict__ rhs, double* p,
                                                const uint8_t* __restrict__ solid, const int* __restrict__ solid_list,
                                                int n_solid, double* block_max, SolverState* st, GridSync gs,
                                                int nx, int ny, int nz)
{
    __shared__ GsStage sg;
    __shared__ double wmax[WAVE_TJ];
    const int b = blockIdx.x, nb = gridDim.x;   // one tile per block at a time
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gt = b * WT + threadIdx.x, gn = nb * WT;
    const double one_m_omega = 1 - omega;
    const double omega_coef = omega * coef;
    const int si = ny * nz, sj = nz;
    const int nfaces_i = ny * nz;
    int sweeps = 0;
    bool converged = false;
    for (int iter = 0; iter < max_iter; ++iter) {
        double maxr = 0.0;
        bool ok = true;
        const int bs = base + iter * (W.steps + 1);
        for (int t = b; t < W.ntiles && ok; t += nb)
            ok = gs_tile<POW2>(W, t, bs, d2x, d2y, d2z, one_m_omega, omega_coef, rhs, p, maxr, sg);
        if (!grid_barrier(gs) || !ok) return;
        // apply_pressure_BCs faces: every face cell from interior values
        {
            const int nface = 2 * nfaces_i + 2 * (nx - 2) * nz + 2 * (nx - 2) * (ny - 2);
            for (int q = gt; q < nface; q += gn) {
                int i, j, k;
                if (q < 2 * nfaces_i) {
                    const int e = q % nfaces_i;
                    i = (q < nfaces_i) ? 0 : nx - 1;
                    j = e / nz; k = e - j * nz;
                } else if (q < 2 * nfaces_i + 2 * (nx - 2) * nz) {
                    int e = q - 2 * nfaces_i;
                    const int half = (nx - 2) * nz;
                    j = (e < half) ? 0 : ny - 1;
                    e = e % half;
                    i = 1 + e / nz; k = e % nz;
                } else {
                    int e = q - 2 * nfaces_i - 2 * (nx - 2) * nz;
                    const int half = (nx - 2) * (ny - 2);
                    k = (e < half) ? 0 : nz - 1;
                    e = e % half;
                    i = 1 + e / (ny - 2); j = 1 + e % (ny - 2);
                }
                const int id = i * si + j * sj + k;
                if (i == nx - 1) { p[id] = 0.0; continue; }
                const int jc = j < 1 ? 1 : (j > ny - 2 ? ny - 2 : j);
                const int kc = k < 1 ? 1 : (k > nz - 2 ? nz - 2 : k);
                const int ic = i == 0 ? 1 : i;
                p[id] = __ldcg(p + ic * si + jc * sj + kc);
            }
        }
        if (!grid_barrier(gs)) return;
        for (int q = gt; q < n_solid; q += gn) {
            const int id = solid_list[q];
            if (!solid[id + si]) p[id] = __ldcg(p + id + si);
            else if (!solid[id - si]) p[id] = __ldcg(p + id - si);
            else if (!solid[id + sj]) p[id] = __ldcg(p + id + sj);
            else if (!solid[id - sj]) p[id] = __ldcg(p + id - sj);
            else if (!solid[id + 1]) p[id] = __ldcg(p + id + 1);
            else if (!solid[id - 1]) p[id] = __ldcg(p + id - 1);
        }
        // block max -> global max (exact), the same value in every thread (so
        // that the break below is uniform)
        maxr = warp_max_all(maxr);
        if (lane == 0) wmax[w] = maxr;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int q = 0; q < WAVE_TJ; ++q) m = fmax(m, wmax[q]);
            block_max[b] = m;
        }
        if (!grid_barrier(gs)) return;
        double gmax = 0.0;
        for (int q = lane; q < nb; q += 32) gmax = fmax(gmax, __ldcg(block_max + q));
        gmax = warp_max_all(gmax);
        sweeps = iter + 1;
        if (gmax < tol) { converged = true; break; }
        // block_max is rewritten next sweep only after the sweep's barrier
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->iters = sweeps;
        st->k = sweeps;
        st->done = 1;
        st->status = converged ? LES_OK : LES_NOT_CONVERGED;
    }
}

__global__ void k_stat_rhs_gs(Plane P, double coef, double two_dx, double two_dy, double two_dz,
                              const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, double* __restrict__ rhs, int n)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    int i = id / P.si, rem = id - i * P.si, j = rem / P.sj, k = rem - j * P.sj;
    if (i < 1 || i > P.nx - 2 || j < 1 || j > P.ny - 2 || k < 1 || k > P.nz - 2) { rhs[id] = 0.0; return; }
    double div = (u[id + P.si] - u[id - P.si]) / two_dx + (v[id + P.sj] - v[id - P.sj]) / two_dy +
                 (w[id + 1] - w[id - 1]) / two_dz;
    rhs[id] = coef * div;
}

Plane plane_of(const Geo& g) { return Plane{g.nx, g.ny, g.nz, g.si, g.sj}; }

les_status coop_launch(les_ctx* c, const void* fn, void** args, int* grid_out, int pid = -1)
{
    int per_sm = 0;
    les_status st = check_cuda(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0), "occupancy");
    if (st) return st;
    if (per_sm < 1) return fail(c, LES_CUDA_ERROR, "wavefront kernel cannot be resident");
    int grid = c->sms;   // one block per SM: enough threads for the widest hyperplane
    if (grid_out) *grid_out = grid;
    // count and generation only: the error word stays set until the host reads it
    st = check_cuda(c, cudaMemsetAsync(c->gsync, 0, sizeof(unsigned) * 2, c->stream), "reset barrier");
    if (st) return st;
    cudaEvent_t e1 = nullptr;
    if (pid >= 0 && c->prof_on) prof_begin(c, pid, &e1);
    st = check_cuda(c, cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, c->stream),
                    "cooperative launch");
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return st;
}

GridSync grid_sync(les_ctx* c, int grid)
{
    GridSync gs;
    gs.count = c->gsync + 0;
    gs.gen = c->gsync + 1;
    gs.error = (int*)(c->gsync + 2);
    gs.nblocks = (unsigned)grid;
    return gs;
}

les_status check_barrier(les_ctx* c)
{
    unsigned h[4];
    les_status st = check_cuda(c, cudaMemcpyAsync(h, c->gsync, sizeof(h), cudaMemcpyDeviceToHost, c->stream),
                               "read barrier");
    if (st) return st;
    st = check_cuda(c, cudaStreamSynchronize(c->stream), "sync");
    if (st) return st;
    if (h[2]) {
        st = check_cuda(c, cudaMemsetAsync(c->gsync + 2, 0, sizeof(unsigned), c->stream), "clear error");
        if (st) return st;
        return fail(c, LES_TIMEOUT, "a bounded wavefront wait timed out");
    }
    return LES_OK;
}

// The warp tiles of a pipelined sweep over the box [0,nx)x[0,ny)x[0,nz)
// starting at grid cell `off`, and the progress base of this launch: the
// launch uses progress values in (base, base + span]; the counters are only
// compared against later bases, so they need no reset between launches.
les_status wave_setup(les_ctx* c, int nx, int ny, int nz, int off, int span, Wave& W, int& base)
{
    W.nx = nx;
    W.ny = ny;
    W.nz = nz;
    W.si = c->g.si;
    W.sj = c->g.sj;
    W.off = off;
    W.wj = (ny + WAVE_TJ - 1) / WAVE_TJ;
    W.wk = (nz + 31) / 32;
    W.ntiles = W.wj * W.wk;
    W.steps = nx + 31 + WAVE_TJ - 1;
    if (c->wave_prog_len < W.ntiles) {
        cudaFree(c->wave_prog);
        c->wave_prog = nullptr;
        c->wave_prog_len = 0;
        les_status st = check_cuda(c, cudaMalloc(&c->wave_prog, sizeof(int) * (size_t)W.ntiles), "cudaMalloc(wave)");
        if (st) return st;
        c->wave_prog_len = W.ntiles;
        c->wave_epoch = 0;
        st = check_cuda(c, cudaMemsetAsync(c->wave_prog, 0, sizeof(int) * (size_t)W.ntiles, c->stream), "memset");
        if (st) return st;
    }
    if (span < 0 || span > (1 << 29)) return fail(c, LES_BAD_ARG, "wavefront: too many sweeps in one launch");
    if (c->wave_epoch > (1 << 30) - span) {   // restart the counters well before the int range ends
        les_status st = check_cuda(c, cudaMemsetAsync(c->wave_prog, 0, sizeof(int) * (size_t)c->wave_prog_len,
                                                      c->stream), "memset");
        if (st) return st;
        c->wave_epoch = 0;
    }
    base = c->wave_epoch;
    c->wave_epoch += span + 1;
    W.prog = c->wave_prog;
    W.err = (int*)(c->gsync + 2);
    W.stall = c->test_stall ? 0 : -1;
    return LES_OK;
}

// Cooperative launch of a pipelined sweep: one tile per block at a time, as many blocks
// as tiles but no more than can be resident at once (the tiles are handed out
// in producer-first order, so any resident count finishes).
les_status wave_launch(les_ctx* c, const void* fn, void** args, const Wave& W, GridSync* gs, int pid)
{
    int per_sm = 0;
    les_status st = check_cuda(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, WT, 0), "occupancy");
    if (st) return st;
    if (per_sm < 1) return fail(c, LES_CUDA_ERROR, "wavefront kernel cannot be resident");
    const long long cap = (long long)per_sm * c->sms;
    const int grid = (int)(W.ntiles < cap ? W.ntiles : cap);
    gs->nblocks = (unsigned)grid;
    // count and generation only: the error word stays set until the host reads it
    st = check_cuda(c, cudaMemsetAsync(c->gsync, 0, sizeof(unsigned) * 2, c->stream), "reset barrier");
    if (st) return st;
    cudaEvent_t e1 = nullptr;
    if (pid >= 0 && c->prof_on) prof_begin(c, pid, &e1);
    st = check_cuda(c, cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(WT), args, 0, c->stream),
                    "cooperative launch");
    ++c->launches;
    if (e1) cudaEventRecord(e1, c->stream);
    return st;
}

}  // namespace

namespace les {

// LES_TIMEOUT (and the flag cleared) if a wavefront wait gave up since the last check.
les_status wave_check(les_ctx* c) { return check_barrier(c); }

les_status ic_apply_dev(les_ctx* c, const double* r, double* z, const double* const* Lsrc, int skip_done)
{
    const double* const* L = Lsrc ? Lsrc : (const double* const*)c->L;
    Wave W;
    int base = 0;
    les_status st = wave_setup(c, c->g.nx, c->g.ny, c->g.nz, 0, 2 * (c->g.nx + 32 + WAVE_TJ), W, base);
    if (st) return st;
    const double *Lc = L[0], *Lw = L[4], *Ls = L[2], *Lb = L[6];
    GridSync gs = grid_sync(c, 0);
    const SolverState* stp = c->state;
    int skip = skip_done;
    void* args[] = {&W, &base, (void*)&Lc, (void*)&Lw, (void*)&Ls, (void*)&Lb, (void*)&r, (void*)&z, &gs,
                    (void*)&stp, &skip};
    return wave_launch(c, (const void*)k_ic_wave<double>, args, W, &gs, PROF_IC);
}

les_status ic_apply_dev32(les_ctx* c, const float* r, float* z, const float* const* L, SolverState* st)
{
    Wave W;
    int base = 0;
    les_status s2 = wave_setup(c, c->g.nx, c->g.ny, c->g.nz, 0, 2 * (c->g.nx + 32 + WAVE_TJ), W, base);
    if (s2) return s2;
    const float *Lc = L[0], *Lw = L[4], *Ls = L[2], *Lb = L[6];
    GridSync gs = grid_sync(c, 0);
    const SolverState* stp = st;
    int skip = st ? 1 : 0;
    void* args[] = {&W, &base, (void*)&Lc, (void*)&Lw, (void*)&Ls, (void*)&Lb, (void*)&r, (void*)&z, &gs,
                    (void*)&stp, &skip};
    return wave_launch(c, (const void*)k_ic_wave<float>, args, W, &gs, PROF_IC);
}

les_status build_ic_dev(les_ctx* c)
{
    const size_t nb = sizeof(double) * (size_t)c->g.n;
    for (int q = 0; q < 7; ++q) {
        if (!c->L[q]) {
            les_status st = check_cuda(c, cudaMalloc(&c->L[q], nb), "cudaMalloc(L)");
            if (st) return st;
        }
        cudaMemsetAsync(c->L[q], 0, nb, c->stream);
    }
    Plane P = plane_of(c->g);
    StencilView A = stencil_view(c);
    GridSync gs = grid_sync(c, c->sms);
    double *Lc = c->L[0], *Lw = c->L[4], *Ls = c->L[2], *Lb = c->L[6];
    void* args[] = {&P, &A, &Lc, &Lw, &Ls, &Lb, &gs};
    les_status st = coop_launch(c, (const void*)k_ic_build, args, nullptr);
    if (st) return st;
    st = check_barrier(c);
    if (st) return st;
    c->have_L = true;
    return LES_OK;
}

les_status solve_gs_dev(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps)
{
    les_status st = ensure_work(c);
    if (st) return st;
    const les_mesh& m = c->mesh;
    Plane P = plane_of(c->g);
    double* rhs = c->w[0];
    // one slot per warp of the cooperative grid
    double* block_max = c->partials;
    launch(c, k_stat_rhs_gs, (c->g.n + 255) / 256, 256, P, rho / dt, 2 * m.dx, 2 * m.dy, 2 * m.dz,
                                                               c->slot[LES_U], c->slot[LES_V], c->slot[LES_W],
                                                               rhs, c->g.n);
    st = check_launch(c, "gs rhs");
    if (st) return st;
    const double dx2 = m.dx * m.dx, dy2 = m.dy * m.dy, dz2 = m.dz * m.dz;
    const double coef = 1.0 / (2.0 * (1.0 / dx2 + 1.0 / dy2 + 1.0 / dz2));
    const Geo& g = c->g;
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return fail(c, LES_BAD_ARG, "GS-SOR needs an interior");
    Wave W;
    int base = 0;
    st = wave_setup(c, g.nx - 2, g.ny - 2, g.nz - 2, g.si + g.sj + 1, max_iter * (g.nx - 2 + 32 + WAVE_TJ), W, base);
    if (st) return st;
    // x / d2 for a power of two d2 is exactly x * (1 / d2)
    auto pow2 = [](double v) { int e; return std::frexp(v, &e) == 0.5; };
    const bool p2 = pow2(dx2) && pow2(dy2) && pow2(dz2);
    double d2x = p2 ? 1.0 / dx2 : dx2, d2y = p2 ? 1.0 / dy2 : dy2, d2z = p2 ? 1.0 / dz2 : dz2;
    double* p = c->slot[LES_P];
    const uint8_t* solid = c->mask;
    const int* list = c->solid_list;
    int ns = c->n_solid;
    SolverState* stp = c->state;
    GridSync gs = grid_sync(c, 0);
    int nx = g.nx, ny = g.ny, nz = g.nz;
    void* args[] = {&W, &base, &d2x, &d2y, &d2z, &omega, (void*)&coef, &tol, &max_iter, (void*)&rhs, &p,
                    (void*)&solid, (void*)&list, &ns, &block_max, &stp, &gs, &nx, &ny, &nz};
    if ((size_t)W.ntiles > c->partials_len) return fail(c, LES_BAD_ARG, "internal: partials too small");
    st = wave_launch(c, p2 ? (const void*)k_gs_wave<true> : (const void*)k_gs_wave<false>, args, W, &gs, -1);
    if (st) return st;
    st = check_barrier(c);
    if (st) return st;
    st = read_state(c);
    if (st) return st;
    if (sweeps) *sweeps = max_iter > 0 ? c->h_state->iters : 0;
    return LES_OK;
}

}  // namespace les

extern "C" {

les_status les_build_ic(les_ctx* c)
{
    if (!c) return LES_BAD_ARG;
    if (!c->stencil_mode) return fail(c, LES_BAD_ARG, "no matrix: call les_build_stencil or les_set_stencil");
    cudaSetDevice(c->device);
    return build_ic_dev(c);
}

les_status les_solve_gs(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps)
{
    if (!c || max_iter < 0) return LES_BAD_ARG;
    cudaSetDevice(c->device);
    return solve_gs_dev(c, dt, rho, max_iter, omega, tol, sweeps);
}

}  // extern "C"
