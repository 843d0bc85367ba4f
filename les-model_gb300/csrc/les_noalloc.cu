// les_noalloc.cu -- a dot product of two device vectors that allocates no
// memory, for callers that cannot call cudaMalloc: code running inside a
// memory pool or arena that owns every device allocation of the process, a
// host that has reserved all device memory up front, or a thread that must
// not take the allocator's locks in the middle of a time step.
//
// The reduction's scratch (one FP64 partial per block and the last-block
// counter) lives in a file-scope __device__ array of fixed size.  CUDA loads
// this translation unit's module lazily (the default loading mode since
// CUDA 12.2), so the array is reserved on a device when the first call on
// that device looks up its address -- not when the library is loaded -- and
// is then held until the process exits.  Callers that reserve the rest of
// device memory up front make one call during set-up first; the same first
// call must come before any stream capture.  Its size caps the vector length
// at LES_NOALLOC_MAX_CELLS.  The kernel reads the array through the address
// that cudaGetSymbolAddress returns with the device current; host code never
// passes the array's own name to a kernel (on the host that name is only a
// stand-in, not a device address).  The address is cached per device
// together with the id of the CUDA context it belongs to, and looked up again
// when the current context differs (after cudaDeviceReset, or under another
// driver-API context).
//
// Every call shares the array, and the array keeps the last call's contents:
// the counter is cleared on the caller's stream before each launch, and calls
// that overlap on the GPU (different streams, no ordering between them) race
// on the scratch and give wrong results.
#include <cuda.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "les_internal.cuh"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_PER_THREAD = 8;
constexpr long long NA_CELLS_PER_BLOCK = (long long)NA_THREADS * NA_PER_THREAD;
constexpr int NA_MAX_BLOCKS = 65536;
// partials (one double per block) followed by the counter
constexpr size_t NA_SCRATCH_BYTES = sizeof(double) * NA_MAX_BLOCKS + 256;

static __device__ __align__(256) unsigned char g_na_scratch[NA_SCRATCH_BYTES];

std::mutex g_mu;
struct NaScratch {
    void* addr;                  // device address of g_na_scratch
    unsigned long long ctx_id;   // CUDA context it was looked up in (0: none yet)
};
NaScratch g_cache[128] = {};     // per device, filled on first use

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current CUDA context, 0 if there is none or the
// driver entry points are unavailable (then the address is looked up again).
unsigned long long current_ctx_id()
{
    static CtxGetCurrent get_cur = nullptr;
    static CtxGetId get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetId>(f);
        cudaGetLastError();
    }
    if (!get_cur || !get_id) return 0;
    CUcontext cx = nullptr;
    unsigned long long id = 0;
    if (get_cur(&cx) != CUDA_SUCCESS || !cx || get_id(cx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

__global__ void __launch_bounds__(NA_THREADS) k_dot_na(const double* __restrict__ a, const double* __restrict__ b,
                                                       long long n, double* out, unsigned char* scratch)
{
    __shared__ double sm[32];
    double* partials = reinterpret_cast<double*>(scratch);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + sizeof(double) * NA_MAX_BLOCKS);
    const long long base = (long long)blockIdx.x * NA_CELLS_PER_BLOCK + threadIdx.x;
    double s[1] = {0.0};
#pragma unroll
    for (int q = 0; q < NA_PER_THREAD; ++q) {
        const long long i = base + (long long)q * NA_THREADS;
        if (i < n) s[0] += a[i] * b[i];
    }
    if (les::last_block_sum<1>(s, partials, counter, sm)) {
        if (threadIdx.x == 0) *out = s[0];
    }
}

// The entry point has no context to hold a message: errors go to stderr
// beside the status code.
les_status na_fail(les_status st, const std::string& msg)
{
    std::fprintf(stderr, "%s\n", msg.c_str());
    return st;
}

static_assert((long long)NA_MAX_BLOCKS * NA_CELLS_PER_BLOCK == LES_NOALLOC_MAX_CELLS,
              "scratch size and the documented limit disagree");

}  // namespace

extern "C" les_status les_dot_noalloc(const double* a, const double* b, long long n, double* out, void* stream)
{
    if (!a || !b || !out) return na_fail(LES_BAD_ARG, "les_dot_noalloc: null pointer");
    if (n <= 0) return na_fail(LES_BAD_ARG, "les_dot_noalloc: n must be positive");
    if (n > LES_NOALLOC_MAX_CELLS) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "les_dot_noalloc: n = %lld exceeds the fixed scratch limit of %lld cells",
                      n, (long long)LES_NOALLOC_MAX_CELLS);
        return na_fail(LES_BAD_ARG, buf);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(LES_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 128) return na_fail(LES_BAD_ARG, "les_dot_noalloc: device index out of range");
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        NaScratch& slot = g_cache[dev];
        const unsigned long long id = current_ctx_id();
        if (!slot.addr || id == 0 || slot.ctx_id != id) {
            // set-up, once per device (and context), with that device current:
            // the lookup loads this module on the device, which reserves the array
            void* addr = nullptr;
            e = cudaGetSymbolAddress(&addr, g_na_scratch);
            if (e != cudaSuccess) {
                slot.addr = nullptr;
                slot.ctx_id = 0;
                return na_fail(LES_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            }
            slot.addr = addr;
            slot.ctx_id = current_ctx_id();   // the lookup made the primary context current
        }
        scratch = slot.addr;
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* counter = static_cast<unsigned char*>(scratch) + sizeof(double) * NA_MAX_BLOCKS;
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return na_fail(LES_CUDA_ERROR, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const unsigned blocks = (unsigned)((n + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK);
    k_dot_na<<<blocks, NA_THREADS, 0, s>>>(a, b, n, out, static_cast<unsigned char*>(scratch));
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(LES_CUDA_ERROR, std::string("k_dot_na launch: ") + cudaGetErrorString(e));
    return LES_OK;
}
