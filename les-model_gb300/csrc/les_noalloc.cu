// les_noalloc.cu -- a dot product of two device vectors that allocates no
// memory, for callers that cannot call cudaMalloc: code running inside a
// memory pool or arena that owns every device allocation of the process, a
// host that has reserved all device memory up front, or a thread that must
// not take the allocator's locks in the middle of a time step.
//
// The reduction's scratch (one FP64 partial per block and the last-block
// counter) lives in a file-scope __device__ array of fixed size, reserved when
// the library is loaded on a device and held by every device that loads the
// library until the process exits.  Its size caps the vector length at
// LES_NOALLOC_MAX_CELLS.  The kernel reads the array through the address that
// cudaGetSymbolAddress returns for the current device; host code never passes
// the array's own name to a kernel (on the host that name is only a stand-in,
// not a device address).
//
// Every call shares the array, and the array keeps the last call's contents:
// the counter is cleared on the caller's stream before each launch, and calls
// that overlap on the GPU (different streams, no ordering between them) race
// on the scratch and give wrong results.
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
void* g_addr[128] = {};   // scratch address per device, filled on first use

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
        if (!g_addr[dev]) {
            // set-up, once per device, with that device current
            e = cudaGetSymbolAddress(&g_addr[dev], g_na_scratch);
            if (e != cudaSuccess) {
                g_addr[dev] = nullptr;
                return na_fail(LES_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            }
        }
        scratch = g_addr[dev];
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
