// les_mixed.cuh -- FP32 view of the pressure matrix for the mixed-precision
// inner solve (les_mixed.cu, les_fused.cu).
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
    __device__ __forceinline__ CoefF at(int id) const
    {
        CoefF a;
        if (code) {
            unsigned cd = code[id];
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

bool fused_supported(const les_pcg_opts* o);
les_status inner_solve_fused(les_ctx* c, const les_pcg_opts* o, ViewF A, SolverState* in, SolverState* out,
                             int inner_cap);

}  // namespace les
