// dev_common.cuh - device helpers shared by the CUDA translation units.
#ifndef EMOO_DEV_COMMON_CUH
#define EMOO_DEV_COMMON_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "emoo_internal.h"

namespace emoo {

// Division as the reference writes it; when the divisor is a power of two the
// exact reciprocal gives the identical result without the long FP64 divide.
__device__ __forceinline__ double ddiv(double a, double d, double id, int p2) { return p2 ? a * id : a / d; }

__device__ __forceinline__ int64_t gidx(const Geom &g, int i, int j, int k) {
    return (int64_t)i * g.sx + (int64_t)j * g.sy + k;
}

// The 1-based indices (i, j, k) of physical point t (0 <= t < n0 n1 n2, k
// fastest). 32-bit divisions where t fits (every grid these forms allocate):
// a 64-bit divide is a long emulated sequence.
__device__ __forceinline__ void phys_ijk(const int n[3], int64_t t, int &i, int &j, int &k) {
    if (t < ((int64_t)1 << 32)) {
        const uint32_t u = (uint32_t)t, n2 = (uint32_t)n[2], n1 = (uint32_t)n[1];
        const uint32_t r = u / n2;
        k = (int)(u - r * n2) + 1;
        const uint32_t q = r / n1;
        j = (int)(r - q * n1) + 1;
        i = (int)q + 1;
    } else {
        const int64_t r = t / n[2];
        k = (int)(t - r * n[2]) + 1;
        j = (int)(r % n[1]) + 1;
        i = (int)(r / n[1]) + 1;
    }
}

// Grid::getCellID, src/grid/oGrid.cpp:208-227: C truncation plus the ghost
// offset, per axis.
__device__ __forceinline__ void cell_of(const Geom &g, double x, double y, double z, int &ix, int &iy, int &iz) {
    ix = __double2int_rz((x - g.x0[0]) * g.id[0]) + 1;
    iy = __double2int_rz((y - g.x0[1]) * g.id[1]) + 1;
    iz = __double2int_rz((z - g.x0[2]) * g.id[2]) + 1;
}

__device__ __forceinline__ int cell_id(const Geom &g, int ix, int iy, int iz) { return g.cny * ix + g.cnz * iy + iz; }

// Cell indices must address points that exist: ix, ix+1 < n+3. The reference
// asserts 0 <= ix < n+3 (src/grid/oGrid.cpp:212); a position outside that
// range is recorded in the error word and the particle is skipped.
__device__ __forceinline__ bool cell_ok(const Geom &g, int ix, int iy, int iz) {
    return ix >= 0 && iy >= 0 && iz >= 0 && ix + 1 < g.tot[0] && iy + 1 < g.tot[1] && iz + 1 < g.tot[2];
}

__device__ __forceinline__ int species_of(const SpeciesTab &st, int64_t p) {
    int s = 0;
    while (s + 1 < st.nspec && p >= st.off[s + 1]) s++;
    return s;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Index of the last lane of the run of equal keys that lane `lane` belongs
// to, given the ballot of run heads (keys sorted or not: runs are maximal
// stretches of equal consecutive keys).
__device__ __forceinline__ int run_end(unsigned heads, int lane) {
    unsigned later = heads & ~((2u << lane) - 1u);  // heads strictly after lane (lane 31: none)
    if (lane == 31) later = 0u;
    return later ? (__ffs(later) - 2) : 31;
}

// Sum of v over lanes [lane, run_end] of the calling lane's run (suffix sum
// inside the run); the run head ends up with the run total.
template <typename T>
__device__ __forceinline__ T run_suffix_sum(T v, int lane, int rend) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        T o = __shfl_down_sync(0xffffffffu, v, off);
        if (lane + off <= rend) v += o;
    }
    return v;
}

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    // non-negative doubles order like their bit patterns
    atomicMax((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}

}  // namespace emoo

#endif
