// sort.cu - stable counting sort of particles by (species, cell).
//
// The key (species * ncell + cellID, < 2^32) is sorted by least-significant-
// digit passes of a stable counting sort over digits of up to 9 bits (a
// 26-bit key takes three passes instead of four 8-bit ones), carrying the
// original particle index; the SoA payload is then gathered once through the
// resulting permutation. Each pass: a per-tile digit histogram, an exclusive
// scan of the digit-major (digit, tile) table, and a scatter in which every
// warp ranks its items in order with __match_any_sync, so equal keys keep
// their input order (stability) and the permutation is deterministic.
// This replaces Particle_Handler::SortParticles / std::sort with
// Particle_Compare (src/particles/particle_handler.cpp:180-183,
// src/particles/particle_utils.hpp:18-69).
#include <cuda_runtime.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>

#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;  // per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_BINS = 256;   // 8-bit digits
constexpr int RS_BINS9 = 512;  // 9-bit digits

template <int BINS>
__global__ void __launch_bounds__(RS_THREADS) k_hist(const uint32_t *keys, int64_t n, int shift, uint32_t mask,
                                                     uint32_t *hist, int nblocks) {
    __shared__ uint32_t cnt[BINS];
    for (int d = threadIdx.x; d < BINS; d += RS_THREADS) cnt[d] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int i = 0; i < RS_ITEMS; i++) {
        int64_t idx = base + (int64_t)i * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < BINS; d += RS_THREADS) hist[(int64_t)d * nblocks + blockIdx.x] = cnt[d];
}

// One stable counting-sort pass over a tile: rank every item within the tile
// (warps in order, items of a warp in order), reorder the tile by digit in
// shared memory, then write each digit's items as one contiguous stretch at
// the digit's global offset for this tile, so the stores are coalesced.
// BINS: 256 (8-bit digits) or 512 (9-bit). The per-warp digit counts (at most
// 32 * RS_ITEMS) and their within-tile offsets (below RS_TILE) fit 16 bits.
// Register budget for five resident blocks (48 registers, no spills): faster
// than the unconstrained 64 registers at full size (the loop's sort of a
// 536,870,912-particle store drifted 20 steps, 2.4 ms less).
template <int BINS>
__global__ void __launch_bounds__(RS_THREADS, 5) k_scatter(const uint32_t *kin, const uint32_t *vin, uint32_t *kout,
                                                        uint32_t *vout, int64_t n, int shift, uint32_t mask,
                                                        const uint32_t *hist, int nblocks) {
    static_assert(BINS % RS_THREADS == 0 && RS_TILE <= 65535, "digits per thread; 16-bit counts");
    constexpr int DPT = BINS / RS_THREADS;  // digits per thread
    __shared__ uint16_t wc[RS_THREADS / 32][BINS];
    __shared__ uint32_t s_key[RS_TILE];
    __shared__ uint32_t s_val[RS_TILE];
    __shared__ uint32_t s_start[BINS];  // tile-local start of each digit
    __shared__ uint32_t s_gbase[BINS];  // global start of each digit's stretch from this tile
    __shared__ uint32_t s_wsum[RS_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (RS_THREADS / 32) * BINS; i += RS_THREADS) (&wc[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * (32 * RS_ITEMS);
    // keys and values are read again when the tile is placed, and the ranks
    // are kept two to a register: few registers, more resident blocks
    uint32_t rank2[RS_ITEMS / 2];  // two 16-bit ranks (< 32 * RS_ITEMS) per word
    const unsigned lt = lanemask_lt();
    {
        uint32_t key[RS_ITEMS];
#pragma unroll
        for (int c = 0; c < RS_ITEMS; c++) {
            int64_t idx = base + c * 32 + lane;
            key[c] = idx < n ? __ldg(kin + idx) : 0u;
        }
#pragma unroll
        for (int c = 0; c < RS_ITEMS; c++) {
            int64_t idx = base + c * 32 + lane;
            bool valid = idx < n;
            uint32_t dg = (key[c] >> shift) & mask;
            unsigned tag = valid ? dg : (0x10000u + lane);
            unsigned peers = __match_any_sync(0xffffffffu, tag);
            uint32_t b = valid ? (uint32_t)wc[w][dg] : 0u;
            const uint32_t r = b + __popc(peers & lt);
            rank2[c >> 1] = (c & 1) ? (rank2[c >> 1] | (r << 16)) : r;
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) wc[w][dg] = (uint16_t)(b + __popc(peers));
            __syncwarp();
        }
    }
    __syncthreads();
    // per digit (DPT consecutive digits per thread): warp offsets within the
    // tile's digit stretch, the tile's digit totals, then an exclusive scan
    // over digits
    uint32_t totd[DPT];
    uint32_t tot = 0;
#pragma unroll
    for (int k = 0; k < DPT; k++) {
        const int d = threadIdx.x * DPT + k;
        uint32_t t = 0;
        for (int ww = 0; ww < RS_THREADS / 32; ww++) {
            const uint32_t x = wc[ww][d];
            wc[ww][d] = (uint16_t)t;
            t += x;
        }
        totd[k] = t;
        tot += t;
    }
    uint32_t incl = tot;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) s_wsum[w] = incl;
    __syncthreads();
    uint32_t run = incl - tot;
    for (int ww = 0; ww < w; ww++) run += s_wsum[ww];
#pragma unroll
    for (int k = 0; k < DPT; k++) {
        const int d = threadIdx.x * DPT + k;
        s_start[d] = run;
        run += totd[k];
        s_gbase[d] = hist[(int64_t)d * nblocks + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < RS_ITEMS; c++) {
        int64_t idx = base + c * 32 + lane;
        if (idx >= n) continue;
        const uint32_t k = __ldg(kin + idx);  // read again (L2)
        uint32_t dg = (k >> shift) & mask;
        uint32_t lp = s_start[dg] + wc[w][dg] + ((rank2[c >> 1] >> (16 * (c & 1))) & 0xffffu);
        s_key[lp] = k;
        s_val[lp] = vin ? __ldg(vin + idx) : (uint32_t)idx;
    }
    __syncthreads();
    const int64_t tbase = (int64_t)blockIdx.x * RS_TILE;
    const int cnt = n - tbase < RS_TILE ? (int)(n - tbase) : RS_TILE;
    for (int i = threadIdx.x; i < cnt; i += RS_THREADS) {
        const uint32_t k = s_key[i];
        const uint32_t dg = (k >> shift) & mask;
        const uint32_t pos = s_gbase[dg] + ((uint32_t)i - s_start[dg]);
        if (kout) kout[pos] = k;
        vout[pos] = s_val[i];
    }
}

// In-place exclusive scan of each RS_TILE-element tile; tile totals to sums.
__global__ void __launch_bounds__(RS_THREADS) k_scan_tile(uint32_t *data, int64_t m, uint32_t *sums) {
    __shared__ uint32_t wsum[RS_THREADS / 32];
    int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)threadIdx.x * RS_ITEMS;
    uint32_t v[RS_ITEMS];
    uint32_t tot = 0;
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        v[i] = (base + i < m) ? data[base + i] : 0u;
        tot += v[i];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = tot;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    uint32_t wpre = 0, all = 0;
    for (int ww = 0; ww < RS_THREADS / 32; ww++) {
        if (ww < w) wpre += wsum[ww];
        all += wsum[ww];
    }
    uint32_t run = wpre + incl - tot;
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        if (base + i < m) data[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0 && sums) sums[blockIdx.x] = all;
}

__global__ void k_scan_add(uint32_t *data, int64_t m, const uint32_t *sums) {
    int64_t base = (int64_t)blockIdx.x * RS_TILE;
    uint32_t a = sums[blockIdx.x];
    for (int i = threadIdx.x; i < RS_TILE; i += blockDim.x) {
        int64_t idx = base + i;
        if (idx < m) data[idx] += a;
    }
}

int64_t tiles(int64_t m) { return (m + RS_TILE - 1) / RS_TILE; }

// Scratch words a recursive scan of m elements needs.
int64_t scan_scratch(int64_t m) {
    int64_t t = tiles(m);
    if (t <= 1) return 1;
    return t + scan_scratch(t);
}

int scan_excl(emoo_handle *h, uint32_t *data, int64_t m, uint32_t *tmp) {
    int64_t t = tiles(m);
    if (t <= 1) {
        h->launches++;
        k_scan_tile<<<1, RS_THREADS, 0, h->stream>>>(data, m, nullptr);
        EMOO_CUDA(cudaGetLastError());
        return EMOO_OK;
    }
    h->launches++;
    k_scan_tile<<<(unsigned)t, RS_THREADS, 0, h->stream>>>(data, m, tmp);
    EMOO_TRY(scan_excl(h, tmp, t, tmp + t));
    h->launches++;
    k_scan_add<<<(unsigned)t, RS_THREADS, 0, h->stream>>>(data, m, tmp);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// dst[i] = src[perm[i]]. Each thread gathers 4 consecutive items at a time
// (one 16-byte permutation load, 4 independent loads in flight, vector
// stores); the < 4 items of the tail go one by one.
template <typename T>
__global__ void k_gather(const T *__restrict__ src, T *__restrict__ dst, const uint32_t *__restrict__ perm, int64_t n) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "payload element size");
    const int64_t n4 = n >> 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n4; j += stride) {
        const uint4 pp = __ldg(reinterpret_cast<const uint4 *>(perm) + j);
        const T a = src[pp.x], b = src[pp.y], c = src[pp.z], d = src[pp.w];
        T *o = dst + 4 * j;
        if constexpr (sizeof(T) == 4) {
            *reinterpret_cast<uint4 *>(o) = make_uint4(*reinterpret_cast<const uint32_t *>(&a),
                                                       *reinterpret_cast<const uint32_t *>(&b),
                                                       *reinterpret_cast<const uint32_t *>(&c),
                                                       *reinterpret_cast<const uint32_t *>(&d));
        } else {
            reinterpret_cast<ulonglong2 *>(o)[0] = make_ulonglong2(*reinterpret_cast<const unsigned long long *>(&a),
                                                                   *reinterpret_cast<const unsigned long long *>(&b));
            reinterpret_cast<ulonglong2 *>(o)[1] = make_ulonglong2(*reinterpret_cast<const unsigned long long *>(&c),
                                                                   *reinterpret_cast<const unsigned long long *>(&d));
        }
    }
    for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[perm[i]];
}

// Permutes one SoA array through the scratch buffer of its element size and
// swaps the two: every array only ever trades places with a buffer of the
// same capacity and element size (h->pay holds cap 8-byte elements, h->pay4
// cap 4-byte elements).
template <typename T>
int gather_one(emoo_handle *h, T *&arr, const uint32_t *perm, int64_t n) {
    static_assert(sizeof(T) == 8 || sizeof(T) == 4, "payload element size");
    if (!arr) return EMOO_OK;
    void *&scratch = sizeof(T) == 8 ? h->pay : h->pay4;
    if (!scratch || n > h->cap) return EMOO_ERR_STATE;
    T *tmp = (T *)scratch;
    // Four blocks per SM: the outputs in flight then read their sources from a
    // window of cells that stays in L2, so a fetched sector serves the other
    // elements in it. At sixteen per SM the window is wider and DRAM reads ran
    // at 1.47 times the bytes used (sort of a 536,870,912-particle store drifted
    // 20 steps: 26.9 ms at four blocks per SM, 32.9 ms at sixteen, 34.3 ms at one).
    int nb = (int)std::min<int64_t>((n / 4 + 255) / 256, 152 * 4);
    h->launches++;
    k_gather<T><<<std::max(nb, 1), 256, 0, h->stream>>>(arr, tmp, perm, n);  // base pointers are cudaMalloc'd
    EMOO_CUDA(cudaGetLastError());
    scratch = (void *)arr;
    arr = tmp;
    return EMOO_OK;
}

__global__ void k_species_bounds(const uint32_t *keys, int64_t n, int nspec, int64_t ncell, int64_t *bounds) {
    int s = threadIdx.x;
    if (s > nspec) return;
    uint64_t target = (uint64_t)s * (uint64_t)ncell;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if ((uint64_t)keys[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    bounds[s] = lo;
}

}  // namespace

// Digit widths: ceil(key_bits / 9) passes of equal width (at most 9 bits);
// a pass wider than 8 bits uses the 512-bin kernels.
int radix_sort_perm(emoo_handle *h, int64_t n, int key_bits) {
    if (key_bits > 32) return EMOO_ERR_UNSUPPORTED;  // keys are 32-bit words
    if (n <= 0) return EMOO_OK;
    const int kb = std::max(1, key_bits);
    const int passes = (kb + 8) / 9;
    const int width = (kb + passes - 1) / passes;
    const int bins = width > 8 ? RS_BINS9 : RS_BINS;
    int nblocks = (int)tiles(n);
    size_t need_hist = (size_t)bins * nblocks;
    if (h->hist_cap < need_hist) {
        if (h->hist) cudaFree(h->hist);
        h->hist = nullptr;
        EMOO_CUDA(cudaMalloc(&h->hist, need_hist * sizeof(uint32_t)));
        h->hist_cap = need_hist;
    }
    size_t need_scan = (size_t)scan_scratch((int64_t)need_hist) + 1;
    if (h->scan_cap < need_scan) {
        if (h->scan_tmp) cudaFree(h->scan_tmp);
        h->scan_tmp = nullptr;
        EMOO_CUDA(cudaMalloc(&h->scan_tmp, need_scan * sizeof(uint32_t)));
        h->scan_cap = need_scan;
    }
    int cur = 0, shift = 0;
    for (int ps = 0; ps < passes; ps++) {
        const int bits = std::min(width, kb - shift);
        const uint32_t mask = (1u << bits) - 1u;
        const int64_t nh = (int64_t)(bits > 8 ? RS_BINS9 : RS_BINS) * nblocks;
        const uint32_t *vin = ps == 0 ? nullptr : h->perm[cur];
        h->launches++;
        if (bits > 8)
            k_hist<RS_BINS9><<<nblocks, RS_THREADS, 0, h->stream>>>(h->key[cur], n, shift, mask, h->hist, nblocks);
        else
            k_hist<RS_BINS><<<nblocks, RS_THREADS, 0, h->stream>>>(h->key[cur], n, shift, mask, h->hist, nblocks);
        EMOO_CUDA(cudaGetLastError());
        EMOO_TRY(scan_excl(h, h->hist, nh, h->scan_tmp));
        h->launches++;
        if (bits > 8)
            k_scatter<RS_BINS9><<<nblocks, RS_THREADS, 0, h->stream>>>(h->key[cur], vin, h->key[cur ^ 1],
                                                                       h->perm[cur ^ 1], n, shift, mask, h->hist,
                                                                       nblocks);
        else
            k_scatter<RS_BINS><<<nblocks, RS_THREADS, 0, h->stream>>>(h->key[cur], vin, h->key[cur ^ 1],
                                                                      h->perm[cur ^ 1], n, shift, mask, h->hist,
                                                                      nblocks);
        EMOO_CUDA(cudaGetLastError());
        cur ^= 1;
        shift += bits;
    }
    // leave the result in slot 0
    if (cur == 1) {
        std::swap(h->key[0], h->key[1]);
        std::swap(h->perm[0], h->perm[1]);
    }
    return EMOO_OK;
}

// The mixed form's sorted cells straight from the sorted keys (species *
// npts + cell; removed particles carry keys from live_end on): a streaming
// pass in place of a gather through the permutation.
__global__ void k_cells_from_keys(const uint32_t *__restrict__ key, int64_t n, uint32_t npts, uint32_t live_end,
                                  int32_t *__restrict__ cell) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride) {
        const uint32_t k = key[j];
        cell[j] = k < live_end ? (int32_t)(k % npts) : -1;
    }
}

int gather_payload(emoo_handle *h, int64_t n, bool cells_from_keys) {
    const uint32_t *perm = h->perm[0];
    if (h->precision == EMOO_FP64) {
        EMOO_TRY(gather_one(h, h->x, perm, n));
        EMOO_TRY(gather_one(h, h->y, perm, n));
        EMOO_TRY(gather_one(h, h->z, perm, n));
        EMOO_TRY(gather_one(h, h->vx, perm, n));
        EMOO_TRY(gather_one(h, h->vy, perm, n));
        EMOO_TRY(gather_one(h, h->vz, perm, n));
        EMOO_TRY(gather_one(h, h->gam, perm, n));
    } else if (cells_from_keys) {
        // the sort keys of mixed_sort_keys: the cell is the key modulo npts
        int nb = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
        h->launches++;
        k_cells_from_keys<<<std::max(nb, 1), 256, 0, h->stream>>>(
            h->key[0], n, (uint32_t)h->g.npts, (uint32_t)((int64_t)h->nspec * h->g.npts), h->cell);
        EMOO_CUDA(cudaGetLastError());
    } else {
        EMOO_TRY(gather_one(h, h->cell, perm, n));
    }
    if (h->precision != EMOO_FP64) {
        EMOO_TRY(gather_one(h, h->ox, perm, n));
        EMOO_TRY(gather_one(h, h->oy, perm, n));
        EMOO_TRY(gather_one(h, h->oz, perm, n));
        EMOO_TRY(gather_one(h, h->ux, perm, n));
        EMOO_TRY(gather_one(h, h->uy, perm, n));
        EMOO_TRY(gather_one(h, h->uz, perm, n));
        if (h->first_push) EMOO_TRY(gather_one(h, h->g0, perm, n));
    }
    EMOO_TRY(gather_one(h, h->ids, perm, n));
    return EMOO_OK;
}

// Species segment bounds from the sorted keys; returns the per-species
// counts (removed particles are past the last bound).
int count_species(emoo_handle *h, int64_t n, int64_t stride, int64_t *counts_host) {
    if (!h->d_spec_count) EMOO_CUDA(cudaMalloc(&h->d_spec_count, sizeof(int64_t) * (EMOO_NSPEC + 1)));
    h->launches++;
    k_species_bounds<<<1, 64, 0, h->stream>>>(h->key[0], n, h->nspec, stride, h->d_spec_count);
    EMOO_CUDA(cudaGetLastError());
    int64_t b[EMOO_NSPEC + 1];
    EMOO_CUDA(cudaMemcpyAsync(b, h->d_spec_count, sizeof(int64_t) * (h->nspec + 1), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (int s = 0; s < h->nspec; s++) counts_host[s] = b[s + 1] - b[s];
    return EMOO_OK;
}

}  // namespace emoo

// ---------------------------------------------------------------------------
// Allocation-free stable sort permutation.
//
// Some callers of this library cannot call cudaMalloc: hosts that hand all
// device memory to their own pool allocator up front and reject any other
// allocation, and loops that must not pay the device-wide synchronisation a
// cudaMalloc / cudaFree can cause. emoo_sort_permutation_noalloc serves them:
// it runs the same counting-sort passes as the particle sort, with all of its
// scratch in one file-scope device array of fixed size, and allocates nothing.
//
// The array is created when the library is loaded on a device and lives until
// the process exits (12.25 MiB on every GPU that loads the library). Every call
// uses the same array and leaves its contents behind; nothing in it has to
// start at zero, because each pass writes every histogram slot and every
// buffer element it later reads. Calls whose GPU work overlaps (for example on
// two streams at once) race on the array: the caller must order them.
// ---------------------------------------------------------------------------
namespace emoo {
namespace {

constexpr int64_t NA_MAX = EMOO_NOALLOC_SORT_MAX;
constexpr int64_t NA_TILES = (NA_MAX + RS_TILE - 1) / RS_TILE;
constexpr int64_t NA_HIST = RS_BINS * NA_TILES;
constexpr int64_t NA_SCAN = 1024;  // > tiles(NA_HIST) + tiles(tiles(NA_HIST)) + 1

struct NoAllocScratch {
    uint32_t key[2][NA_MAX];
    uint32_t perm[NA_MAX];
    uint32_t hist[NA_HIST];
    uint32_t scan[NA_SCAN];
};

__device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current (the host-side symbol is not a device address).
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_ptr[256] = {};

int noalloc_scratch(NoAllocScratch **out) {
    int dev = 0;
    EMOO_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return EMOO_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e);
        g_noalloc_ptr[dev] = (NoAllocScratch *)p;
    }
    *out = g_noalloc_ptr[dev];
    return EMOO_OK;
}

int noalloc_scan(cudaStream_t s, uint32_t *data, int64_t m, uint32_t *tmp) {
    int64_t t = tiles(m);
    if (t <= 1) {
        k_scan_tile<<<1, RS_THREADS, 0, s>>>(data, m, nullptr);
        EMOO_CUDA(cudaGetLastError());
        return EMOO_OK;
    }
    k_scan_tile<<<(unsigned)t, RS_THREADS, 0, s>>>(data, m, tmp);
    EMOO_TRY(noalloc_scan(s, tmp, t, tmp + t));
    k_scan_add<<<(unsigned)t, RS_THREADS, 0, s>>>(data, m, tmp);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

}  // namespace

}  // namespace emoo

extern "C" int emoo_sort_permutation_noalloc(const uint32_t *keys, int64_t n, int key_bits, uint32_t *perm,
                                             void *stream) {
    using namespace emoo;
    if (n < 0 || n > NA_MAX) {
        fprintf(stderr, "emoo_sort_permutation_noalloc: n = %lld is outside [0, %lld]\n", (long long)n,
                (long long)NA_MAX);
        return EMOO_ERR_ARG;
    }
    if (key_bits < 1 || key_bits > 32) return EMOO_ERR_ARG;
    if (n == 0) return EMOO_OK;
    if (!keys || !perm) return EMOO_ERR_ARG;
    NoAllocScratch *sc = nullptr;
    EMOO_TRY(noalloc_scratch(&sc));
    cudaStream_t s = (cudaStream_t)stream;
    int nblocks = (int)tiles(n);
    int64_t nhist = (int64_t)RS_BINS * nblocks;
    int passes = (key_bits + 7) / 8;
    uint32_t *scr_perm = sc->perm;
    const uint32_t *kin = keys;
    const uint32_t *vin = nullptr;  // first pass: the identity
    for (int ps = 0; ps < passes; ps++) {
        int shift = ps * 8;
        int bits = key_bits - shift < 8 ? key_bits - shift : 8;
        uint32_t mask = (1u << bits) - 1u;
        bool last = ps == passes - 1;
        uint32_t *kout = last ? nullptr : sc->key[ps & 1];
        // alternate so that the last pass lands in the caller's array
        uint32_t *vout = ((passes - 1 - ps) % 2 == 0) ? perm : scr_perm;
        k_hist<RS_BINS><<<nblocks, RS_THREADS, 0, s>>>(kin, n, shift, mask, sc->hist, nblocks);
        EMOO_CUDA(cudaGetLastError());
        EMOO_TRY(noalloc_scan(s, sc->hist, nhist, sc->scan));
        k_scatter<RS_BINS><<<nblocks, RS_THREADS, 0, s>>>(kin, vin, kout, vout, n, shift, mask, sc->hist, nblocks);
        EMOO_CUDA(cudaGetLastError());
        kin = kout;
        vin = vout;
    }
    return EMOO_OK;
}
