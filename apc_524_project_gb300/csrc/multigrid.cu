// multigrid.cu - geometric multigrid for the field start (no reference
// counterpart). It solves the discrete equations whose fixed point
// Poisson_Solver::run_poisson_solver_ (src/poisson/poisson.cpp:216-241)
// iterates towards: at every unknown point of the grid the 7-point Laplacian
// of u equals f = mult R. A dimension with periodic field boundaries has the
// unknowns 1..n and wraps; one with external boundaries holds the PoissonBC
// values on planes 1 and n + 1 (src/poisson/poissonBC.cpp:67-80) and has the
// unknowns 2..n.
//
// Precision: FP64 throughput on this GPU is a small fraction of FP32's, so
// the solution u and the residual r = f - Lu are FP64, and each outer step
// solves the correction equation L e = r approximately by one FP32 V-cycle,
// then u += e (iterative refinement: the FP64 residual sets the accuracy, the
// V-cycle only the rate).
//
// Levels are vertex-centred: coarse index C sits on fine index 2C - 1 along a
// coarsened dimension, so periodic grids of even P halve and external grids
// keep their boundary planes on boundary planes (the correction is zero
// there). A dimension coarsens while its P is even and at least 4; the others
// keep their spacing (semi-coarsening). One V-cycle: two red-black
// Gauss-Seidel sweeps, residual, full-weighting restriction, the coarser
// cycle, trilinear prolongation, two sweeps; the coarsest level is swept
// until its few unknowns settle. The levels of at most 4096 unknowns run
// their whole part of the cycle inside one thread block, in its shared memory
// (one launch, block barriers between the stages): launched one kernel per
// stage, they would cost a launch latency each for a few microseconds of
// work, and from global memory each stage would wait on L2. Each level is a dense
// (P+2)^3 block; periodic neighbours are found by index wrap, so no ghost
// planes are kept. Red and black do not colour a periodic dimension of odd P
// (points 1 and P are neighbours of one colour), so a level with one smooths
// by damped Jacobi half-steps between u and a second buffer instead: no two
// threads touch one point, and the result does not depend on their order.
// One outer step (V-cycle, correction, new FP64 residual and its maximum) is
// a CUDA graph, replayed until max |r| <= rtol max |r0|.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {
namespace {

struct Lv {
    int P[3];         // points per dimension (see above)
    int per[3];       // 1: periodic
    int lo[3], hi[3]; // unknown index range
    int crs[3];       // 1: the next level halves this dimension
    int64_t sx, sy;   // strides of the (P+2)^3 block
    float c[3];       // 1 / h^2
    float diag;       // 2 (c0 + c1 + c2)
    float idiag;      // 1 / diag
    int rb;           // 1: red-black Gauss-Seidel; 0: damped Jacobi via t
    float *u, *f, *r;
    float *t;         // Jacobi partner of u, or null
};

// the FP64 solution and right side, on level 0's layout
struct Fine {
    double c[3];
    double diag;
    double *u, *f;
};

struct MgState {
    int n[3];
    int per[3];
    double d[3];
    std::vector<Lv> lv;
    size_t tail_from = 0;  // first level of the shared-memory tail (lv.size(): none)
    Fine fine = {};
    double *part = nullptr;   // per-block sums
    double *hpart = nullptr;  // pinned host copy
    double *dmax = nullptr;   // device max |r|
    double *hmax = nullptr;   // pinned host copy
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_launches = 0;   // kernels per replay
};

constexpr int RB = 256;      // reduction blocks
constexpr int NU = 2;        // smoothing sweeps before and after the coarse correction
constexpr float OMEGA = 6.0f / 7.0f;  // Jacobi damping, the 7-point stencil's smoothing optimum
constexpr int TAIL_MAX = 4096;    // levels of at most this many unknowns run in the one-block tail
constexpr int TAIL_LEVELS = 16;
constexpr int TAIL_THREADS = 1024;

__device__ __forceinline__ int64_t lidx(const Lv &L, int i, int j, int k) {
    return (int64_t)i * L.sx + (int64_t)j * L.sy + k;
}
__device__ __forceinline__ int wrap_dn(const Lv &L, int d, int i) { return (L.per[d] && i == 1) ? L.P[d] : i - 1; }
__device__ __forceinline__ int wrap_up(const Lv &L, int d, int i) { return (L.per[d] && i == L.P[d]) ? 1 : i + 1; }

// sum over the six neighbours, each weighted by 1/h^2 of its dimension
template <class R, class C>
__device__ __forceinline__ R nb_sum(const Lv &L, const C *c, const R *u, int i, int j, int k) {
    return c[0] * (u[lidx(L, wrap_dn(L, 0, i), j, k)] + u[lidx(L, wrap_up(L, 0, i), j, k)]) +
           c[1] * (u[lidx(L, i, wrap_dn(L, 1, j), k)] + u[lidx(L, i, wrap_up(L, 1, j), k)]) +
           c[2] * (u[lidx(L, i, j, wrap_dn(L, 2, k))] + u[lidx(L, i, j, wrap_up(L, 2, k))]);
}

__device__ __forceinline__ void gs_point(const Lv &L, int i, int j, int k) {
    const int64_t o = lidx(L, i, j, k);
    L.u[o] = (nb_sum(L, L.c, L.u, i, j, k) - L.f[o]) * L.idiag;
}

__device__ __forceinline__ void jacobi_point(const Lv &L, const float *src, float *dst, int i, int j, int k) {
    const int64_t o = lidx(L, i, j, k);
    const float x = src[o];
    dst[o] = x + OMEGA * ((nb_sum(L, L.c, src, i, j, k) - L.f[o]) * L.idiag - x);
}

// One colour of a red-black Gauss-Seidel sweep: the points with
// (i + j + k) & 1 == colour take u = (neighbour sum - f) / diag.
__global__ void k_mg_smooth(Lv L, int colour) {
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (j > L.hi[1] || i > L.hi[0]) return;
    const int k = L.lo[2] + ((colour + i + j + L.lo[2]) & 1) + 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (k > L.hi[2]) return;
    gs_point(L, i, j, k);
}

// One damped Jacobi half-step at the unknowns, src -> dst.
__global__ void k_mg_jacobi(Lv L, const float *src, float *dst) {
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (k > L.hi[2] || j > L.hi[1] || i > L.hi[0]) return;
    jacobi_point(L, src, dst, i, j, k);
}

// r = f - Laplacian(u) at the unknowns (FP32 levels)
__device__ __forceinline__ void residual_point(const Lv &L, int i, int j, int k) {
    const int64_t o = lidx(L, i, j, k);
    L.r[o] = L.f[o] - (nb_sum(L, L.c, L.u, i, j, k) - L.diag * L.u[o]);
}

__global__ void k_mg_residual(Lv L) {
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (k > L.hi[2] || j > L.hi[1] || i > L.hi[0]) return;
    residual_point(L, i, j, k);
}

// The FP64 residual of the fine problem: level 0's right side takes it (as
// FP32), level 0's correction restarts at zero, and *dmax the maximum |r|,
// taken over the FP32 values (the stop test needs no more): this kernel runs
// on the FP64 pipe, so everything after the residual itself stays off it.
__global__ void k_mg_residual64(Lv L, Fine F, double *dmax) {
    __shared__ float sh[8];
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    float a = 0.0f;
    if (k <= L.hi[2] && j <= L.hi[1] && i <= L.hi[0]) {
        const int64_t o = lidx(L, i, j, k);
        const float r = (float)(F.f[o] - (nb_sum(L, F.c, F.u, i, j, k) - F.diag * F.u[o]));
        L.f[o] = r;
        L.u[o] = 0.0f;
        a = fabsf(r);
    }
    for (int off = 16; off > 0; off >>= 1) a = fmaxf(a, __shfl_down_sync(0xffffffffu, a, off));
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if ((tid & 31) == 0) sh[tid >> 5] = a;
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < (int)((blockDim.x * blockDim.y) >> 5); w++) a = fmaxf(a, sh[w]);
        atomic_max_nonneg(dmax, (double)a);
    }
}

// u += e at the unknowns (e: level 0's correction)
__global__ void k_mg_correct(Lv L, Fine F) {
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (k > L.hi[2] || j > L.hi[1] || i > L.hi[0]) return;
    const int64_t o = lidx(L, i, j, k);
    F.u[o] += (double)L.u[o];
}

// fine index and weight of tap t (0..2) of coarse index C along dimension d
__device__ __forceinline__ int tap(const Lv &F, int d, int C, int t, float &w) {
    if (!F.crs[d]) {
        w = t == 1 ? 1.0f : 0.0f;
        return C;
    }
    w = t == 1 ? 0.5f : 0.25f;
    int f = 2 * C - 1 + (t - 1);
    if (F.per[d]) f = f < 1 ? f + F.P[d] : (f > F.P[d] ? f - F.P[d] : f);
    return f;
}

// coarse f = full-weighting restriction of the fine residual; coarse u = 0
__device__ __forceinline__ void restrict_point(const Lv &F, const Lv &Cl, int I, int J, int K) {
    float s = 0.0f;
    for (int a = 0; a < 3; a++) {
        float wa;
        const int fi = tap(F, 0, I, a, wa);
        if (wa == 0.0f) continue;
        for (int b = 0; b < 3; b++) {
            float wb;
            const int fj = tap(F, 1, J, b, wb);
            if (wb == 0.0f) continue;
            float row = 0.0f;
            for (int e = 0; e < 3; e++) {
                float we;
                const int fk = tap(F, 2, K, e, we);
                if (we == 0.0f) continue;
                row += we * F.r[lidx(F, fi, fj, fk)];
            }
            s += wa * wb * row;
        }
    }
    const int64_t o = lidx(Cl, I, J, K);
    Cl.f[o] = s;
    Cl.u[o] = 0.0f;
}

__global__ void k_mg_restrict(Lv F, Lv Cl) {
    const int K = Cl.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int J = Cl.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int I = Cl.lo[0] + blockIdx.z;
    if (K > Cl.hi[2] || J > Cl.hi[1] || I > Cl.hi[0]) return;
    restrict_point(F, Cl, I, J, K);
}

// coarse index pair and weight of the second feeding fine index f along d
__device__ __forceinline__ void interp(const Lv &F, const Lv &Cl, int d, int f, int &c0, int &c1, float &w1) {
    if (!F.crs[d]) {
        c0 = c1 = f;
        w1 = 0.0f;
        return;
    }
    if (f & 1) {
        c0 = c1 = (f + 1) >> 1;
        w1 = 0.0f;
        return;
    }
    c0 = f >> 1;
    c1 = c0 + 1;
    if (Cl.per[d] && c1 > Cl.P[d]) c1 = 1;
    w1 = 0.5f;
}

// fine u += trilinear interpolation of the coarse correction
__device__ __forceinline__ void prolong_point(const Lv &Cl, const Lv &F, int i, int j, int k) {
    int ci[2], cj[2], ck[2];
    float wi, wj, wk;
    interp(F, Cl, 0, i, ci[0], ci[1], wi);
    interp(F, Cl, 1, j, cj[0], cj[1], wj);
    interp(F, Cl, 2, k, ck[0], ck[1], wk);
    // all eight taps, zero-weighted ones on a repeated (cached) address: the
    // weights change with the parity of k, so skipping taps would split warps
    const float Wi[2] = {1.0f - wi, wi}, Wj[2] = {1.0f - wj, wj}, Wk[2] = {1.0f - wk, wk};
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            const int64_t row = (int64_t)ci[a] * Cl.sx + (int64_t)cj[b] * Cl.sy;
            s += Wi[a] * Wj[b] * (Wk[0] * Cl.u[row + ck[0]] + Wk[1] * Cl.u[row + ck[1]]);
        }
    F.u[lidx(F, i, j, k)] += s;
}

__global__ void k_mg_prolong(Lv Cl, Lv F) {
    const int k = F.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = F.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = F.lo[0] + blockIdx.z;
    if (k > F.hi[2] || j > F.hi[1] || i > F.hi[0]) return;
    prolong_point(Cl, F, i, j, k);
}

// ---- the one-block tail: levels lv[0..nl-1] of at most TAIL_MAX unknowns,
// lv[0]'s right side already restricted and its u zero

struct Tail {
    int nl;
    int sweeps;  // on the coarsest
    int smem;    // floats of shared memory the levels take
    Lv lv[TAIL_LEVELS];  // the global levels (lv[0]'s f in, u out)
    int ou[TAIL_LEVELS], of[TAIL_LEVELS], orr[TAIL_LEVELS], ot[TAIL_LEVELS];  // their shared copies; ot < 0: none
};

// level l of the tail with its arrays in shared memory
__device__ __forceinline__ Lv tail_level(const Tail &T, int l, float *sm) {
    Lv L = T.lv[l];
    L.u = sm + T.ou[l];
    L.f = sm + T.of[l];
    L.r = sm + T.orr[l];
    L.t = T.ot[l] >= 0 ? sm + T.ot[l] : nullptr;
    return L;
}

__device__ __forceinline__ void pt_of(const Lv &L, int t, int &i, int &j, int &k) {
    const int m1 = L.hi[1] - L.lo[1] + 1, m2 = L.hi[2] - L.lo[2] + 1;
    k = L.lo[2] + t % m2;
    j = L.lo[1] + (t / m2) % m1;
    i = L.lo[0] + t / (m1 * m2);
}

__device__ __forceinline__ int npts_of(const Lv &L) {
    return (L.hi[0] - L.lo[0] + 1) * (L.hi[1] - L.lo[1] + 1) * (L.hi[2] - L.lo[2] + 1);
}

// Every loop below has a trip count fixed by the level; every thread of the
// block reaches every barrier.
__device__ void blk_smooth(const Lv &L, int sweeps) {
    const int n = npts_of(L);
    int i, j, k;
    for (int s = 0; s < sweeps; s++)
        for (int half = 0; half < 2; half++) {
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                pt_of(L, t, i, j, k);
                if (L.rb) {
                    if (((i + j + k) & 1) == half) gs_point(L, i, j, k);
                } else if (half == 0) {
                    jacobi_point(L, L.u, L.t, i, j, k);
                } else {
                    jacobi_point(L, L.t, L.u, i, j, k);
                }
            }
            __syncthreads();
        }
}

__global__ void __launch_bounds__(TAIL_THREADS) k_mg_tail(Tail T) {
    extern __shared__ float sm[];
    int i, j, k;
    for (int t = threadIdx.x; t < T.smem; t += blockDim.x) sm[t] = 0.0f;
    __syncthreads();
    {
        const Lv G = T.lv[0], L = tail_level(T, 0, sm);
        for (int t = threadIdx.x; t < npts_of(L); t += blockDim.x) {
            pt_of(L, t, i, j, k);
            L.f[lidx(L, i, j, k)] = G.f[lidx(G, i, j, k)];
        }
    }
    __syncthreads();
    for (int l = 0; l + 1 < T.nl; l++) {
        const Lv L = tail_level(T, l, sm), C = tail_level(T, l + 1, sm);
        blk_smooth(L, NU);
        for (int t = threadIdx.x; t < npts_of(L); t += blockDim.x) {
            pt_of(L, t, i, j, k);
            residual_point(L, i, j, k);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < npts_of(C); t += blockDim.x) {
            pt_of(C, t, i, j, k);
            restrict_point(L, C, i, j, k);
        }
        __syncthreads();
    }
    blk_smooth(tail_level(T, T.nl - 1, sm), T.sweeps);
    for (int l = T.nl - 2; l >= 0; l--) {
        const Lv L = tail_level(T, l, sm), C = tail_level(T, l + 1, sm);
        for (int t = threadIdx.x; t < npts_of(L); t += blockDim.x) {
            pt_of(L, t, i, j, k);
            prolong_point(C, L, i, j, k);
        }
        __syncthreads();
        blk_smooth(L, NU);
    }
    const Lv G = T.lv[0], L = tail_level(T, 0, sm);
    for (int t = threadIdx.x; t < npts_of(L); t += blockDim.x) {
        pt_of(L, t, i, j, k);
        G.u[lidx(G, i, j, k)] = L.u[lidx(L, i, j, k)];
    }
}

// the FP64 problem from the grid slots: u takes the slot's values on the
// unknowns and on external boundary planes (the PoissonBC values), f = mult R
__global__ void k_mg_load(Geom g, Lv L, Fine F, const double *slot, const double *R, double mult) {
    const int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = 1 + blockIdx.z;
    const int ek = L.per[2] ? L.P[2] : L.P[2] + 1, ej = L.per[1] ? L.P[1] : L.P[1] + 1;
    if (k > ek || j > ej) return;
    const int64_t o = lidx(L, i, j, k), s = gidx(g, i, j, k);
    F.u[o] = slot[s];
    F.f[o] = mult * R[s];
}

// the unknowns of the solution (less `shift`) into the zeroed slot
__global__ void k_mg_store(Geom g, Lv L, const double *u, double *slot, double shift) {
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (k > L.hi[2] || j > L.hi[1] || i > L.hi[0]) return;
    slot[gidx(g, i, j, k)] = u[lidx(L, i, j, k)] - shift;
}

// per-block sums of a over the unknowns (fixed order within a block)
__global__ void k_mg_sum(Lv L, const double *a, double *part) {
    __shared__ double sh[32];
    const int64_t m0 = L.hi[0] - L.lo[0] + 1, m1 = L.hi[1] - L.lo[1] + 1, m2 = L.hi[2] - L.lo[2] + 1;
    const int64_t n = m0 * m1 * m2;
    double v = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = L.lo[2] + (int)(t % m2);
        const int64_t q = t / m2;
        const int j = L.lo[1] + (int)(q % m1);
        const int i = L.lo[0] + (int)(q / m1);
        v += a[lidx(L, i, j, k)];
    }
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sh[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) s += sh[q];
        part[blockIdx.x] = s;
    }
}

__global__ void k_mg_shift(Lv L, double *a, double m) {
    const int k = L.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = L.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    const int i = L.lo[0] + blockIdx.z;
    if (k > L.hi[2] || j > L.hi[1] || i > L.hi[0]) return;
    a[lidx(L, i, j, k)] -= m;
}

dim3 pts_grid(const Lv &L, dim3 blk) {
    return dim3((L.hi[2] - L.lo[2] + 1 + blk.x - 1) / blk.x, (L.hi[1] - L.lo[1] + 1 + blk.y - 1) / blk.y,
                L.hi[0] - L.lo[0] + 1);
}

int64_t unknowns(const Lv &L) {
    return (int64_t)(L.hi[0] - L.lo[0] + 1) * (L.hi[1] - L.lo[1] + 1) * (L.hi[2] - L.lo[2] + 1);
}

void mg_release(MgState *s) {
    for (Lv &L : s->lv) {
        cudaFree(L.u);
        cudaFree(L.f);
        cudaFree(L.r);
        if (L.t) cudaFree(L.t);
    }
    s->lv.clear();
    cudaFree(s->fine.u);
    cudaFree(s->fine.f);
    s->fine = Fine{};
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
    cudaFree(s->part);
    cudaFree(s->dmax);
    cudaFreeHost(s->hpart);
    cudaFreeHost(s->hmax);
    s->part = s->dmax = s->hpart = s->hmax = nullptr;
}

int alloc_zero(void **p, size_t bytes, cudaStream_t st) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, st);
    return e == cudaSuccess ? EMOO_OK : cuda_status(e);
}

void smooth(emoo_handle *h, const Lv &L, int sweeps, int &launches) {
    dim3 blk(32, 8);
    if (!L.rb) {
        for (int s = 0; s < sweeps; s++) {
            launches += 2;
            k_mg_jacobi<<<pts_grid(L, blk), blk, 0, h->stream>>>(L, L.u, L.t);
            k_mg_jacobi<<<pts_grid(L, blk), blk, 0, h->stream>>>(L, L.t, L.u);
        }
        return;
    }
    const int m2 = L.hi[2] - L.lo[2] + 1;
    dim3 grd(((m2 + 1) / 2 + blk.x - 1) / blk.x, (L.hi[1] - L.lo[1] + 1 + blk.y - 1) / blk.y, L.hi[0] - L.lo[0] + 1);
    for (int s = 0; s < sweeps; s++)
        for (int c = 0; c < 2; c++) {
            launches++;
            k_mg_smooth<<<grd, blk, 0, h->stream>>>(L, c);
        }
}

int coarse_sweeps(const Lv &L) {
    int m = 1;
    for (int d = 0; d < 3; d++) m = std::max(m, L.hi[d] - L.lo[d] + 1);
    return std::min(500, 2 * m * m + 8);
}

constexpr int TAIL_SMEM_MAX = 200 * 1024;

// the tail from level l: its shared-memory layout, or nl = 0 when it does not fit
Tail make_tail(const MgState *s, size_t l) {
    Tail T = {};
    if (s->lv.size() - l > (size_t)TAIL_LEVELS) return T;
    int off = 0;
    for (size_t q = l; q < s->lv.size(); q++) {
        const Lv &L = s->lv[q];
        const int n = (L.P[0] + 2) * (int)L.sx;
        const int i = (int)(q - l);
        T.lv[i] = L;
        T.ou[i] = off;
        T.of[i] = off + n;
        T.orr[i] = off + 2 * n;
        T.ot[i] = L.t ? off + 3 * n : -1;
        off += (L.t ? 4 : 3) * n;
    }
    if ((size_t)off * sizeof(float) > (size_t)TAIL_SMEM_MAX) return T;
    T.nl = (int)(s->lv.size() - l);
    T.smem = off;
    T.sweeps = coarse_sweeps(s->lv.back());
    return T;
}

void vcycle(emoo_handle *h, MgState *s, size_t l, int &launches) {
    const Lv &L = s->lv[l];
    dim3 blk(32, 8);
    if (l == s->tail_from) {
        const Tail T = make_tail(s, l);
        launches++;
        k_mg_tail<<<1, TAIL_THREADS, T.smem * sizeof(float), h->stream>>>(T);
        return;
    }
    if (l + 1 == s->lv.size()) {  // a coarsest level too large for the tail
        smooth(h, L, coarse_sweeps(L), launches);
        return;
    }
    const Lv &C = s->lv[l + 1];
    smooth(h, L, NU, launches);
    launches += 2;
    k_mg_residual<<<pts_grid(L, blk), blk, 0, h->stream>>>(L);
    k_mg_restrict<<<pts_grid(C, blk), blk, 0, h->stream>>>(L, C);
    vcycle(h, s, l + 1, launches);
    launches++;
    k_mg_prolong<<<pts_grid(L, blk), blk, 0, h->stream>>>(C, L);
    smooth(h, L, NU, launches);
}

// the FP64 residual, its maximum into the pinned host word
void residual64(emoo_handle *h, MgState *s, int &launches) {
    dim3 blk(32, 8);
    const Lv &L0 = s->lv[0];
    cudaMemsetAsync(s->dmax, 0, sizeof(double), h->stream);
    launches++;
    k_mg_residual64<<<pts_grid(L0, blk), blk, 0, h->stream>>>(L0, s->fine, s->dmax);
    cudaMemcpyAsync(s->hmax, s->dmax, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
}

// one outer step: V-cycle on the correction, u += e, new residual
void outer_step(emoo_handle *h, MgState *s, int &launches) {
    dim3 blk(32, 8);
    vcycle(h, s, 0, launches);
    launches++;
    k_mg_correct<<<pts_grid(s->lv[0], blk), blk, 0, h->stream>>>(s->lv[0], s->fine);
    residual64(h, s, launches);
}

int mg_setup(emoo_handle *h, MgState *s) {
    const Geom &g = h->g;
    bool same = !s->lv.empty();
    for (int d = 0; d < 3 && same; d++)
        same = s->n[d] == g.n[d] && s->per[d] == (h->bc.fbc[2 * d] == FBC_PERIODIC) && s->d[d] == g.d[d];
    if (same) return EMOO_OK;
    mg_release(s);
    for (int d = 0; d < 3; d++) {
        s->n[d] = g.n[d];
        s->per[d] = h->bc.fbc[2 * d] == FBC_PERIODIC;
        s->d[d] = g.d[d];
    }
    int P[3] = {g.n[0], g.n[1], g.n[2]};
    double hh[3] = {g.d[0], g.d[1], g.d[2]};
    for (;;) {
        Lv L = {};
        for (int d = 0; d < 3; d++) {
            L.P[d] = P[d];
            L.per[d] = s->per[d];
            L.lo[d] = L.per[d] ? 1 : 2;
            L.hi[d] = P[d];
            L.c[d] = (float)(1.0 / (hh[d] * hh[d]));
            L.crs[d] = (P[d] % 2 == 0) && P[d] >= 4;
        }
        if (L.hi[0] < L.lo[0] || L.hi[1] < L.lo[1] || L.hi[2] < L.lo[2] || L.hi[0] - L.lo[0] + 1 > 65535) {
            mg_release(s);  // no unknowns (checked by the caller first), or too many planes for one grid launch
            return EMOO_ERR_UNSUPPORTED;
        }
        const double diag = 2.0 * (1.0 / (hh[0] * hh[0]) + 1.0 / (hh[1] * hh[1]) + 1.0 / (hh[2] * hh[2]));
        L.diag = (float)diag;
        L.idiag = (float)(1.0 / diag);
        L.rb = 1;
        for (int d = 0; d < 3; d++)
            if (L.per[d] && (P[d] & 1)) L.rb = 0;
        L.sy = P[2] + 2;
        L.sx = (int64_t)(P[1] + 2) * (P[2] + 2);
        const size_t bytes = (size_t)(P[0] + 2) * L.sx * sizeof(float);
        int rc = alloc_zero((void **)&L.u, bytes, h->stream);
        if (rc == EMOO_OK) rc = alloc_zero((void **)&L.f, bytes, h->stream);
        if (rc == EMOO_OK) rc = alloc_zero((void **)&L.r, bytes, h->stream);
        if (rc == EMOO_OK && !L.rb) rc = alloc_zero((void **)&L.t, bytes, h->stream);
        const bool more = L.crs[0] || L.crs[1] || L.crs[2];
        s->lv.push_back(L);
        if (rc != EMOO_OK) {
            mg_release(s);
            return rc;
        }
        if (!more) break;
        for (int d = 0; d < 3; d++)
            if (L.crs[d]) {
                P[d] /= 2;
                hh[d] *= 2.0;
            }
    }
    // the shared-memory tail: the first level of at most TAIL_MAX unknowns
    // from which the rest fits
    s->tail_from = s->lv.size();
    for (size_t q = 0; q < s->lv.size(); q++)
        if (unknowns(s->lv[q]) <= TAIL_MAX && make_tail(s, q).nl > 0) {
            s->tail_from = q;
            const Tail T = make_tail(s, q);
            cudaError_t e = cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)(T.smem * sizeof(float)));
            if (e != cudaSuccess) {
                mg_release(s);
                return cuda_status(e);
            }
            break;
        }
    const Lv &L0 = s->lv[0];
    const size_t b64 = (size_t)(L0.P[0] + 2) * L0.sx * sizeof(double);
    for (int d = 0; d < 3; d++) s->fine.c[d] = 1.0 / (g.d[d] * g.d[d]);
    s->fine.diag = 2.0 * (s->fine.c[0] + s->fine.c[1] + s->fine.c[2]);
    int rc = alloc_zero((void **)&s->fine.u, b64, h->stream);
    if (rc == EMOO_OK) rc = alloc_zero((void **)&s->fine.f, b64, h->stream);
    if (rc == EMOO_OK) rc = alloc_zero((void **)&s->part, RB * sizeof(double), h->stream);
    if (rc == EMOO_OK) rc = alloc_zero((void **)&s->dmax, sizeof(double), h->stream);
    if (rc == EMOO_OK && cudaMallocHost(&s->hpart, RB * sizeof(double)) != cudaSuccess) rc = EMOO_ERR_OOM;
    if (rc == EMOO_OK && cudaMallocHost(&s->hmax, sizeof(double)) != cudaSuccess) rc = EMOO_ERR_OOM;
    if (rc == EMOO_OK) {  // one outer step as a graph
        int launches = 0;
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            outer_step(h, s, launches);
            e = cudaStreamEndCapture(h->stream, &s->graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&s->exec, s->graph, 0);
        if (e != cudaSuccess) rc = cuda_status(e);
        s->graph_launches = launches;
    }
    if (rc != EMOO_OK) mg_release(s);
    return rc;
}

int sum_unknowns(emoo_handle *h, MgState *s, const double *a, double *out) {
    h->launches++;
    k_mg_sum<<<RB, 256, 0, h->stream>>>(s->lv[0], a, s->part);
    EMOO_CUDA(cudaGetLastError());
    EMOO_CUDA(cudaMemcpyAsync(s->hpart, s->part, RB * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    double v = 0.0;
    for (int b = 0; b < RB; b++) v += s->hpart[b];
    *out = v;
    return EMOO_OK;
}

}  // namespace

void multigrid_free(emoo_handle *h) {
    if (!h->mg) return;
    MgState *s = (MgState *)h->mg;
    mg_release(s);
    delete s;
    h->mg = nullptr;
}

// The solve of one field: u in slot id1 (ghost planes by the reference's
// boundary fill, a copy in id2), f = mult R from slot rid. *cycles receives
// the outer steps (V-cycles) run, *converged whether max |r| <= rtol max |r0|
// was met within the cap.
int multigrid_f64(emoo_handle *h, int id1, int id2, int rid, double mult, int *cycles, int *converged) {
    bool none = false;  // an external dimension of one cell has no unknowns: the boundary planes are the solution
    for (int d = 0; d < 3; d++) none = none || (h->bc.fbc[2 * d] != FBC_PERIODIC && h->g.n[d] < 2);
    if (none) {
        EMOO_CUDA(cudaMemsetAsync(h->slot[id1], 0, (size_t)h->g.npts * sizeof(double), h->stream));
        EMOO_TRY(poisson_field_bc(h, id1));
        EMOO_CUDA(cudaMemcpyAsync(h->slot[id2], h->slot[id1], (size_t)h->g.npts * sizeof(double),
                                  cudaMemcpyDeviceToDevice, h->stream));
        if (cycles) *cycles = 0;
        if (converged) *converged = 1;
        return EMOO_OK;
    }
    if (!h->mg) h->mg = new MgState();
    MgState *s = (MgState *)h->mg;
    EMOO_TRY(mg_setup(h, s));
    const Geom &g = h->g;
    const Lv &L0 = s->lv[0];
    dim3 blk(32, 8);
    // the slot zeroed, then its boundary planes from the reference's fill
    EMOO_CUDA(cudaMemsetAsync(h->slot[id1], 0, (size_t)g.npts * sizeof(double), h->stream));
    EMOO_TRY(poisson_field_bc(h, id1));
    {
        const int ek = L0.per[2] ? L0.P[2] : L0.P[2] + 1, ej = L0.per[1] ? L0.P[1] : L0.P[1] + 1;
        const int ei = L0.per[0] ? L0.P[0] : L0.P[0] + 1;
        dim3 grd((ek + blk.x - 1) / blk.x, (ej + blk.y - 1) / blk.y, ei);
        h->launches++;
        k_mg_load<<<grd, blk, 0, h->stream>>>(g, L0, s->fine, h->slot[id1], h->slot[rid], mult);
    }
    const bool allper = L0.per[0] && L0.per[1] && L0.per[2];
    const double nunk = (double)unknowns(L0);
    if (allper) {  // the singular periodic system is consistent only for a mean-free right side
        double sum;
        EMOO_TRY(sum_unknowns(h, s, s->fine.f, &sum));
        h->launches++;
        k_mg_shift<<<pts_grid(L0, blk), blk, 0, h->stream>>>(L0, s->fine.f, sum / nunk);
    }
    int launches = 0;
    residual64(h, s, launches);
    h->launches += launches;
    EMOO_CUDA(cudaGetLastError());
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    const double r0 = *s->hmax;
    const double tol = h->poisson_rtol * r0;
    int it = 0;
    const int cap = 200;
    bool ok = r0 == 0.0;
    while (!ok && it < cap) {
        EMOO_CUDA(cudaGraphLaunch(s->exec, h->stream));
        h->launches += s->graph_launches;
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
        it++;
        ok = *s->hmax <= tol;
    }
    double shift = 0.0;
    if (allper) {
        double sum;
        EMOO_TRY(sum_unknowns(h, s, s->fine.u, &sum));
        shift = sum / nunk;
    }
    h->launches++;
    k_mg_store<<<pts_grid(L0, blk), blk, 0, h->stream>>>(g, L0, s->fine.u, h->slot[id1], shift);
    EMOO_CUDA(cudaGetLastError());
    EMOO_TRY(poisson_field_bc(h, id1));
    EMOO_CUDA(cudaMemcpyAsync(h->slot[id2], h->slot[id1], (size_t)g.npts * sizeof(double), cudaMemcpyDeviceToDevice,
                              h->stream));
    if (cycles) *cycles = it;
    if (converged) *converged = ok ? 1 : 0;
    return EMOO_OK;
}

}  // namespace emoo
