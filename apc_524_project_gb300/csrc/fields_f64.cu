// fields_f64.cu - FP64 grid kernels: Yee E/B update, ghost fill, periodic
// J/rho fold, LightBC / Dirichlet plane sets, Jacobi Poisson sweeps, phiToE,
// AToB, field-energy and Gauss-law reductions.
//
// Compiled with --fmad=false: every expression keeps the reference's order of
// operations with separately rounded multiplies and adds, so on identical
// inputs the results are bit-identical to the reference serial build.
// All kernels are HBM-bound stencils over the (n+3)^3 reference layout with
// k (the contiguous axis) mapped to threadIdx.x for coalescing.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {

namespace {

constexpr double FOURPI = 4.0 * PI_D;

struct F3 {
    double *p[3];
};
struct CF3 {
    const double *p[3];
};

dim3 phys_grid(const Geom &g, dim3 blk) {
    return dim3((g.n[2] + blk.x - 1) / blk.x, (g.n[1] + blk.y - 1) / blk.y, g.n[0]);
}

// Grid::evolveFields, E half (src/grid/oGrid.cpp:23-40): E -= dt (curl-ish of
// B_tm1 + 4 pi J) over physical points, B_tm1 being the freshly swapped role.
__global__ void k_yee_e(Geom g, double dt, F3 E, CF3 T, CF3 J) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    const double *Tx = T.p[0], *Ty = T.p[1], *Tz = T.p[2];
    double dx = g.d[0], dy = g.d[1], dz = g.d[2];
    double ex = E.p[0][o] - dt * (ddiv(Ty[o] - Ty[o - 1], dz, g.id[2], g.p2[2]) -
                                  ddiv(Tz[o] - Tz[o - g.sy], dy, g.id[1], g.p2[1]) + FOURPI * J.p[0][o]);
    double ey = E.p[1][o] - dt * (ddiv(Tz[o] - Tz[o - g.sx], dx, g.id[0], g.p2[0]) -
                                  ddiv(Tx[o] - Tx[o - 1], dz, g.id[2], g.p2[2]) + FOURPI * J.p[1][o]);
    double ez = E.p[2][o] - dt * (ddiv(Tx[o] - Tx[o - g.sy], dy, g.id[1], g.p2[1]) -
                                  ddiv(Ty[o] - Ty[o - g.sx], dx, g.id[0], g.p2[0]) + FOURPI * J.p[2][o]);
    E.p[0][o] = ex;
    E.p[1][o] = ey;
    E.p[2][o] = ez;
}

// Grid::evolveFields, B half (src/grid/oGrid.cpp:43-57): B = B_tm1 + dt curl E.
// Reads the E ghost planes as they are (refreshed only after the update).
__global__ void k_yee_b(Geom g, double dt, F3 B, CF3 T, CF3 E) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    const double *Ex = E.p[0], *Ey = E.p[1], *Ez = E.p[2];
    double dx = g.d[0], dy = g.d[1], dz = g.d[2];
    B.p[0][o] = T.p[0][o] + dt * (ddiv(Ey[o + 1] - Ey[o], dz, g.id[2], g.p2[2]) -
                                  ddiv(Ez[o + g.sy] - Ez[o], dy, g.id[1], g.p2[1]));
    B.p[1][o] = T.p[1][o] + dt * (ddiv(Ez[o + g.sx] - Ez[o], dx, g.id[0], g.p2[0]) -
                                  ddiv(Ex[o + 1] - Ex[o], dz, g.id[2], g.p2[2]));
    B.p[2][o] = T.p[2][o] + dt * (ddiv(Ex[o + g.sy] - Ex[o], dy, g.id[1], g.p2[1]) -
                                  ddiv(Ey[o + g.sx] - Ey[o], dx, g.id[0], g.p2[0]));
}

// Grid::evolveFieldsES, src/grid/oGrid.cpp:67-81
__global__ void k_yee_es(Geom g, double dt, F3 E, CF3 J) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    double mdt = -dt;
    E.p[0][o] = mdt * (FOURPI * J.p[0][o]);
    E.p[1][o] = mdt * (FOURPI * J.p[1][o]);
    E.p[2][o] = mdt * (FOURPI * J.p[2][o]);
}

struct FieldList {
    double *p[6];
    int n;
};

// Periodic ghost fill (BC_F_Periodic::completeBC for sendID -1 or one field,
// src/boundaries/b_fields/bc_f_periodic.cpp:47-52 via
// src/grid/spookyGrid.cpp:17-184): ghost plane 0 <- plane n, ghost plane
// n+1 <- plane 1, over the physical transverse range only. All copies read
// physical points and write ghost points, so any set of dims runs at once.
// blockIdx.z = (field * 3 + dim) * 2 + side.
__global__ void k_ghost(Geom g, FieldList fl, int dims_mask, const int *skip) {
    if (skip && *skip) return;
    int z = blockIdx.z;
    int r = z & 1;
    int d = (z >> 1) % 3;
    int f = (z >> 1) / 3;
    if (!((dims_mask >> d) & 1) || f >= fl.n) return;
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int p = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || p > g.n[o1]) return;
    int nd = g.n[d];
    int src = r == 0 ? nd : 1, dst = r == 0 ? 0 : nd + 1;
    int is[3], it[3];
    is[d] = src;
    it[d] = dst;
    is[o1] = it[o1] = p;
    is[o2] = it[o2] = q;
    double *F = fl.p[f];
    F[gidx(g, it[0], it[1], it[2])] = F[gidx(g, is[0], is[1], is[2])];
}

// Periodic fold of one dimension (BC_F_Periodic::completeBC(-2) of the left
// side, src/boundaries/b_fields/bc_f_periodic.cpp:40-46): the two transverse
// J components and rho of ghost plane n+1 are added into plane 1.
__global__ void k_fold(Geom g, int d, double *f0, double *f1, double *f2) {
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int p = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || p > g.n[o1]) return;
    int is[3], it[3];
    is[d] = g.n[d] + 1;
    it[d] = 1;
    is[o1] = it[o1] = p;
    is[o2] = it[o2] = q;
    int64_t s = gidx(g, is[0], is[1], is[2]), t = gidx(g, it[0], it[1], it[2]);
    double *F = blockIdx.z == 0 ? f0 : (blockIdx.z == 1 ? f1 : f2);
    F[t] += F[s];
}

struct PlaneList {
    PlaneSet s[12];
    int n;
};

// Grid::setFieldInPlane over the whole (n+3)^2 plane, src/grid/oGrid.cpp:446-476.
__global__ void k_plane_set(Geom g, PlaneList pl, const int *skip) {
    if (skip && *skip) return;
    int e = blockIdx.z;
    if (e >= pl.n) return;
    const PlaneSet &ps = pl.s[e];
    int d = ps.dim;
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int p = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= g.tot[o2] || p >= g.tot[o1]) return;
    int ii[3];
    ii[d] = ps.idx;
    ii[o1] = p;
    ii[o2] = q;
    double v = ps.v;
    if (ps.t1) v = __dadd_rn(v, __dmul_rn(__dmul_rn(ps.vs, ps.t1[p]), ps.t2[q]));  // v + (vs t1) t2
    ps.f[gidx(g, ii[0], ii[1], ii[2])] = v;
}

__global__ void k_fill(double *p, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// ---- Jacobi ----

struct JacobiState {
    int done;
    int iter;       // iterations completed
    int converged;
    int skip;       // boundary fills no-ops (one sweep after done, with the test in the sweep)
    double maxdiff; // current iteration's max |u2 - u1|
    unsigned int blocks_done;
    unsigned int pad2;
};

// One Jacobi sweep, src/poisson/poisson.cpp:216-241.
__global__ void k_jacobi(Geom g, const double *src, double *dst, const double *R, double ax, double ay, double az,
                         double af, double mult, const JacobiState *st) {
    if (st->done) return;
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    dst[o] = ax * (src[o - g.sx] + src[o + g.sx]) + ay * (src[o - g.sy] + src[o + g.sy]) +
             az * (src[o - 1] + src[o + 1]) - af * R[o] * mult;
}

// max |u2 - u1| over physical points, then convergence bookkeeping by the
// last block (src/poisson/poisson.cpp:250-283).
__global__ void k_jacobi_check(Geom g, const double *u1, const double *u2, double tol, JacobiState *st) {
    if (st->done) return;
    __shared__ double smax[32];
    __shared__ bool last;
    double m = 0.0;
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nphys; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        phys_ijk(g.n, t, i, j, k);
        int64_t o = gidx(g, i, j, k);
        double a = fabs(u2[o] - u1[o]);
        m = a > m ? a : m;
    }
    for (int off = 16; off > 0; off >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) smax[w] = m;
    __syncthreads();
    if (w == 0) {
        m = lane < (int)(blockDim.x >> 5) ? smax[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            double o = __shfl_down_sync(0xffffffffu, m, off);
            m = o > m ? o : m;
        }
        if (lane == 0) {
            atomic_max_nonneg(&st->maxdiff, m);
            __threadfence();
            unsigned int prev = atomicAdd(&st->blocks_done, 1u);
            last = (prev == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double md = *((volatile double *)&st->maxdiff);
        int it = st->iter;  // iternum of this iteration
        if (md < tol) {
            st->done = 1;
            st->converged = 1;
        } else if (it >= ITER_MAX) {
            st->done = 1;
            st->converged = 0;
        }
        st->iter = it + 1;
        st->maxdiff = 0.0;
        st->blocks_done = 0u;
    }
}

// One Jacobi sweep with the stop test of k_jacobi_check folded in, for grids
// periodic on every side: there the boundary fill writes only ghost planes,
// so max |u2 - u1| over the physical points is max |dst - src| of this sweep,
// the same value in any order. The sweep's arithmetic is k_jacobi's. Once the
// test has fired, the next sweep sets `skip`, so the fill after the last
// sweep still runs and the later ones do not.
__global__ void k_jacobi_fused(Geom g, const double *src, double *dst, const double *R, double ax, double ay,
                               double az, double af, double mult, double tol, JacobiState *st) {
    if (st->done) {
        if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0) st->skip = 1;
        return;
    }
    __shared__ double smax[32];
    __shared__ bool last;
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int i = blockIdx.z + 1;
    double m = 0.0;
    if (k <= g.n[2] && j <= g.n[1]) {
        const int64_t o = gidx(g, i, j, k);
        const double v = ax * (src[o - g.sx] + src[o + g.sx]) + ay * (src[o - g.sy] + src[o + g.sy]) +
                         az * (src[o - 1] + src[o + 1]) - af * R[o] * mult;
        dst[o] = v;
        m = fabs(v - src[o]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double q = __shfl_down_sync(0xffffffffu, m, off);
        m = q > m ? q : m;
    }
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nw = (int)((blockDim.x * blockDim.y) >> 5);
    if (lane == 0) smax[w] = m;
    __syncthreads();
    if (w == 0) {
        m = lane < nw ? smax[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            const double q = __shfl_down_sync(0xffffffffu, m, off);
            m = q > m ? q : m;
        }
        if (lane == 0) {
            atomic_max_nonneg(&st->maxdiff, m);
            __threadfence();
            const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
            const unsigned int prev = atomicAdd(&st->blocks_done, 1u);
            last = (prev == nb - 1);
        }
    }
    __syncthreads();
    if (last && tid == 0) {
        __threadfence();
        const double md = *((volatile double *)&st->maxdiff);
        const int it = st->iter;
        if (md < tol) {
            st->done = 1;
            st->converged = 1;
        } else if (it >= ITER_MAX) {
            st->done = 1;
            st->converged = 0;
        }
        st->iter = it + 1;
        st->maxdiff = 0.0;
        st->blocks_done = 0u;
    }
}

// phiToE, src/poisson/convertFields.cpp:20-68 (reads phi1 storage).
__global__ void k_phi_to_e(Geom g, const double *phi, F3 E) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    E.p[0][o] = ddiv(-(phi[o + g.sx] - phi[o]), g.d[0], g.id[0], g.p2[0]);
    E.p[1][o] = ddiv(-(phi[o + g.sy] - phi[o]), g.d[1], g.id[1], g.p2[1]);
    E.p[2][o] = ddiv(-(phi[o + 1] - phi[o]), g.d[2], g.id[2], g.p2[2]);
}

// AToB, src/poisson/convertFields.cpp:83-154, including its use of the same
// A component in both differences.
__global__ void k_a_to_b(Geom g, const double *Ax, const double *Ay, const double *Az, F3 B) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    int64_t o = gidx(g, i, j, k);
    // Bx: Ak = Az (hk = dz), Aj = Ay (hj = dy); next_k = Ak[j+1], next_j = Ak[k+1]
    B.p[0][o] = ddiv(Az[o + g.sy] - Az[o], g.d[1], g.id[1], g.p2[1]) + ddiv(Az[o + 1] - Ay[o], g.d[2], g.id[2], g.p2[2]);
    // By: Ak = Ax (hk = dx), Aj = Az (hj = dz); next_k = Ak[k+1], next_j = Ak[i+1]
    B.p[1][o] = ddiv(Ax[o + 1] - Ax[o], g.d[2], g.id[2], g.p2[2]) + ddiv(Ax[o + g.sx] - Az[o], g.d[0], g.id[0], g.p2[0]);
    // Bz: Ak = Ay (hk = dy), Aj = Ax (hj = dx); next_k = Ak[i+1], next_j = Ak[j+1]
    B.p[2][o] = ddiv(Ay[o + g.sx] - Ay[o], g.d[0], g.id[0], g.p2[0]) + ddiv(Ay[o + g.sy] - Ax[o], g.d[1], g.id[1], g.p2[1]);
}

// Per-block partial sums of the six field energies of the history row
// (src/IO/output.cpp:98-114; SQR(x) expands to x*x unparenthesised).
__global__ void k_field_energy(Geom g, CF3 E, CF3 B, double *part) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    double hv = 0.5 * g.vol;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nphys; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        phys_ijk(g.n, t, i, j, k);
        int64_t o = gidx(g, i, j, k);
        int64_t nb[3] = {o + g.sx, o + g.sy, o + 1};
        for (int q = 0; q < 3; q++) {
            double s = E.p[q][o] + E.p[q][nb[q]];
            acc[q] += hv * (0.5 * s * 0.5 * s);
            double sb = B.p[q][o] + B.p[q][nb[q]];
            acc[3 + q] += hv * (0.5 * sb * 0.5 * sb);
        }
    }
    __shared__ double sh[32][6];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 6; q++) {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) v += sh[ww][threadIdx.x];
        part[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

// Gauss-law residual partials: {max |div E - 4 pi rho|, sum r^2}.
__global__ void k_gauss(Geom g, CF3 E, const double *rho, double *part) {
    double mx = 0.0, s2 = 0.0;
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nphys; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        phys_ijk(g.n, t, i, j, k);
        int64_t o = gidx(g, i, j, k);
        double dv = ddiv(E.p[0][o] - E.p[0][o - g.sx], g.d[0], g.id[0], g.p2[0]) +
                    ddiv(E.p[1][o] - E.p[1][o - g.sy], g.d[1], g.id[1], g.p2[1]) +
                    ddiv(E.p[2][o] - E.p[2][o - 1], g.d[2], g.id[2], g.p2[2]);
        double res = dv - FOURPI * rho[o];
        double a = fabs(res);
        mx = a > mx ? a : mx;
        s2 += res * res;
    }
    __shared__ double sh[32][2];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, mx, off);
        mx = o > mx ? o : mx;
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
    }
    if (lane == 0) {
        sh[w][0] = mx;
        sh[w][1] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) {
            a = sh[ww][0] > a ? sh[ww][0] : a;
            b += sh[ww][1];
        }
        part[blockIdx.x * 2] = a;
        part[blockIdx.x * 2 + 1] = b;
    }
}

int ensure_red(emoo_handle *h, size_t n) {
    if (h->red_cap >= n) return EMOO_OK;
    if (h->red) cudaFree(h->red);
    h->red = nullptr;
    EMOO_CUDA(cudaMalloc(&h->red, n * sizeof(double)));
    h->red_cap = n;
    return EMOO_OK;
}

int reduce_blocks(const Geom &g) {
    int64_t nphys = (int64_t)g.n[0] * g.n[1] * g.n[2];
    int64_t b = (nphys + 255) / 256;
    return (int)std::min<int64_t>(b, 152 * 8);
}

}  // namespace

double *role_b(emoo_handle *h, int c) { return h->bswap ? h->slot[EMOO_BX_TM1 + c] : h->slot[EMOO_BX + c]; }
double *role_t(emoo_handle *h, int c) { return h->bswap ? h->slot[EMOO_BX + c] : h->slot[EMOO_BX_TM1 + c]; }

int yee_f64(emoo_handle *h, double dt) {
    // std::swap of the member pointers only (src/grid/oGrid.cpp:18-20)
    h->bswap ^= 1;
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 grd = phys_grid(g, blk);
    F3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
    CF3 T = {{role_t(h, 0), role_t(h, 1), role_t(h, 2)}};
    CF3 J = {{h->slot[EMOO_JX], h->slot[EMOO_JY], h->slot[EMOO_JZ]}};
    h->launches++;
    k_yee_e<<<grd, blk, 0, h->stream>>>(g, dt, E, T, J);
    // The B half reads E one plane past the high faces. The reference refreshes
    // those ghosts only after both halves, so at the periodic wrap B sees the
    // previous step's E: the leapfrog loses its time centring there and vacuum
    // fields grow without bound at dt 0.5. The corrected policy refreshes them.
    if (h->policy == EMOO_POLICY_CORRECTED) EMOO_TRY(ghost_e_full_f64(h));
    F3 B = {{role_b(h, 0), role_b(h, 1), role_b(h, 2)}};
    CF3 Ec = {{E.p[0], E.p[1], E.p[2]}};
    h->launches++;
    k_yee_b<<<grd, blk, 0, h->stream>>>(g, dt, B, T, Ec);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int yee_half_f64(emoo_handle *h, double dt, int half) {
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 grd = phys_grid(g, blk);
    CF3 T = {{role_t(h, 0), role_t(h, 1), role_t(h, 2)}};
    h->launches++;
    if (half == 0) {
        F3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
        CF3 J = {{h->slot[EMOO_JX], h->slot[EMOO_JY], h->slot[EMOO_JZ]}};
        k_yee_e<<<grd, blk, 0, h->stream>>>(g, dt, E, T, J);
    } else {
        F3 B = {{role_b(h, 0), role_b(h, 1), role_b(h, 2)}};
        CF3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
        k_yee_b<<<grd, blk, 0, h->stream>>>(g, dt, B, T, E);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int yee_es_f64(emoo_handle *h, double dt) {
    const Geom &g = h->g;
    dim3 blk(32, 8);
    F3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
    CF3 J = {{h->slot[EMOO_JX], h->slot[EMOO_JY], h->slot[EMOO_JZ]}};
    h->launches++;
    k_yee_es<<<phys_grid(g, blk), blk, 0, h->stream>>>(g, dt, E, J);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

static int ghost_launch(emoo_handle *h, const int *ids, int nids, int dims_mask, const int *skip) {
    const Geom &g = h->g;
    FieldList fl;
    fl.n = nids;
    for (int i = 0; i < nids; i++) fl.p[i] = h->slot[ids[i]];
    int ta = std::max(g.n[1], g.n[0]);
    int tb = std::max(g.n[2], g.n[1]);
    dim3 blk(32, 8);
    dim3 grd((tb + 31) / 32, (ta + 7) / 8, nids * 6);
    h->launches++;
    k_ghost<<<grd, blk, 0, h->stream>>>(g, fl, dims_mask, skip);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int ghost_fill_f64(emoo_handle *h, const int *ids, int nids, int dims_mask) {
    return ghost_launch(h, ids, nids, dims_mask, nullptr);
}

// what: FOLD_J (the two transverse J components), FOLD_RHO, or both
int fold_f64(emoo_handle *h, int d, int what) {
    const Geom &g = h->g;
    int f0 = (d == 0) ? EMOO_JY : EMOO_JX;
    int f1 = (d == 2) ? EMOO_JY : EMOO_JZ;
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    dim3 blk(32, 8);
    double *a = h->slot[f0], *b = h->slot[f1], *r = h->slot[EMOO_RHO];
    int nz = 3;
    if (what == FOLD_J) nz = 2;
    if (what == FOLD_RHO) {
        nz = 1;
        a = r;
    }
    dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, nz);
    h->launches++;
    k_fold<<<grd, blk, 0, h->stream>>>(g, d, a, b, r);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// ---- corrected policy: periodic copies and folds over the whole range ----

struct Slots9 {
    double *p[9];
};

// Along dim d, for every transverse point of the whole (n+3)^2 plane:
// fold = 1: f[n] += f[0], f[1] += f[n+1], f[2] += f[n+2] (the ghost planes'
// deposits to their periodic images); fold = 0: f[0] = f[n], f[n+1] = f[1],
// f[n+2] = f[2] (the ghost planes refreshed). One field per blockIdx.z.
__global__ void k_periodic_full(Geom g, Slots9 fl, int d, int fold) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= g.tot[o2] || r >= g.tot[o1]) return;
    double *F = fl.p[blockIdx.z];
    const int n = g.n[d];
    int c[3];
    c[o1] = r;
    c[o2] = q;
    auto at = [&](int i) -> double & {
        c[d] = i;
        return F[gidx(g, c[0], c[1], c[2])];
    };
    if (fold) {
        at(n) += at(0);
        at(1) += at(n + 1);
        at(2) += at(n + 2);
    } else {
        at(0) = at(n);
        at(n + 1) = at(1);
        at(n + 2) = at(2);
    }
}

// Mirror fold at a reflecting wall (corrected policy, no reference
// counterpart): a particle reflected at the wall moved along the mirror image
// of the part of its straight path beyond it, so the current that part
// deposited in the ghost layer goes to the mirrored points inside - the
// component normal to the wall negated, the transverse ones as they are - and
// the ghost values are cleared. Left wall (vertex plane 1): normal edge 0 ->
// 1, transverse plane 0 -> 2; right wall (plane n+1): normal edge n+1 -> n,
// transverse plane n+2 -> n. Whole transverse range; blockIdx.z = component.
__global__ void k_mirror_fold(Geom g, Slots9 fl, int d, int right) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= g.tot[o2] || r >= g.tot[o1]) return;
    const int a = blockIdx.z;
    double *F = fl.p[a];
    const int n = g.n[d];
    const bool normal = a == d;
    const int src = normal ? (right ? n + 1 : 0) : (right ? n + 2 : 0);
    const int dst = normal ? (right ? n : 1) : (right ? n : 2);
    int c[3];
    c[o1] = r;
    c[o2] = q;
    c[d] = src;
    const int64_t ks = gidx(g, c[0], c[1], c[2]);
    c[d] = dst;
    const int64_t kd = gidx(g, c[0], c[1], c[2]);
    if (normal) F[kd] -= F[ks];
    else F[kd] += F[ks];
    F[ks] = 0.0;
}

// The corrected policy's folds (fold = 1, the arrays J and / or rho) or ghost
// copies (fold = 0), dimension by dimension so edge and corner lines follow:
// periodic dimensions as images over the whole range; walled dimensions
// (corrected policy with reflecting or absorbing particle sides) fold J by
// mirror at reflecting sides only (at absorbing ones the current of the path
// beyond the wall stays in the ghost layer) and copy nothing (their field
// sides are LightBC planes).
static int periodic_full(emoo_handle *h, const int *ids, int nids, int fold) {
    const Geom &g = h->g;
    Slots9 fl;
    for (int k = 0; k < nids; k++) fl.p[k] = h->slot[ids[k]];
    dim3 blk(32, 8);
    for (int d = 0; d < 3; d++) {
        const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
        if (h->bc.fbc[2 * d] != FBC_PERIODIC) {
            const bool j3 = fold && nids >= 3 && ids[0] == EMOO_JX && ids[1] == EMOO_JY && ids[2] == EMOO_JZ;
            for (int r = 0; r < 2 && j3; r++) {
                if (h->bc.pbc[2 * d + r] != PBC_REFLECTING) continue;
                dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, 3);
                h->launches++;
                k_mirror_fold<<<grd, blk, 0, h->stream>>>(g, fl, d, r);
            }
            continue;
        }
        dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, nids);
        h->launches++;
        k_periodic_full<<<grd, blk, 0, h->stream>>>(g, fl, d, fold);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// what: FOLD_J (the three J components), FOLD_RHO, or both
int fold_full_f64(emoo_handle *h, int what) {
    int ids[4], n = 0;
    if (what & FOLD_J)
        for (int c = 0; c < 3; c++) ids[n++] = EMOO_JX + c;
    if (what & FOLD_RHO) ids[n++] = EMOO_RHO;
    return periodic_full(h, ids, n, 1);
}

// LightBC planes of every external side (E and B roles through the slots).
static int light_all_f64(emoo_handle *h) {
    for (int s = 0; s < 6; s++) {
        if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
        PlaneSet ps[6];
        const int n = light_planes_slots(h, s, ps);
        EMOO_TRY(plane_set_f64(h, ps, n));
    }
    return EMOO_OK;
}

// E's boundary values between the Yee halves (corrected policy): periodic
// images and LightBC planes, so the B half reads E at the new time everywhere.
int ghost_e_full_f64(emoo_handle *h) {
    static const int ids[3] = {EMOO_EX, EMOO_EY, EMOO_EZ};
    EMOO_TRY(periodic_full(h, ids, 3, 0));
    return light_all_f64(h);
}

int periodic_copies_f64(emoo_handle *h, const int *ids, int nids) { return periodic_full(h, ids, nids, 0); }

int ghost_full_f64(emoo_handle *h) {
    static const int ids[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ, EMOO_BX_TM1, EMOO_BY_TM1,
                               EMOO_BZ_TM1};
    EMOO_TRY(periodic_full(h, ids, 9, 0));
    return light_all_f64(h);
}

static int plane_launch(emoo_handle *h, const PlaneSet *ps, int n, const int *skip) {
    const Geom &g = h->g;
    for (int b = 0; b < n; b += 12) {
        PlaneList pl;
        pl.n = std::min(12, n - b);
        for (int i = 0; i < pl.n; i++) pl.s[i] = ps[b + i];
        int m = std::max(std::max(g.tot[0], g.tot[1]), g.tot[2]);
        dim3 blk(32, 8);
        dim3 grd((m + 31) / 32, (m + 7) / 8, pl.n);
        h->launches++;
        k_plane_set<<<grd, blk, 0, h->stream>>>(g, pl, skip);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int plane_set_f64(emoo_handle *h, const PlaneSet *ps, int n) { return plane_launch(h, ps, n, nullptr); }

// rho += background at the physical points with x index >= i0 (immobile
// neutralising ions; no reference counterpart).
__global__ void k_add_phys(Geom g, double *f, double v, int i0) {
    int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    int i = blockIdx.z + i0;
    if (k > g.n[2] || j > g.n[1]) return;
    f[(int64_t)i * g.sx + (int64_t)j * g.sy + k] += v;
}

int rho_background_f64(emoo_handle *h, int with_rho) {
    if (!with_rho || h->opts.rho_background == 0.0 || h->rho_bg_first > h->g.n[0]) return EMOO_OK;
    const Geom &g = h->g;
    dim3 blk(32, 8);
    dim3 grd((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0] - h->rho_bg_first + 1);
    h->launches++;
    k_add_phys<<<grd, blk, 0, h->stream>>>(g, h->slot[EMOO_RHO], h->opts.rho_background, h->rho_bg_first);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int fill_f64(emoo_handle *h, double *p, int64_t n, double v, cudaStream_t s) {
    (void)h;
    int64_t b = std::min<int64_t>((n + 255) / 256, 152 * 16);
    if (b < 1) b = 1;
    h->launches++;
    k_fill<<<(int)b, 256, 0, s>>>(p, n, v);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// executeBC(fieldID) for one Poisson field: periodic dims by ghost copy,
// external sides by PoissonBC Dirichlet planes (left: plane 1, right: n+1),
// in the reference's dimension order; `skip` makes the launches no-ops once
// the Jacobi loop has finished.
static int single_field_bc(emoo_handle *h, int id, const int *skip) {
    int mask_run = 0;
    for (int d = 0; d < 3; d++) {
        bool per = h->bc.fbc[2 * d] == FBC_PERIODIC;
        if (per) {
            mask_run |= 1 << d;
            continue;
        }
        if (mask_run) {
            EMOO_TRY(ghost_launch(h, &id, 1, mask_run, skip));
            mask_run = 0;
        }
        if (!h->poisson || id <= 0) continue;
        PlaneSet ps[2] = {};
        int np = 0;
        for (int r = 0; r < 2; r++) {
            int s = 2 * d + r;
            if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
            int fid = (id == EMOO_PHI1 || id == EMOO_PHI2) ? 0 : (id == EMOO_AX1 || id == EMOO_AX2) ? 1
                      : (id == EMOO_AY1 || id == EMOO_AY2) ? 2 : (id == EMOO_AZ1 || id == EMOO_AZ2) ? 3 : -1;
            if (fid < 0) continue;
            double v = fid == 0 ? h->info.bound_phi[s] : fid == 1 ? h->info.bound_Ax[s]
                                : fid == 2 ? h->info.bound_Ay[s] : h->info.bound_Az[s];
            ps[np].f = h->slot[id];
            ps[np].dim = d;
            ps[np].idx = r == 0 ? 1 : h->g.n[d] + 1;
            ps[np].v = v;
            np++;
        }
        for (int i = 0; i < np; i++) EMOO_TRY(plane_launch(h, &ps[i], 1, skip));
    }
    if (mask_run) EMOO_TRY(ghost_launch(h, &id, 1, mask_run, skip));
    return EMOO_OK;
}

// The Poisson fields' boundary fill (executeBC(fieldID)) as the Jacobi loop
// applies it, for the multigrid's start and result.
int poisson_field_bc(emoo_handle *h, int id) { return single_field_bc(h, id, nullptr); }

// Poisson_Solver::run_poisson_solver_, src/poisson/poisson.cpp:172-287, with
// the iteration control on the device: iterations are queued in batches and
// become no-ops once the stop test of the reference has fired.
int jacobi_f64(emoo_handle *h, int id1, int id2, int rid, double tol, double mult, int *iters, int *converged) {
    const Geom &g = h->g;
    double dx = g.d[0], dy = g.d[1], dz = g.d[2];
    double celldist2 = pow(dx, 2.0) * pow(dy, 2.0) + pow(dy, 2.0) * pow(dz, 2.0) + pow(dx, 2.0) * pow(dz, 2.0);
    double ax = pow(dy, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    double ay = pow(dx, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    double az = pow(dx, 2.0) * pow(dy, 2.0) / (2.0 * celldist2);
    double af = pow(dx, 2.0) * pow(dy, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    if (!h->jacobi_state) EMOO_CUDA(cudaMalloc(&h->jacobi_state, sizeof(JacobiState)));
    JacobiState *st = (JacobiState *)h->jacobi_state;
    EMOO_CUDA(cudaMemsetAsync(st, 0, sizeof(JacobiState), h->stream));
    EMOO_TRY(single_field_bc(h, id1, nullptr));
    double *u1 = h->slot[id1], *u2 = h->slot[id2];
    const double *R = h->slot[rid];
    dim3 blk(32, 8);
    dim3 grd = phys_grid(g, blk);
    int rb = reduce_blocks(g);
    // Sweeps are queued in batches of 32 (an even count, so every batch starts
    // on the same ping-pong parity), captured once as a CUDA graph and
    // replayed: at small grids each sweep's three kernels would otherwise cost
    // a launch latency each. Once the stop test has fired they are no-ops.
    const int batch = 32;
    int batch_launches = 0;
    // With every side periodic the stop test can run inside the sweep: one
    // kernel fewer per sweep, which pays where launches dominate. On large
    // grids the sweep's per-block FP64 max trees (FP64 pipe) cost more than
    // the separate check's grid-stride reduction, so it stays separate there.
    bool all_periodic = (int64_t)g.n[0] * g.n[1] * g.n[2] <= (int64_t)1 << 21;
    for (int sd = 0; sd < 6; sd++) all_periodic = all_periodic && h->bc.fbc[sd] == FBC_PERIODIC;
    auto queue_batch = [&]() -> int {
        for (int b = 0; b < batch; b++) {
            const bool even = (b % 2) == 0;
            batch_launches++;
            if (all_periodic)  // (and small)
                k_jacobi_fused<<<grd, blk, 0, h->stream>>>(g, even ? u1 : u2, even ? u2 : u1, R, ax, ay, az, af, mult,
                                                           tol, st);
            else
                k_jacobi<<<grd, blk, 0, h->stream>>>(g, even ? u1 : u2, even ? u2 : u1, R, ax, ay, az, af, mult, st);
            const int64_t before = h->launches;
            EMOO_TRY(single_field_bc(h, even ? id2 : id1, all_periodic ? &st->skip : &st->done));
            batch_launches += (int)(h->launches - before);
            h->launches = before;
            if (!all_periodic) {
                batch_launches++;
                k_jacobi_check<<<rb, 256, 0, h->stream>>>(g, u1, u2, tol, st);
            }
        }
        return EMOO_OK;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    EMOO_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int qrc = queue_batch();
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (qrc != EMOO_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return qrc != EMOO_OK ? qrc : cuda_status(ce);
    }
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_status(ie);
    JacobiState hs;
    int launched = 0;
    int rc = EMOO_OK;
    for (;;) {
        cudaError_t e = cudaGraphLaunch(exec, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) {
            rc = cuda_status(e);
            break;
        }
        h->launches += batch_launches;
        launched += batch;
        if (hs.done || launched > ITER_MAX) break;
    }
    cudaGraphExecDestroy(exec);
    if (rc != EMOO_OK) return rc;
    if (iters) *iters = hs.iter - 1;
    if (converged) *converged = hs.converged;
    return EMOO_OK;
}

int phi_to_e_f64(emoo_handle *h) {
    const Geom &g = h->g;
    dim3 blk(32, 8);
    F3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
    h->launches++;
    k_phi_to_e<<<phys_grid(g, blk), blk, 0, h->stream>>>(g, h->slot[EMOO_PHI1], E);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int a_to_b_f64(emoo_handle *h) {
    const Geom &g = h->g;
    dim3 blk(32, 8);
    // AToB writes through the field pointer table: the fixed B slots.
    F3 B = {{h->slot[EMOO_BX], h->slot[EMOO_BY], h->slot[EMOO_BZ]}};
    h->launches++;
    k_a_to_b<<<phys_grid(g, blk), blk, 0, h->stream>>>(g, h->slot[EMOO_AX1], h->slot[EMOO_AY1], h->slot[EMOO_AZ1], B);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int field_energy_f64(emoo_handle *h, double out6[6]) {
    const Geom &g = h->g;
    int rb = reduce_blocks(g);
    EMOO_TRY(ensure_red(h, (size_t)rb * 6));
    CF3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
    // the history reads the field pointer table: fixed B slots
    CF3 B = {{h->slot[EMOO_BX], h->slot[EMOO_BY], h->slot[EMOO_BZ]}};
    h->launches++;
    k_field_energy<<<rb, 256, 0, h->stream>>>(g, E, B, h->red);
    EMOO_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)rb * 6);
    EMOO_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (int q = 0; q < 6; q++) out6[q] = 0.0;
    for (int b = 0; b < rb; b++)
        for (int q = 0; q < 6; q++) out6[q] += part[(size_t)b * 6 + q];
    return EMOO_OK;
}

int gauss_residual_f64(emoo_handle *h, double out2[2]) {
    const Geom &g = h->g;
    int rb = reduce_blocks(g);
    EMOO_TRY(ensure_red(h, (size_t)rb * 2));
    CF3 E = {{h->slot[EMOO_EX], h->slot[EMOO_EY], h->slot[EMOO_EZ]}};
    h->launches++;
    k_gauss<<<rb, 256, 0, h->stream>>>(g, E, h->slot[EMOO_RHO], h->red);
    EMOO_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)rb * 2);
    EMOO_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    double mx = 0.0, s2 = 0.0;
    for (int b = 0; b < rb; b++) {
        mx = std::max(mx, part[(size_t)b * 2]);
        s2 += part[(size_t)b * 2 + 1];
    }
    out2[0] = mx;
    out2[1] = sqrt(s2);
    return EMOO_OK;
}

}  // namespace emoo
