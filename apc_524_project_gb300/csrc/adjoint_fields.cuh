// adjoint_fields.cuh - transposed field kernels of the differentiated step,
// templated on the adjoint's scalar (double for the FP64 form, float for the
// mixed form). The forward maps are the same linear stencils in both forms
// (the Yee update of src/grid/oGrid.cpp:15-60, the periodic ghost copy of
// src/boundaries/b_fields/bc_f_periodic.cpp:47-52 over the physical
// transverse range, the J fold of src/grid/spookyGrid.cpp:21-26, LightBC's
// plane sets), so one transpose serves both.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {
namespace adf {

constexpr double FOURPI = 4.0 * PI_D;

template <class R>
struct FOutT {
    R *E[3], *B[3], *T[3];  // E, B role, B_tm1 role
};
template <class R>
struct JPtrsT {
    R *J[3];
};
template <class R>
struct Slots6T {
    R *p[6];
};
template <class R>
struct Slots9T {
    R *p[9];
};

__device__ __forceinline__ bool phys(const Geom &g, int i, int j, int k) {
    return i >= 1 && i <= g.n[0] && j >= 1 && j <= g.n[1] && k >= 1 && k <= g.n[2];
}

// The stencil coefficients dt / d (and -4 pi dt), computed once on the host:
// per-thread FP64 divisions would run on this GPU's narrow FP64 pipe.
template <class R>
struct YeeCoef {
    R cx, cy, cz, cj;
};

template <class R>
YeeCoef<R> yee_coef(const Geom &g, double dt) {
    return YeeCoef<R>{(R)(dt / g.d[0]), (R)(dt / g.d[1]), (R)(dt / g.d[2]), (R)(-FOURPI * dt)};
}

// Adjoint of the B update (B = T + dt curl E over the physical points),
// gather form over every grid point: LT += LB (physical), LE += dt C_E^T LB.
template <class R>
__global__ void k_yee_b_adj(Geom g, YeeCoef<R> yc, FOutT<R> A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= g.tot[2] || j >= g.tot[1] || i >= g.tot[0]) return;
    const int64_t p = gidx(g, i, j, k), sx = g.sx, sy = g.sy;
    const R cx = yc.cx, cy = yc.cy, cz = yc.cz;
    const bool here = phys(g, i, j, k);
    if (here)
        for (int c = 0; c < 3; c++) A.T[c][p] += A.B[c][p];
    const R *Bx = A.B[0], *By = A.B[1], *Bz = A.B[2];
    // Ey: Bx(o) += cz (Ey[o+1] - Ey[o]); Bz(o) -= cx (Ey[o+sx] - Ey[o])
    R ley = 0, lez = 0, lex = 0;
    if (phys(g, i, j, k - 1)) ley += cz * Bx[p - 1];
    if (here) ley += -cz * Bx[p] + cx * Bz[p];
    if (phys(g, i - 1, j, k)) ley += -cx * Bz[p - sx];
    // Ez: Bx(o) -= cy (Ez[o+sy] - Ez[o]); By(o) += cx (Ez[o+sx] - Ez[o])
    if (phys(g, i, j - 1, k)) lez += -cy * Bx[p - sy];
    if (here) lez += cy * Bx[p] - cx * By[p];
    if (phys(g, i - 1, j, k)) lez += cx * By[p - sx];
    // Ex: By(o) -= cz (Ex[o+1] - Ex[o]); Bz(o) += cy (Ex[o+sy] - Ex[o])
    if (phys(g, i, j, k - 1)) lex += -cz * By[p - 1];
    if (here) lex += cz * By[p] - cy * Bz[p];
    if (phys(g, i, j - 1, k)) lex += cy * Bz[p - sy];
    A.E[0][p] += lex;
    A.E[1][p] += ley;
    A.E[2][p] += lez;
}

// Adjoint of the E update (E -= dt (curl T + 4 pi J) over the physical
// points): LJ = -4 pi dt LE (physical, 0 elsewhere), LT += transposed curl;
// the B role was overwritten by the step, so its physical points' adjoint is
// cleared.
template <class R>
__global__ void k_yee_e_adj(Geom g, YeeCoef<R> yc, FOutT<R> A, JPtrsT<R> LJ) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= g.tot[2] || j >= g.tot[1] || i >= g.tot[0]) return;
    const int64_t p = gidx(g, i, j, k), sx = g.sx, sy = g.sy;
    const R cx = yc.cx, cy = yc.cy, cz = yc.cz, cj = yc.cj;
    const bool here = phys(g, i, j, k);
    const R *Ex = A.E[0], *Ey = A.E[1], *Ez = A.E[2];
    for (int c = 0; c < 3; c++) LJ.J[c][p] = here ? cj * A.E[c][p] : (R)0;
    R lty = 0, ltz = 0, ltx = 0;
    // Ty: ex(o) -= cz (Ty[o] - Ty[o-1]); ez(o) += cx (Ty[o] - Ty[o-sx])
    if (here) lty += -cz * Ex[p] + cx * Ez[p];
    if (phys(g, i, j, k + 1)) lty += cz * Ex[p + 1];
    if (phys(g, i + 1, j, k)) lty += -cx * Ez[p + sx];
    // Tz: ex(o) += cy (Tz[o] - Tz[o-sy]); ey(o) -= cx (Tz[o] - Tz[o-sx])
    if (here) ltz += cy * Ex[p] - cx * Ey[p];
    if (phys(g, i, j + 1, k)) ltz += -cy * Ex[p + sy];
    if (phys(g, i + 1, j, k)) ltz += cx * Ey[p + sx];
    // Tx: ey(o) += cz (Tx[o] - Tx[o-1]); ez(o) -= cy (Tx[o] - Tx[o-sy])
    if (here) ltx += cz * Ey[p] - cy * Ez[p];
    if (phys(g, i, j, k + 1)) ltx += -cz * Ey[p + 1];
    if (phys(g, i, j + 1, k)) ltx += cy * Ez[p + sy];
    A.T[0][p] += ltx;
    A.T[1][p] += lty;
    A.T[2][p] += ltz;
    if (here)
        for (int c = 0; c < 3; c++) A.B[c][p] = (R)0;
}

// Adjoint of the fold (F[plane 1] += F[plane n+1], transverse physical
// range, the two transverse J components): LF[n+1] += LF[1].
template <class R>
__global__ void k_fold_adj(Geom g, int d, R *f0, R *f1) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int r = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || r > g.n[o1]) return;
    int is[3], it[3];
    is[d] = g.n[d] + 1;
    it[d] = 1;
    is[o1] = it[o1] = r;
    is[o2] = it[o2] = q;
    const int64_t s = gidx(g, is[0], is[1], is[2]), t = gidx(g, it[0], it[1], it[2]);
    R *F = blockIdx.z == 0 ? f0 : f1;
    F[s] += F[t];
}

// Adjoint of one side of the ghost copy (ghost plane <- physical plane,
// transverse physical range): LF[src] += LF[dst], LF[dst] = 0.
template <class R>
__global__ void k_ghost_adj(Geom g, Slots6T<R> fl, int d, int side) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int r = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (q > g.n[o2] || r > g.n[o1]) return;
    const int nd = g.n[d];
    const int src = side == 0 ? nd : 1, dst = side == 0 ? 0 : nd + 1;
    int is[3], it[3];
    is[d] = src;
    it[d] = dst;
    is[o1] = it[o1] = r;
    is[o2] = it[o2] = q;
    R *F = fl.p[blockIdx.z];
    const int64_t ps = gidx(g, is[0], is[1], is[2]), pd = gidx(g, it[0], it[1], it[2]);
    F[ps] += F[pd];
    F[pd] = (R)0;
}

// ---- corrected policy ------------------------------------------------------
//
// Adjoint of the whole-range periodic operations along d, per transverse
// point of the (n+3)^2 plane, the forward steps reversed (so any n is exact):
// fold = 1 reverses f[n] += f[0], f[1] += f[n+1], f[2] += f[n+2];
// fold = 0 reverses f[0] = f[n], f[n+1] = f[1], f[n+2] = f[2].
// One field per blockIdx.z.
template <class R>
__global__ void k_periodic_full_adj(Geom g, Slots9T<R> fl, int d, int fold) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= g.tot[o2] || r >= g.tot[o1]) return;
    R *F = fl.p[blockIdx.z];
    const int n = g.n[d];
    int c[3];
    c[o1] = r;
    c[o2] = q;
    auto at = [&](int i) -> R & {
        c[d] = i;
        return F[gidx(g, c[0], c[1], c[2])];
    };
    if (fold) {
        at(n + 2) += at(2);
        at(n + 1) += at(1);
        at(0) += at(n);
    } else {
        at(2) += at(n + 2);
        at(n + 2) = (R)0;
        at(1) += at(n + 1);
        at(n + 1) = (R)0;
        at(n) += at(0);
        at(0) = (R)0;
    }
}

// Adjoint of the mirror fold at a reflecting wall (dst += s src, src = 0, s =
// -1 for the component normal to the wall): L[src] = s L[dst]. Same launch
// shape as the forward; blockIdx.z = component.
template <class R>
__global__ void k_mirror_fold_adj(Geom g, Slots9T<R> fl, int d, int right) {
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (q >= g.tot[o2] || r >= g.tot[o1]) return;
    const int a = blockIdx.z;
    R *F = fl.p[a];
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
    F[ks] = normal ? -F[kd] : F[kd];
}

// Clears three arrays at the physical points (the adjoint of values a step
// overwrites there).
template <class R>
__global__ void k_clear_phys(Geom g, Slots9T<R> fl) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int i = blockIdx.z + 1;
    if (k > g.n[2] || j > g.n[1]) return;
    const int64_t p = gidx(g, i, j, k);
    for (int c = 0; c < 3; c++) fl.p[c][p] = (R)0;
}

// Adjoint of a plane set v + vs t1[p] t2[q]: the plane's values depend only
// on the wave parameters, so the step needs sum(LF) and sum(LF t1 t2) over
// the plane; the host turns them into the parameter gradient. Block b of the
// PLANE_BLOCKS launched writes its partial pair to sums2[2 b], sums2[2 b + 1]
// (FP64, fixed order within the block; the host adds the blocks in order).
// The plane's adjoint is cleared.
constexpr int PLANE_BLOCKS = 64;

template <class R>
__global__ void k_plane_adj(Geom g, R *F, int d, int idx, const double *t1, const double *t2, double *sums2) {
    __shared__ double s_u[32], s_s[32];
    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    double su = 0.0, ss = 0.0;
    const int64_t m = (int64_t)g.tot[o1] * g.tot[o2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        int c[3];
        c[d] = idx;
        c[o1] = (int)(t / g.tot[o2]);
        c[o2] = (int)(t % g.tot[o2]);
        const int64_t p = gidx(g, c[0], c[1], c[2]);
        const double l = (double)F[p];
        su += l;
        if (t1) ss += l * t1[c[o1]] * t2[c[o2]];
        F[p] = (R)0;
    }
    for (int off = 16; off > 0; off >>= 1) {
        su += __shfl_down_sync(0xffffffffu, su, off);
        ss += __shfl_down_sync(0xffffffffu, ss, off);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_u[w] = su;
        s_s[w] = ss;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            a += s_u[i];
            b += s_s[i];
        }
        sums2[2 * blockIdx.x] = a;
        sums2[2 * blockIdx.x + 1] = b;
    }
}

}  // namespace adf
}  // namespace emoo
