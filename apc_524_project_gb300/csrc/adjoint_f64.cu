// adjoint_f64.cu - differentiation of the FP64 time loop (no reference
// counterpart): a tangent-linear run and an adjoint run with checkpoints.
//
// The differentiated step is the loop's step without sorting and without the
// charge density: gather + push + particle boundaries + current deposit (one
// particle kernel), the periodic J fold, the Yee update and executeBC(-1)
// (periodic ghost copies, LightBC planes). Its parameters are the initial
// particle velocities, the amplitude and phase of every injected wave and the
// coefficients of sine-series envelopes; the objective is the field energy
// 0.5 V sum(E^2 + B^2) over the grid points of an x slab, or the kinetic
// energy of the particles in an x range, at the last step.
//
//  * Tangent: the particle kernel runs in dual numbers (ad_math.cuh) next to
//    the primal one; the field part is linear, so the tangent fields go
//    through the primal field kernels themselves (with the slot table pointed
//    at the tangent arrays) and the planes take the derivative of their
//    values.
//  * Adjoint: every kernel has a transposed twin here. The deposit's adjoint
//    is a gather of the J adjoint at the particle's 12 points, the gather's
//    adjoint a scatter (atomics) of the field adjoint with the same weights,
//    the Yee and ghost/fold adjoints are the transposed stencils and copies,
//    a plane's adjoint reduces the field adjoint over the plane (plain and
//    weighted by the transverse spot) and clears the plane; the host forms
//    the wave-parameter gradient from those sums. State is checkpointed
//    every `checkpoint_every` steps; each segment is recomputed forward,
//    storing the state before each of its steps, then reversed.
//
// Compiled with --fmad=false like the FP64 kernels, so the dual numbers'
// primal values and the adjoint's recomputed forward are bit-identical to the
// primal step, and every cell and boundary decision agrees with it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ad_math.cuh"
#include "adjoint_fields.cuh"
#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {

double *role_b(emoo_handle *h, int c);
double *role_t(emoo_handle *h, int c);

namespace {

using ad::CellGeo;
using ad::Dual;
using ad::mk;

constexpr int NSLOT = EMOO_BZ_TM1 + 1;  // E, B, J, rho, B_tm1: the slots a step touches

struct PArr {
    double *p[7];  // x, y, z, vx, vy, vz, gamma
};
struct CPArr {
    const double *p[7];
};
struct FPtrs {
    const double *E[3], *B[3], *T[3];  // E, B role, B_tm1 role
};
using FOut = adf::FOutT<double>;
using JPtrs = adf::JPtrsT<double>;
using Slots6 = adf::Slots6T<double>;
using adf::k_fold_adj;
using adf::k_ghost_adj;
using adf::k_plane_adj;
using adf::k_yee_b_adj;
using adf::k_yee_e_adj;

// the kernels' own geometry, reciprocals and power-of-two flags (so the
// recomputed forward divides exactly as the primal step does)
__device__ __forceinline__ CellGeo cell_geo(const Geom &g) {
    CellGeo c;
    for (int a = 0; a < 3; a++) {
        c.d[a] = g.d[a];
        c.area[a] = g.area[a];
        c.id[a] = g.id[a];
        c.iarea[a] = g.iarea[a];
        c.p2[a] = g.p2[a];
        c.p2area[a] = g.area_p2[a];
    }
    c.vol = g.vol;
    c.ivol = g.ivol;
    c.p2vol = g.vol_p2;
    return c;
}

// grid point of J contribution q (< 12) of cell o (Grid::addJ, the Jx quirk
// at q = 3, src/grid/oGrid.cpp:98-111)
__device__ __forceinline__ int64_t jpoint(const Geom &g, int64_t o, int q) {
    const int64_t sx = g.sx, sy = g.sy;
    switch (q) {
        case 0: return o;
        case 1: return o + sy;
        case 2: return o + sy + 1;
        case 3: return o + sy;
        case 4: return o;
        case 5: return o + 1;
        case 6: return o + sx + 1;
        case 7: return o + sx;
        case 8: return o;
        case 9: return o + sx;
        case 10: return o + sx + sy;
        default: return o + sy;
    }
}

// the 18 gather inputs of cell o: 12 E edge points, 6 B face points
__device__ __forceinline__ void gather_points(const Geom &g, int64_t o, int64_t pt[18]) {
    const int64_t sx = g.sx, sy = g.sy;
    const int64_t e[12] = {o, o + sy, o + sy + 1, o + 1, o, o + 1, o + sx + 1, o + sx, o, o + sx, o + sx + sy, o + sy};
    for (int k = 0; k < 12; k++) pt[k] = e[k];
    pt[12] = o;
    pt[13] = o + sx;
    pt[14] = o;
    pt[15] = o + sy;
    pt[16] = o;
    pt[17] = o + 1;
}

// executeBC of the particles (apply_bc in particles_f64.cu) on any scalar;
// decisions on the primal values. Returns -1 when the particle is removed,
// else a 3-bit mask of the axes reflected an odd number of times.
template <class T>
__device__ __forceinline__ int bc_t(const BCTab &bc, T p[3], T v[3]) {
    int flips = 0;
    for (int s = 0; s < 6; s++) {
        const int d = s >> 1;
        const bool right = s & 1;
        const double xmin = bc.xmin[d], xmax = bc.xmax[d];
        const double pv = ad::val(p[d]);
        const bool hit = right ? (pv > xmax) : (pv < xmin);
        if (!hit) continue;
        const int kind = bc.pbc[s];
        if (kind == PBC_PERIODIC) {
            if (right) p[d] = p[d] - (xmax - xmin);
            else p[d] = p[d] + (xmax - xmin);
        } else if (kind == PBC_REFLECTING) {
            p[d] = right ? 2.0 * xmax - p[d] : 2.0 * xmin - p[d];
            v[d] = -v[d];
            flips ^= 1 << d;
        } else {
            return -1;
        }
    }
    return flips;
}

// ---- charge-conserving current (corrected policy) ----------------------------

__device__ __forceinline__ ad::VbGeo vb_geo(const Geom &g) {
    ad::VbGeo v;
    for (int a = 0; a < 3; a++) {
        v.x0[a] = g.x0[a];
        v.id[a] = g.id[a];
        v.d[a] = g.d[a];
    }
    return v;
}

// Grid point of weight e of axis a of a current piece in cell c (the indexing
// of vb_deposit in particles_f64.cu), or -1 where that deposit skips the
// piece (a cell outside -1..n along some axis).
__device__ __forceinline__ int64_t vb_point(const Geom &g, const int c[3], int a, int e) {
    for (int b = 0; b < 3; b++)
        if (c[b] < -1 || c[b] + 2 >= g.tot[b]) return -1;
    int ii[3] = {c[0] + 1, c[1] + 1, c[2] + 1};
    ii[(a + 1) % 3] += e & 1;
    ii[(a + 2) % 3] += e >> 1;
    return gidx(g, ii[0], ii[1], ii[2]);
}

// Tangent of vb_deposit: the derivative of every weight added to dJ.
__device__ void vb_tlm(const Geom &g, const JPtrs &dJ, const Dual p0[3], const Dual p1[3], double coef) {
    ad::VbPiece<Dual> pc[4];
    const int n = ad::vb_eval(vb_geo(g), p0, p1, coef, pc);
    for (int k = 0; k < n; k++)
        for (int a = 0; a < 3; a++)
            for (int e = 0; e < 4; e++) {
                const int64_t pt = vb_point(g, pc[k].cell, a, e);
                if (pt >= 0) atomicAdd(dJ.J[a] + pt, pc[k].W[4 * a + e].d);
            }
}

// Adjoint of vb_deposit: adds the derivatives of sum(LJ W) to lp0, lp1.
__device__ void vb_adj(const Geom &g, const JPtrs &LJ, const double p0[3], const double p1[3], double coef,
                       double lp0[3], double lp1[3]) {
    auto lw = [&](int, const int *c, int a, int e) -> double {
        const int64_t pt = vb_point(g, c, a, e);
        return pt >= 0 ? LJ.J[a][pt] : 0.0;
    };
    ad::vb_rev(vb_geo(g), p0, p1, coef, lw, lp0, lp1);
}

// The exit extension past absorbing walls (absorbed_exit in particles_f64.cu):
// from the end of the move, along each axis whose absorbing side was crossed,
// a straight piece to the fixed vertex plane beyond the wall.
__device__ int exit_path(const Geom &g, const BCTab &bc, const double p1[3], double A[4][3], int dk[3]) {
    int K = 0;
    for (int c = 0; c < 3; c++) A[0][c] = p1[c];
    for (int d = 0; d < 3; d++) {
        double b[3] = {A[K][0], A[K][1], A[K][2]};
        if (bc.pbc[2 * d] == PBC_ABSORBING && A[K][d] < bc.xmin[d]) b[d] = bc.xmin[d] - g.d[d];
        else if (bc.pbc[2 * d + 1] == PBC_ABSORBING && A[K][d] > bc.xmax[d]) b[d] = bc.xmax[d] + g.d[d];
        else continue;
        dk[K] = d;
        for (int c = 0; c < 3; c++) A[K + 1][c] = b[c];
        K++;
    }
    return K;
}

__device__ void exit_tlm(const Geom &g, const BCTab &bc, const JPtrs &dJ, const Dual p1[3], double coef) {
    Dual a[3] = {p1[0], p1[1], p1[2]};
    for (int d = 0; d < 3; d++) {
        Dual b[3] = {a[0], a[1], a[2]};
        if (bc.pbc[2 * d] == PBC_ABSORBING && a[d].v < bc.xmin[d]) b[d] = mk(bc.xmin[d] - g.d[d]);
        else if (bc.pbc[2 * d + 1] == PBC_ABSORBING && a[d].v > bc.xmax[d]) b[d] = mk(bc.xmax[d] + g.d[d]);
        else continue;
        vb_tlm(g, dJ, a, b, coef);
        a[d] = b[d];
    }
}

// Adjoint of the exit extension: the pieces in reverse; the coordinate a piece
// sets to the wall's plane is a constant, its other ones pass through.
__device__ void exit_adj(const Geom &g, const BCTab &bc, const JPtrs &LJ, const double p1[3], double coef,
                         double lp1[3]) {
    double A[4][3];
    int dk[3];
    const int K = exit_path(g, bc, p1, A, dk);
    double lA[3] = {0.0, 0.0, 0.0};
    for (int k = K - 1; k >= 0; k--) {
        double la[3] = {0.0, 0.0, 0.0}, lb[3] = {lA[0], lA[1], lA[2]};
        vb_adj(g, LJ, A[k], A[k + 1], coef, la, lb);
        lb[dk[k]] = 0.0;
        for (int c = 0; c < 3; c++) lA[c] = la[c] + lb[c];
    }
    for (int c = 0; c < 3; c++) lp1[c] += lA[c];
}

// ---- tangent particle kernel ---------------------------------------------
//
// Reads the primal state before the step (P, F) and the tangents (dP, dF),
// writes the tangents after the step and adds the tangent current to dJ.
// CORR: the corrected policy (gather at the cell's own vertex, the
// charge-conserving current of the move before the boundaries).
template <bool REL, bool CORR>
__global__ void k_tlm_particles(Geom g, SpeciesTab st, BCTab bc, CPArr P, FPtrs F, FPtrs dF, PArr dP, int64_t np,
                                double dt, JPtrs dJ) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double x = P.p[0][p];
    if (x != x) return;  // removed
    const int s = species_of(st, p);
    int ix, iy, iz;
    cell_of(g, x, P.p[1][p], P.p[2][p], ix, iy, iz);
    if (!cell_ok(g, ix, iy, iz)) return;
    const int64_t o = gidx(g, ix, iy, iz);
    int64_t pt[18];
    gather_points(g, o, pt);
    Dual v18[18];
    for (int k = 0; k < 12; k++) {
        const int c = k >> 2;
        v18[k] = mk(F.E[c][pt[k]], dF.E[c][pt[k]]);
    }
    for (int k = 12; k < 18; k++) {
        const int c = (k - 12) >> 1;
        v18[k] = mk((F.T[c][pt[k]] + F.B[c][pt[k]]) / 2, (dF.T[c][pt[k]] + dF.B[c][pt[k]]) / 2);
    }
    const CellGeo cg = cell_geo(g);
    Dual pos[3], vel[3], ds[3], f[6];
    for (int a = 0; a < 3; a++) {
        pos[a] = mk(P.p[a][p], dP.p[a][p]);
        vel[a] = mk(P.p[3 + a][p], dP.p[3 + a][p]);
    }
    const Dual p0[3] = {pos[0], pos[1], pos[2]};
    const int ic[3] = {ix, iy, iz};
    for (int a = 0; a < 3; a++) ds[a] = pos[a] - (g.x0[a] + g.d[a] * (ic[a] - g.vshift));
    ad::gather_eval(cg, v18, ds, f);
    Dual gam = mk(REL ? P.p[6][p] : 1.0, REL ? dP.p[6][p] : 0.0);
    if (REL) ad::vay_eval(st.qp[s], f, dt, pos, vel, gam);
    else ad::boris_eval(st.qp[s], f, dt, pos, vel);
    if (CORR && st.deposit[s] && dt > 0.0) {
        const double coef = st.uq[s] / g.vol / dt;
        vb_tlm(g, dJ, p0, pos, coef);
        exit_tlm(g, bc, dJ, pos, coef);
    }
    if (bc_t(bc, pos, vel) < 0) {
        for (int a = 0; a < 7; a++) dP.p[a][p] = 0.0;
        return;
    }
    if (!CORR && st.deposit[s]) {
        cell_of(g, pos[0].v, pos[1].v, pos[2].v, ix, iy, iz);
        if (cell_ok(g, ix, iy, iz)) {
            const int64_t o2 = gidx(g, ix, iy, iz);
            const int jc[3] = {ix, iy, iz};
            Dual r[3], c12[12];
            for (int a = 0; a < 3; a++) r[a] = pos[a] - (g.x0[a] + g.d[a] * jc[a]);
            ad::jterms_eval(cg, st.uq[s], r, vel, c12);
            for (int q = 0; q < 12; q++) atomicAdd(dJ.J[q >> 2] + jpoint(g, o2, q), c12[q].d);
        }
    }
    for (int a = 0; a < 3; a++) {
        dP.p[a][p] = pos[a].d;
        dP.p[3 + a][p] = vel[a].d;
    }
    if (REL) dP.p[6][p] = gam.d;
}

// ---- adjoint particle kernel ---------------------------------------------
//
// P, F: the primal state before the step (from the tape). L: the particle
// adjoints, after the step on entry, before it on exit. LJ: the adjoint of
// the deposited current. LF: field adjoints that receive the gather's
// adjoint (atomics). CORR as in k_tlm_particles.
template <bool REL, bool CORR>
__global__ void k_adj_particles(Geom g, SpeciesTab st, BCTab bc, CPArr P, FPtrs F, PArr L, int64_t np, double dt,
                                JPtrs LJ, FOut LF) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double x = P.p[0][p];
    if (x != x) return;
    const int s = species_of(st, p);
    int ix, iy, iz;
    cell_of(g, x, P.p[1][p], P.p[2][p], ix, iy, iz);
    if (!cell_ok(g, ix, iy, iz)) return;
    const int64_t o = gidx(g, ix, iy, iz);
    int64_t pt[18];
    gather_points(g, o, pt);
    double v18[18];
    for (int k = 0; k < 12; k++) v18[k] = F.E[k >> 2][pt[k]];
    for (int k = 12; k < 18; k++) {
        const int c = (k - 12) >> 1;
        v18[k] = (F.T[c][pt[k]] + F.B[c][pt[k]]) / 2;
    }
    const CellGeo cg = cell_geo(g);
    const int ic[3] = {ix, iy, iz};
    double pos[3], vel[3], ds[3], f[6], p0[3];
    for (int a = 0; a < 3; a++) {
        pos[a] = p0[a] = P.p[a][p];
        vel[a] = P.p[3 + a][p];
        ds[a] = pos[a] - (g.x0[a] + g.d[a] * (ic[a] - g.vshift));
    }
    ad::gather_eval(cg, v18, ds, f);
    const double v_in[3] = {vel[0], vel[1], vel[2]};
    const double g_in = REL ? P.p[6][p] : 1.0;
    double gam = g_in;
    ad::VayTape vt;
    if (REL) ad::vay_fwd(st.qp[s], f, dt, pos, vel, gam, vt);
    else ad::boris_eval(st.qp[s], f, dt, pos, vel);
    const double p1[3] = {pos[0], pos[1], pos[2]};  // the end of the move, before the boundaries
    const int flips = bc_t(bc, pos, vel);
    double lx[3], lv[3], lg = REL ? L.p[6][p] : 0.0;
    for (int a = 0; a < 3; a++) {
        lx[a] = L.p[a][p];
        lv[a] = L.p[3 + a][p];
    }
    if (flips < 0) {  // removed: nothing after the step depends on it
        for (int a = 0; a < 3; a++) lx[a] = lv[a] = 0.0;
        lg = 0.0;
    } else {
        if (!CORR && st.deposit[s]) {
            int jx, jy, jz;
            cell_of(g, pos[0], pos[1], pos[2], jx, jy, jz);
            if (cell_ok(g, jx, jy, jz)) {
                const int64_t o2 = gidx(g, jx, jy, jz);
                const int jc[3] = {jx, jy, jz};
                double r[3], l12[12];
                for (int a = 0; a < 3; a++) r[a] = pos[a] - (g.x0[a] + g.d[a] * jc[a]);
                for (int q = 0; q < 12; q++) l12[q] = LJ.J[q >> 2][jpoint(g, o2, q)];
                ad::jterms_rev(cg, st.uq[s], r, vel, l12, lx, lv);
            }
        }
        for (int a = 0; a < 3; a++)
            if ((flips >> a) & 1) {
                lx[a] = -lx[a];
                lv[a] = -lv[a];
            }
    }
    double lp0[3] = {0.0, 0.0, 0.0};
    if (CORR && st.deposit[s] && dt > 0.0) {  // the current of the move, also for a removed particle
        const double coef = st.uq[s] / g.vol / dt;
        double lp1[3] = {0.0, 0.0, 0.0};
        vb_adj(g, LJ, p0, p1, coef, lp0, lp1);
        exit_adj(g, bc, LJ, p1, coef, lp1);
        for (int a = 0; a < 3; a++) lx[a] += lp1[a];
    }
    double lf[6] = {0, 0, 0, 0, 0, 0};
    if (REL) ad::vay_rev_tape(vt, st.qp[s], f, dt, v_in, g_in, lx, lv, lg, lf);
    else ad::boris_rev(st.qp[s], f, dt, v_in, lx, lv, lf);
    double l18[18] = {0}, lds[3] = {0, 0, 0};
    ad::gather_rev(cg, v18, ds, lf, l18, lds);
    for (int k = 0; k < 12; k++)
        if (l18[k] != 0.0) atomicAdd(LF.E[k >> 2] + pt[k], l18[k]);
    for (int k = 12; k < 18; k++) {
        const int c = (k - 12) >> 1;
        if (l18[k] != 0.0) {
            atomicAdd(LF.B[c] + pt[k], 0.5 * l18[k]);
            atomicAdd(LF.T[c] + pt[k], 0.5 * l18[k]);
        }
    }
    for (int a = 0; a < 3; a++) {
        L.p[a][p] = lx[a] + lds[a] + lp0[a];
        L.p[3 + a][p] = lv[a];
    }
    if (REL) L.p[6][p] = lg;
}

// ---- objective -----------------------------------------------------------

struct Slab {
    int lo, hi;  // grid point x index range [lo, hi)
};

// 0.5 V sum(E^2 + B^2) over the slab (and, with dE/dB, V sum(E dE + B dB)).
__global__ void k_objective(Geom g, Slab sl, FPtrs F, FPtrs dF, int tangent, double *out2) {
    const int64_t ny = g.n[1], nz = g.n[2];
    const int64_t m = (int64_t)(sl.hi - sl.lo) * ny * nz;
    double a = 0.0, b = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % nz) + 1;
        const int j = (int)((t / nz) % ny) + 1;
        const int i = (int)(t / (nz * ny)) + sl.lo;
        const int64_t p = gidx(g, i, j, k);
        for (int c = 0; c < 3; c++) {
            a += F.E[c][p] * F.E[c][p] + F.B[c][p] * F.B[c][p];
            if (tangent) b += F.E[c][p] * dF.E[c][p] + F.B[c][p] * dF.B[c][p];
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out2, 0.5 * g.vol * a);
        atomicAdd(out2 + 1, g.vol * b);
    }
}

// Seeds the field adjoints with d objective / d(E, B role) = V (E, B) on the slab.
__global__ void k_objective_seed(Geom g, Slab sl, FPtrs F, FOut A) {
    const int64_t ny = g.n[1], nz = g.n[2];
    const int64_t m = (int64_t)(sl.hi - sl.lo) * ny * nz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % nz) + 1;
        const int j = (int)((t / nz) % ny) + 1;
        const int i = (int)(t / (nz * ny)) + sl.lo;
        const int64_t p = gidx(g, i, j, k);
        for (int c = 0; c < 3; c++) {
            A.E[c][p] += g.vol * F.E[c][p];
            A.B[c][p] += g.vol * F.B[c][p];
        }
    }
}

// Selection of the kinetic objective: particles of `species` (-1: all),
// alive, with x in [xlo, xhi).
struct KinSel {
    int species;
    double xlo, xhi;
};

__device__ __forceinline__ bool kin_selected(const SpeciesTab &st, const KinSel &ks, int64_t p, double x, int &s) {
    if (x != x) return false;  // removed
    s = species_of(st, p);
    return (ks.species < 0 || s == ks.species) && x >= ks.xlo && x < ks.xhi;
}

// sum m (gamma - 1) (REL) or 0.5 m v^2 over the selected particles; with
// tangent, also its derivative along dP: m dgamma, or m v . dv.
template <bool REL>
__global__ void k_objective_kin(SpeciesTab st, CPArr P, CPArr dP, int64_t np, KinSel ks, int tangent, double *out2) {
    double a = 0.0, b = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        int s;
        if (!kin_selected(st, ks, p, P.p[0][p], s)) continue;
        const double m = st.m[s];
        if (REL) {
            a += m * (P.p[6][p] - 1.0);
            if (tangent) b += m * dP.p[6][p];
        } else {
            const double vx = P.p[3][p], vy = P.p[4][p], vz = P.p[5][p];
            a += 0.5 * m * (vx * vx + vy * vy + vz * vz);
            if (tangent) b += m * (vx * dP.p[3][p] + vy * dP.p[4][p] + vz * dP.p[5][p]);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out2, a);
        atomicAdd(out2 + 1, b);
    }
}

// Seeds the particle adjoints with d objective / d(gamma) = m (REL) or
// d objective / d v = m v on the selected particles.
template <bool REL>
__global__ void k_objective_kin_seed(SpeciesTab st, CPArr P, PArr L, int64_t np, KinSel ks) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        int s;
        if (!kin_selected(st, ks, p, P.p[0][p], s)) continue;
        const double m = st.m[s];
        if (REL) {
            L.p[6][p] += m;
        } else {
            for (int c = 0; c < 3; c++) L.p[3 + c][p] += m * P.p[3 + c][p];
        }
    }
}

// grid of the grid-stride kernels (objectives, seeds)
int pblocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 64)); }
// grid of the one-thread-per-particle kernels: every particle gets a thread
int pblocks_all(int64_t n) { return (int)std::max<int64_t>(1, (n + 255) / 256); }

// ---- host side -----------------------------------------------------------

// The state the differentiated step reads: particles and the E / B slots.
struct Snapshot {
    double *buf = nullptr;
    int bswap = 0;
    double t = 0.0;
    int64_t step = 0;
};

struct AdRun {
    emoo_handle *h;
    int64_t np, npts;
    bool rel;
    std::vector<double *> owned;

    double *alloc(size_t n) {
        double *p = nullptr;
        if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
        owned.push_back(p);
        return p;
    }
    ~AdRun() {
        for (double *p : owned) cudaFree(p);
    }
    size_t snap_words() const { return 7 * (size_t)np + 9 * (size_t)npts; }
    double **particle_ptrs(double **out7) {
        out7[0] = h->x; out7[1] = h->y; out7[2] = h->z;
        out7[3] = h->vx; out7[4] = h->vy; out7[5] = h->vz; out7[6] = h->gam;
        return out7;
    }
    static int slot_of_snapshot(int k) {  // snapshot field k -> slot id
        static const int ids[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ, EMOO_BX_TM1, EMOO_BY_TM1,
                                   EMOO_BZ_TM1};
        return ids[k];
    }
    int save(Snapshot &s) {
        if (!s.buf) s.buf = alloc(snap_words());
        if (!s.buf) return EMOO_ERR_OOM;
        double *P[7];
        particle_ptrs(P);
        for (int a = 0; a < 7; a++) {
            if (!P[a]) continue;
            EMOO_CUDA(cudaMemcpyAsync(s.buf + a * np, P[a], sizeof(double) * np, cudaMemcpyDeviceToDevice, h->stream));
        }
        for (int k = 0; k < 9; k++)
            EMOO_CUDA(cudaMemcpyAsync(s.buf + 7 * np + k * npts, h->slot[slot_of_snapshot(k)], sizeof(double) * npts,
                                      cudaMemcpyDeviceToDevice, h->stream));
        s.bswap = h->bswap;
        s.t = h->t;
        s.step = h->step_index;
        return EMOO_OK;
    }
    int restore(const Snapshot &s) {
        double *P[7];
        particle_ptrs(P);
        for (int a = 0; a < 7; a++) {
            if (!P[a]) continue;
            EMOO_CUDA(cudaMemcpyAsync(P[a], s.buf + a * np, sizeof(double) * np, cudaMemcpyDeviceToDevice, h->stream));
        }
        for (int k = 0; k < 9; k++)
            EMOO_CUDA(cudaMemcpyAsync(h->slot[slot_of_snapshot(k)], s.buf + 7 * np + k * npts, sizeof(double) * npts,
                                      cudaMemcpyDeviceToDevice, h->stream));
        h->bswap = s.bswap;
        h->t = s.t;
        h->step_index = s.step;
        return EMOO_OK;
    }
    CPArr snap_particles(const Snapshot &s) const {
        CPArr P;
        for (int a = 0; a < 7; a++) P.p[a] = s.buf + a * np;
        return P;
    }
    FPtrs snap_fields(const Snapshot &s) const {
        FPtrs F;
        const double *f = s.buf + 7 * np;
        for (int c = 0; c < 3; c++) {
            F.E[c] = f + c * npts;
            const double *b = f + (3 + c) * npts, *t = f + (6 + c) * npts;
            F.B[c] = s.bswap ? t : b;  // the roles at the snapshot's bswap
            F.T[c] = s.bswap ? b : t;
        }
        return F;
    }
};

// Points the handle's slot table at other arrays for the duration of a scope
// (the field kernels act on the slots; the tangent fields reuse them).
struct SlotSwap {
    emoo_handle *h;
    double *saved[EMOO_NFIELDS];
    int bswap;
    SlotSwap(emoo_handle *hh, double *const *alt) : h(hh), bswap(hh->bswap) {
        for (int k = 0; k < EMOO_NFIELDS; k++) {
            saved[k] = h->slot[k];
            if (k < NSLOT) h->slot[k] = alt[k];
        }
    }
    ~SlotSwap() {
        for (int k = 0; k < EMOO_NFIELDS; k++) h->slot[k] = saved[k];
        h->bswap = bswap;
    }
};

FPtrs field_ptrs(emoo_handle *h, double *const *slots, int bswap) {
    FPtrs F;
    for (int c = 0; c < 3; c++) {
        F.E[c] = slots[EMOO_EX + c];
        F.B[c] = bswap ? slots[EMOO_BX_TM1 + c] : slots[EMOO_BX + c];
        F.T[c] = bswap ? slots[EMOO_BX + c] : slots[EMOO_BX_TM1 + c];
    }
    (void)h;
    return F;
}
FOut field_out(double *const *slots, int bswap) {
    FOut F;
    for (int c = 0; c < 3; c++) {
        F.E[c] = slots[EMOO_EX + c];
        F.B[c] = bswap ? slots[EMOO_BX_TM1 + c] : slots[EMOO_BX + c];
        F.T[c] = bswap ? slots[EMOO_BX + c] : slots[EMOO_BX_TM1 + c];
    }
    return F;
}

// One step of the loop without sort and charge density (the primal step the
// tangent and adjoint runs differentiate).
int primal_step(emoo_handle *h) {
    EMOO_TRY(fused_step_f64(h, h->dtp, 0));
    EMOO_TRY(ad_execute_bc(h, EMOO_SEND_JRHO));
    EMOO_TRY(yee_f64(h, h->dtp));
    EMOO_TRY(ad_execute_bc(h, EMOO_SEND_EB));
    h->t += h->dtp;
    h->step_index++;
    return EMOO_OK;
}

dim3 grid_all(const Geom &g, dim3 blk) {
    return dim3((g.tot[2] + blk.x - 1) / blk.x, (g.tot[1] + blk.y - 1) / blk.y, g.tot[0]);
}

struct ObjSpec {
    int kind;  // EMOO_AD_OBJ_FIELD or EMOO_AD_OBJ_KINETIC
    Slab sl;
    KinSel ks;
};

CPArr particle_arrays(emoo_handle *h) { return CPArr{{h->x, h->y, h->z, h->vx, h->vy, h->vz, h->gam}}; }

// The objective (out2[0]) and, with tangent states dslots / dP, its
// derivative along them (out2[1]).
int objective(emoo_handle *h, const ObjSpec &os, double *const *dslots, double *const *dP, double *dev2,
              double out2[2]) {
    EMOO_CUDA(cudaMemsetAsync(dev2, 0, 2 * sizeof(double), h->stream));
    h->launches++;
    if (os.kind == EMOO_AD_OBJ_FIELD) {
        const Slab &sl = os.sl;
        FPtrs F = field_ptrs(h, h->slot, h->bswap);
        FPtrs dF = dslots ? field_ptrs(h, dslots, h->bswap) : F;
        k_objective<<<pblocks((int64_t)(sl.hi - sl.lo) * h->g.n[1] * h->g.n[2]), 256, 0, h->stream>>>(
            h->g, sl, F, dF, dslots ? 1 : 0, dev2);
    } else {
        SpeciesTab st;
        species_tab(h, h->dtp, st);
        const CPArr P = particle_arrays(h);
        const CPArr D = dP ? CPArr{{dP[0], dP[1], dP[2], dP[3], dP[4], dP[5], dP[6]}} : P;
        if (h->info.relativity)
            k_objective_kin<true><<<pblocks(h->np), 256, 0, h->stream>>>(st, P, D, h->np, os.ks, dP ? 1 : 0, dev2);
        else
            k_objective_kin<false><<<pblocks(h->np), 256, 0, h->stream>>>(st, P, D, h->np, os.ks, dP ? 1 : 0, dev2);
    }
    EMOO_CUDA(cudaGetLastError());
    EMOO_CUDA(cudaMemcpyAsync(out2, dev2, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

}  // namespace

// The tangent planes of a list of plane ops: each value's derivative along
// dtheta, written into the tangent slots.
static int tangent_planes(emoo_handle *h, const std::vector<AdBcOp> &ops, double *const *dslot,
                          const double *dtheta) {
    for (const AdBcOp &op : ops) {
        if (op.kind != 1) continue;
        double v = 0.0, vs = 0.0;
        if (dtheta) {
            for (size_t k = 0; k < op.ku.size(); k++) v += op.cu[k] * dtheta[op.ku[k]];
            for (size_t k = 0; k < op.ks.size(); k++) vs += op.cs[k] * dtheta[op.ks[k]];
        }
        PlaneSet ps{dslot[op.slot], op.dim, op.idx, v, vs, op.t1, op.t2, nullptr, nullptr};
        EMOO_TRY(plane_set_f64(h, &ps, 1));
    }
    return EMOO_OK;
}

static bool corrected(const emoo_handle *h) { return h->policy == EMOO_POLICY_CORRECTED; }

template <bool REL>
static void launch_tlm(emoo_handle *h, bool corr, const SpeciesTab &st, CPArr P, FPtrs F, FPtrs dF, PArr D,
                       int64_t np, JPtrs dJ) {
    const int nb = pblocks_all(np);
    if (corr)
        k_tlm_particles<REL, true><<<nb, 256, 0, h->stream>>>(h->g, st, h->bc, P, F, dF, D, np, h->dtp, dJ);
    else
        k_tlm_particles<REL, false><<<nb, 256, 0, h->stream>>>(h->g, st, h->bc, P, F, dF, D, np, h->dtp, dJ);
}

// tangent step: dP, dslot advance with the primal step
static int tlm_step(emoo_handle *h, AdRun &R, double **dP, double *const *dslot, const double *dtheta) {
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    const bool corr = corrected(h);
    for (int c = 0; c < 3; c++)
        EMOO_CUDA(cudaMemsetAsync(dslot[EMOO_JX + c], 0, sizeof(double) * R.npts, h->stream));
    CPArr P{{h->x, h->y, h->z, h->vx, h->vy, h->vz, h->gam}};
    FPtrs F = field_ptrs(h, h->slot, h->bswap), dF = field_ptrs(h, dslot, h->bswap);
    PArr D{{dP[0], dP[1], dP[2], dP[3], dP[4], dP[5], dP[6]}};
    JPtrs dJ{{dslot[EMOO_JX], dslot[EMOO_JY], dslot[EMOO_JZ]}};
    h->launches++;
    if (R.rel) launch_tlm<true>(h, corr, st, P, F, dF, D, R.np, dJ);
    else launch_tlm<false>(h, corr, st, P, F, dF, D, R.np, dJ);
    EMOO_CUDA(cudaGetLastError());
    // primal particle step, then the linear field part on both
    EMOO_TRY(fused_step_f64(h, h->dtp, 0));
    EMOO_TRY(ad_execute_bc(h, EMOO_SEND_JRHO));
    if (corr) {
        // the tangent fields through the same halves, periodic images and
        // plane sets (the planes' derivative values) as the primal ones
        {
            SlotSwap sw(h, dslot);
            EMOO_TRY(ad_execute_bc(h, EMOO_SEND_JRHO));
        }
        EMOO_TRY(yee_f64(h, h->dtp));
        std::vector<AdBcOp> ops;
        EMOO_TRY(ad_bc_ops(h, ops));
        EMOO_TRY(ad_execute_bc(h, EMOO_SEND_EB));
        SlotSwap sw(h, dslot);
        static const int ids_e[3] = {EMOO_EX, EMOO_EY, EMOO_EZ};
        static const int ids9[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ,
                                    EMOO_BX_TM1, EMOO_BY_TM1, EMOO_BZ_TM1};
        EMOO_TRY(yee_half_f64(h, h->dtp, 0));
        EMOO_TRY(periodic_copies_f64(h, ids_e, 3));
        EMOO_TRY(tangent_planes(h, ops, dslot, dtheta));
        EMOO_TRY(yee_half_f64(h, h->dtp, 1));
        EMOO_TRY(periodic_copies_f64(h, ids9, 9));
        EMOO_TRY(tangent_planes(h, ops, dslot, dtheta));
    } else {
        {
            SlotSwap sw(h, dslot);
            EMOO_TRY(ad_execute_bc(h, EMOO_SEND_JRHO));
            EMOO_TRY(yee_f64(h, h->dtp));
        }
        EMOO_TRY(yee_f64(h, h->dtp));
        std::vector<AdBcOp> ops;
        EMOO_TRY(ad_bc_ops(h, ops));
        EMOO_TRY(ad_execute_bc(h, EMOO_SEND_EB));
        SlotSwap sw(h, dslot);
        static const int ids_eb[6] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ};
        for (const AdBcOp &op : ops) {
            if (op.kind == 0) {
                EMOO_TRY(ghost_fill_f64(h, ids_eb, 6, op.mask));
            } else {
                const std::vector<AdBcOp> one(1, op);
                EMOO_TRY(tangent_planes(h, one, dslot, dtheta));
            }
        }
    }
    h->t += h->dtp;
    h->step_index++;
    return EMOO_OK;
}

// The plane sets met by the adjoint steps, in reverse order, with the
// device sums (sum LF, sum LF t1 t2) each one left in `sums`; the wave
// parameter gradient is formed from them on the host at the end.
struct PlaneLedger {
    std::vector<AdBcOp> ops;
    double *sums = nullptr;
    size_t cap = 0;
};

// adjoint of one step, given the state before it (snapshot S)
// Adjoints of plane sets, last first, each recorded in the ledger.
static int planes_adj(emoo_handle *h, const std::vector<AdBcOp> &ops, double *const *lslot, PlaneLedger &pl) {
    for (auto it = ops.rbegin(); it != ops.rend(); ++it) {
        const AdBcOp &op = *it;
        if (op.kind != 1) continue;
        if (pl.ops.size() >= pl.cap) return EMOO_ERR_STATE;
        double *sums = pl.sums + 2 * adf::PLANE_BLOCKS * pl.ops.size();
        pl.ops.push_back(op);
        h->launches++;
        k_plane_adj<<<adf::PLANE_BLOCKS, 256, 0, h->stream>>>(h->g, lslot[op.slot], op.dim, op.idx, op.t1, op.t2,
                                                              sums);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Adjoint of the corrected policy's whole-range periodic copies (fold = 0) or
// folds (fold = 1) of the slots `ids`, with the mirror folds of J at
// reflecting walls (fold = 1 on the J slots): dimensions and sides reversed.
static int periodic_full_adj(emoo_handle *h, double *const *lslot, const int *ids, int nids, int fold) {
    const Geom &g = h->g;
    adf::Slots9T<double> fl{};
    for (int k = 0; k < nids; k++) fl.p[k] = lslot[ids[k]];
    dim3 blk(32, 8);
    for (int d = 2; d >= 0; d--) {
        const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
        if (h->bc.fbc[2 * d] != FBC_PERIODIC) {
            if (!fold) continue;
            for (int r = 1; r >= 0; r--) {
                if (h->bc.pbc[2 * d + r] != PBC_REFLECTING) continue;
                dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, 3);
                h->launches++;
                adf::k_mirror_fold_adj<double><<<grd, blk, 0, h->stream>>>(g, fl, d, r);
            }
            continue;
        }
        dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, nids);
        h->launches++;
        adf::k_periodic_full_adj<double><<<grd, blk, 0, h->stream>>>(g, fl, d, fold);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

template <bool REL>
static void launch_adj(emoo_handle *h, bool corr, const SpeciesTab &st, CPArr P, FPtrs F, PArr LP, int64_t np,
                       JPtrs LJ, FOut LF) {
    const int nb = pblocks_all(np);
    if (corr)
        k_adj_particles<REL, true><<<nb, 256, 0, h->stream>>>(h->g, st, h->bc, P, F, LP, np, h->dtp, LJ, LF);
    else
        k_adj_particles<REL, false><<<nb, 256, 0, h->stream>>>(h->g, st, h->bc, P, F, LP, np, h->dtp, LJ, LF);
}

// adjoint of one step, given the state before it (snapshot S)
static int adj_step(emoo_handle *h, AdRun &R, const Snapshot &S, double **L, double *const *lslot, PlaneLedger &pl) {
    const Geom &g = h->g;
    const bool corr = corrected(h);
    const int b1 = S.bswap ^ 1;  // B roles after the step's Yee update
    // the boundary operations at the step's time and roles
    std::vector<AdBcOp> ops;
    {
        const double t_save = h->t;
        const int b_save = h->bswap;
        h->t = S.t;
        h->bswap = b1;
        int rc = ad_bc_ops(h, ops);
        h->t = t_save;
        h->bswap = b_save;
        EMOO_TRY(rc);
    }
    FOut A = field_out(lslot, b1);
    JPtrs LJ{{lslot[EMOO_JX], lslot[EMOO_JY], lslot[EMOO_JZ]}};
    dim3 blk(32, 8);
    const adf::YeeCoef<double> yc = adf::yee_coef<double>(g, h->dtp);
    if (corr) {
        // forward: E half, E images, planes, B half, E/B/B_tm1 images, planes
        static const int ids_e[3] = {EMOO_EX, EMOO_EY, EMOO_EZ};
        static const int ids9[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ,
                                    EMOO_BX_TM1, EMOO_BY_TM1, EMOO_BZ_TM1};
        static const int ids_j[3] = {EMOO_JX, EMOO_JY, EMOO_JZ};
        EMOO_TRY(planes_adj(h, ops, lslot, pl));
        EMOO_TRY(periodic_full_adj(h, lslot, ids9, 9, 0));
        h->launches += 2;
        k_yee_b_adj<<<grid_all(g, blk), blk, 0, h->stream>>>(g, yc, A);
        // the B half overwrote the B role's physical points: the values the
        // planes set there between the halves reach nothing
        adf::Slots9T<double> lb{{A.B[0], A.B[1], A.B[2]}};
        adf::k_clear_phys<double><<<dim3((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]), blk, 0, h->stream>>>(g, lb);
        EMOO_TRY(planes_adj(h, ops, lslot, pl));
        EMOO_TRY(periodic_full_adj(h, lslot, ids_e, 3, 0));
        h->launches++;
        k_yee_e_adj<<<grid_all(g, blk), blk, 0, h->stream>>>(g, yc, A, LJ);
        EMOO_TRY(periodic_full_adj(h, lslot, ids_j, 3, 1));
    } else {
        // 1. executeBC(-1), in reverse
        for (auto it = ops.rbegin(); it != ops.rend(); ++it) {
            const AdBcOp &op = *it;
            if (op.kind == 0) {
                Slots6 fl{{lslot[EMOO_EX], lslot[EMOO_EY], lslot[EMOO_EZ], lslot[EMOO_BX], lslot[EMOO_BY],
                           lslot[EMOO_BZ]}};
                for (int d = 2; d >= 0; d--) {
                    if (!((op.mask >> d) & 1)) continue;
                    const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
                    dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, 6);
                    for (int side = 1; side >= 0; side--) {
                        h->launches++;
                        k_ghost_adj<<<grd, blk, 0, h->stream>>>(g, fl, d, side);
                    }
                }
            } else {
                const std::vector<AdBcOp> one(1, op);
                EMOO_TRY(planes_adj(h, one, lslot, pl));
            }
        }
        EMOO_CUDA(cudaGetLastError());
        // 2. Yee update, in reverse (B then E), roles after the step
        h->launches += 2;
        k_yee_b_adj<<<grid_all(g, blk), blk, 0, h->stream>>>(g, yc, A);
        k_yee_e_adj<<<grid_all(g, blk), blk, 0, h->stream>>>(g, yc, A, LJ);
        // 3. the J fold, in reverse
        for (int d = 2; d >= 0; d--) {
            if (h->bc.fbc[2 * d] != FBC_PERIODIC) continue;
            const int f0 = (d == 0) ? EMOO_JY : EMOO_JX;
            const int f1 = (d == 2) ? EMOO_JY : EMOO_JZ;
            const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
            dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, 2);
            h->launches++;
            k_fold_adj<<<grd, blk, 0, h->stream>>>(g, d, lslot[f0], lslot[f1]);
        }
    }
    // particles: deposit, boundaries, push, gather, in reverse
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    PArr LP{{L[0], L[1], L[2], L[3], L[4], L[5], L[6]}};
    FOut LF = field_out(lslot, S.bswap);
    h->launches++;
    if (R.rel) launch_adj<true>(h, corr, st, R.snap_particles(S), R.snap_fields(S), LP, R.np, LJ, LF);
    else launch_adj<false>(h, corr, st, R.snap_particles(S), R.snap_fields(S), LP, R.np, LJ, LF);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

}  // namespace emoo

using namespace emoo;

extern "C" int emoo_ad_run(emoo_handle *h, const emoo_ad_spec *spec, int mode, const double *dtheta, const double *dv,
                           emoo_ad_result *out, double *grad_theta, double *grad_v) {
    if (!h || !spec || !out) return EMOO_ERR_ARG;
    if (h->host_mode) return EMOO_ERR_STATE;  // it steps the particle store
    if (h->info.electrostatic == 1) return EMOO_ERR_UNSUPPORTED;
    if (mode < EMOO_AD_FORWARD || mode > EMOO_AD_ADJOINT) return EMOO_ERR_ARG;
    if (spec->nsteps < 0 || spec->slab_lo < 0 || spec->slab_hi > h->g.n[0] || spec->slab_lo >= spec->slab_hi)
        return EMOO_ERR_ARG;
    if (spec->objective != EMOO_AD_OBJ_FIELD && spec->objective != EMOO_AD_OBJ_KINETIC) return EMOO_ERR_ARG;
    if (spec->objective == EMOO_AD_OBJ_KINETIC && (spec->species < -1 || spec->species >= h->nspec))
        return EMOO_ERR_ARG;
    if (mode == EMOO_AD_ADJOINT && spec->checkpoint_every < 1) return EMOO_ERR_ARG;
    EMOO_CUDA(cudaSetDevice(h->dev));
    if (h->precision == EMOO_MIXED) return ad_run_mixed(h, spec, mode, out, grad_theta, grad_v);
    // the run moves the particles; as after emoo_step, rho is left pending
    // (it is deposited at the final positions when read), and particles that
    // absorbing walls remove leave the store when it is next read
    if (h->opts.deposit_rho) h->rho_stale = 1;
    for (int s = 0; s < 6; s++)
        if (h->bc.pbc[s] == PBC_ABSORBING) h->dead_pending = 1;
    AdRun R;
    R.h = h;
    R.np = h->np;
    R.npts = h->g.npts;
    R.rel = h->info.relativity != 0;
    if (R.rel && !h->gam) return EMOO_ERR_STATE;
    ObjSpec os;
    os.kind = spec->objective;
    os.sl = Slab{spec->slab_lo + 1, spec->slab_hi + 1};  // cells -> grid points (first physical point is 1)
    os.ks.species = spec->species;
    os.ks.xlo = h->info.xyz0[0] + spec->slab_lo * h->g.d[0];
    os.ks.xhi = h->info.xyz0[0] + spec->slab_hi * h->g.d[0];
    const int ntheta = emoo_ad_nparams(h);
    double *dev2 = R.alloc(2);
    if (!dev2) return EMOO_ERR_OOM;
    memset(out, 0, sizeof(*out));
    cudaEvent_t ev[4];
    for (auto &e : ev) EMOO_CUDA(cudaEventCreate(&e));
    struct EvFree {
        cudaEvent_t *e;
        ~EvFree() {
            for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]);
        }
    } evfree{ev};
    double o2[2];

    if (mode == EMOO_AD_FORWARD) {
        EMOO_CUDA(cudaEventRecord(ev[0], h->stream));
        for (int n = 0; n < spec->nsteps; n++) EMOO_TRY(primal_step(h));
        EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
        EMOO_TRY(objective(h, os, nullptr, nullptr, dev2, o2));
        float ms = 0;
        EMOO_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        out->forward_ms = ms;
        out->objective = o2[0];
        return read_err(h);
    }

    if (mode == EMOO_AD_TANGENT) {
        double *dP[7];
        double *dslot[NSLOT];
        for (int a = 0; a < 7; a++) {
            if (!(dP[a] = R.alloc((size_t)std::max<int64_t>(R.np, 1)))) return EMOO_ERR_OOM;
            EMOO_CUDA(cudaMemsetAsync(dP[a], 0, sizeof(double) * R.np, h->stream));
        }
        for (int k = 0; k < NSLOT; k++) {
            if (!(dslot[k] = R.alloc((size_t)R.npts))) return EMOO_ERR_OOM;
            EMOO_CUDA(cudaMemsetAsync(dslot[k], 0, sizeof(double) * R.npts, h->stream));
        }
        if (dv)
            for (int a = 0; a < 3; a++)
                EMOO_CUDA(cudaMemcpyAsync(dP[3 + a], dv + a * R.np, sizeof(double) * R.np, cudaMemcpyHostToDevice,
                                          h->stream));
        EMOO_CUDA(cudaEventRecord(ev[0], h->stream));
        for (int n = 0; n < spec->nsteps; n++) EMOO_TRY(tlm_step(h, R, dP, dslot, dtheta));
        EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
        EMOO_TRY(objective(h, os, dslot, dP, dev2, o2));
        float ms = 0;
        EMOO_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        out->forward_ms = ms;
        out->objective = o2[0];
        out->tangent = o2[1];
        return read_err(h);
    }

    // ---- adjoint: forward with checkpoints
    const int K = spec->checkpoint_every, N = spec->nsteps;
    const int nseg = (N + K - 1) / K;
    std::vector<Snapshot> ck(std::max(nseg, 1));
    EMOO_CUDA(cudaEventRecord(ev[0], h->stream));
    for (int n = 0; n < N; n++) {
        if (n % K == 0) EMOO_TRY(R.save(ck[n / K]));
        EMOO_TRY(primal_step(h));
    }
    EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
    EMOO_TRY(objective(h, os, nullptr, nullptr, dev2, o2));  // synchronises
    out->objective = o2[0];
    {
        float ms = 0;
        EMOO_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        out->forward_ms = ms;
    }
    Snapshot fin;
    EMOO_TRY(R.save(fin));
    // adjoint state: particles and slots, seeded from the objective
    double *L[7];
    double *lslot[NSLOT];
    for (int a = 0; a < 7; a++) {
        if (!(L[a] = R.alloc((size_t)std::max<int64_t>(R.np, 1)))) return EMOO_ERR_OOM;
        EMOO_CUDA(cudaMemsetAsync(L[a], 0, sizeof(double) * R.np, h->stream));
    }
    for (int k = 0; k < NSLOT; k++) {
        if (!(lslot[k] = R.alloc((size_t)R.npts))) return EMOO_ERR_OOM;
        EMOO_CUDA(cudaMemsetAsync(lslot[k], 0, sizeof(double) * R.npts, h->stream));
    }
    h->launches++;
    if (os.kind == EMOO_AD_OBJ_FIELD) {
        FPtrs F = field_ptrs(h, h->slot, h->bswap);
        FOut A = field_out(lslot, h->bswap);
        const Slab &sl = os.sl;
        k_objective_seed<<<pblocks((int64_t)(sl.hi - sl.lo) * h->g.n[1] * h->g.n[2]), 256, 0, h->stream>>>(h->g, sl,
                                                                                                           F, A);
    } else {
        SpeciesTab st;
        species_tab(h, h->dtp, st);
        PArr LP{{L[0], L[1], L[2], L[3], L[4], L[5], L[6]}};
        if (R.rel)
            k_objective_kin_seed<true><<<pblocks(R.np), 256, 0, h->stream>>>(st, particle_arrays(h), LP, R.np, os.ks);
        else
            k_objective_kin_seed<false><<<pblocks(R.np), 256, 0, h->stream>>>(st, particle_arrays(h), LP, R.np, os.ks);
    }
    EMOO_CUDA(cudaGetLastError());
    // plane sums of every adjoint step (the plane sets per step do not change)
    PlaneLedger pl;
    {
        std::vector<AdBcOp> ops;
        EMOO_TRY(ad_bc_ops(h, ops));
        size_t per = 0;
        for (const AdBcOp &op : ops) per += op.kind == 1;
        pl.cap = per * (size_t)N * (corrected(h) ? 2 : 1);  // the corrected step sets them twice
        if (pl.cap && !(pl.sums = R.alloc(2 * adf::PLANE_BLOCKS * pl.cap))) return EMOO_ERR_OOM;
        pl.ops.reserve(pl.cap);
    }
    std::vector<Snapshot> tape(std::min(K, std::max(N, 1)));
    float rec_ms = 0, rev_ms = 0;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
        const int n0 = sgi * K, n1 = std::min(N, n0 + K);
        EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
        EMOO_TRY(R.restore(ck[sgi]));
        for (int n = n0; n < n1; n++) {
            EMOO_TRY(R.save(tape[n - n0]));
            if (n + 1 < n1) EMOO_TRY(primal_step(h));
        }
        EMOO_CUDA(cudaEventRecord(ev[2], h->stream));
        for (int n = n1 - 1; n >= n0; n--) EMOO_TRY(adj_step(h, R, tape[n - n0], L, lslot, pl));
        EMOO_CUDA(cudaEventRecord(ev[3], h->stream));
        EMOO_CUDA(cudaEventSynchronize(ev[3]));
        float a = 0, b = 0;
        EMOO_CUDA(cudaEventElapsedTime(&a, ev[1], ev[2]));
        EMOO_CUDA(cudaEventElapsedTime(&b, ev[2], ev[3]));
        rec_ms += a;
        rev_ms += b;
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    out->recompute_ms = rec_ms;
    out->reverse_ms = rev_ms;
    if (grad_theta && ntheta) {
        std::vector<double> part(2 * adf::PLANE_BLOCKS * pl.ops.size());
        if (!part.empty())
            EMOO_CUDA(cudaMemcpy(part.data(), pl.sums, sizeof(double) * part.size(), cudaMemcpyDeviceToHost));
        for (int k = 0; k < ntheta; k++) grad_theta[k] = 0.0;
        for (size_t i = 0; i < pl.ops.size(); i++) {
            const AdBcOp &op = pl.ops[i];
            double su = 0.0, ss = 0.0;
            for (int b = 0; b < adf::PLANE_BLOCKS; b++) {
                su += part[2 * (adf::PLANE_BLOCKS * i + b)];
                ss += part[2 * (adf::PLANE_BLOCKS * i + b) + 1];
            }
            for (size_t k = 0; k < op.ku.size(); k++) grad_theta[op.ku[k]] += op.cu[k] * su;
            for (size_t k = 0; k < op.ks.size(); k++) grad_theta[op.ks[k]] += op.cs[k] * ss;
        }
    }
    if (grad_v)
        for (int a = 0; a < 3; a++)
            EMOO_CUDA(cudaMemcpy(grad_v + a * R.np, L[3 + a], sizeof(double) * R.np, cudaMemcpyDeviceToHost));
    EMOO_TRY(R.restore(fin));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return read_err(h);
}
