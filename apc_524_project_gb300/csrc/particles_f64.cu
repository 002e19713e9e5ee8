// particles_f64.cu - FP64 particle kernels: field gather, Boris / relativistic
// Boris push, particle boundaries, current and charge deposition, and the
// fused gather + push + boundary + deposit kernel of the time loop.
//
// Compiled with --fmad=false and written in the reference's order of
// operations, so each particle's interpolated field, pushed state and
// deposited contributions are bit-identical to the reference serial build on
// the same inputs. Only the order in which contributions of different
// particles are summed differs: consecutive particles of a warp that share a
// cell are summed in a fixed shuffle tree, then added with FP64 atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {

double *role_b(emoo_handle *h, int c);
double *role_t(emoo_handle *h, int c);

namespace {

struct GatherPtrs {
    const double *E[3];
    const double *B[3];  // current B role
    const double *T[3];  // B_tm1 role
};

struct DepositPtrs {
    double *J[3];
    double *rho;
};

struct PState {
    double *x, *y, *z, *vx, *vy, *vz, *g;
};

// Grid::getFieldInterpolatorVec (src/grid/oGrid.cpp:153-197) and
// Interpolator::interpolate_fields (src/particles/interpolate.cpp:11-47) for a
// particle already known to sit in cell (ix, iy, iz).
__device__ __forceinline__ void gather_cell(const Geom &g, const GatherPtrs &P, int ix, int iy, int iz, double px,
                                            double py, double pz, double out[6]) {
    int64_t o = gidx(g, ix, iy, iz);
    const int64_t sx = g.sx, sy = g.sy;
    double v[21];
    v[0] = g.x0[0] + g.d[0] * (ix - g.vshift);
    v[1] = g.x0[1] + g.d[1] * (iy - g.vshift);
    v[2] = g.x0[2] + g.d[2] * (iz - g.vshift);
    v[3] = P.E[0][o];
    v[4] = P.E[0][o + sy];
    v[5] = P.E[0][o + sy + 1];
    v[6] = P.E[0][o + 1];
    v[7] = P.E[1][o];
    v[8] = P.E[1][o + 1];
    v[9] = P.E[1][o + sx + 1];
    v[10] = P.E[1][o + sx];
    v[11] = P.E[2][o];
    v[12] = P.E[2][o + sx];
    v[13] = P.E[2][o + sx + sy];
    v[14] = P.E[2][o + sy];
    v[15] = (P.T[0][o] + P.B[0][o]) / 2;
    v[16] = (P.T[0][o + sx] + P.B[0][o + sx]) / 2;
    v[17] = (P.T[1][o] + P.B[1][o]) / 2;
    v[18] = (P.T[1][o + sy] + P.B[1][o + sy]) / 2;
    v[19] = (P.T[2][o] + P.B[2][o]) / 2;
    v[20] = (P.T[2][o + 1] + P.B[2][o + 1]) / 2;
    double pos[3] = {px, py, pz}, ds[3];
#pragma unroll
    for (int i = 0; i < 3; i++) ds[i] = pos[i] - v[i];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = g.d[j], lk = g.d[k], li = g.d[i];
        double e = 0;
        e += (lj - ds[j]) * (lk - ds[k]) * v[3 + 4 * i];
        e += ds[j] * (lk - ds[k]) * v[3 + 4 * i + 1];
        e += ds[j] * ds[k] * v[3 + 4 * i + 2];
        e += (lj - ds[j]) * ds[k] * v[3 + 4 * i + 3];
        e = ddiv(e, g.area[i], g.iarea[i], g.area_p2[i]);
        double b = 0;
        b += (li - ds[i]) * v[15 + 2 * i];
        b += ds[i] * v[16 + 2 * i];
        b = ddiv(b, li, g.id[i], g.p2[i]);
        out[i] = e;
        out[3 + i] = b;
    }
}

// Boris::Step, src/pusher/boris.cpp:33-85 (q_p precomputed per species).
__device__ __forceinline__ void boris_push(double q_p, const double f[6], double dt, double &x, double &y, double &z,
                                           double &vx, double &vy, double &vz) {
    double ex = f[0], ey = f[1], ez = f[2], bx = f[3], by = f[4], bz = f[5];
    double tx = q_p * bx, ty = q_p * by, tz = q_p * bz;
    double bsqr = bx * bx + by * by + bz * bz;
    double tsqr = 2.0 / (1.0 + q_p * q_p * bsqr);
    double sx = tsqr * tx, sy = tsqr * ty, sz = tsqr * tz;
    double v_mx = vx + q_p * ex, v_my = vy + q_p * ey, v_mz = vz + q_p * ez;
    double v_ix = v_mx + v_my * tz - v_mz * ty;
    double v_iy = v_my + v_mz * tx - v_mx * tz;
    double v_iz = v_mz + v_mx * ty - v_my * tx;
    double v_px = v_mx + v_iy * sz - v_iz * sy;
    double v_py = v_my + v_iz * sx - v_ix * sz;
    double v_pz = v_mz + v_ix * sy - v_iy * sx;
    vx = v_px + q_p * ex;
    vy = v_py + q_p * ey;
    vz = v_pz + q_p * ez;
    x = x + dt * vx;
    y = y + dt * vy;
    z = z + dt * vz;
}

// Relativistic_Boris::Step (Vay), src/pusher/relativisticBoris.cpp:53-140.
__device__ __forceinline__ void vay_push(double q_p, const double f[6], double dt, double &x, double &y, double &z,
                                         double &vx, double &vy, double &vz, double &gamma) {
    double ex = f[0], ey = f[1], ez = f[2], bx = f[3], by = f[4], bz = f[5];
    double vXbx = vy * bz - vz * by, vXby = vz * bx - vx * bz, vXbz = vx * by - vy * bx;
    double uhx = gamma * vx + q_p * (ex + vXbx);
    double uhy = gamma * vy + q_p * (ey + vXby);
    double uhz = gamma * vz + q_p * (ez + vXbz);
    double upx = uhx + q_p * ex, upy = uhy + q_p * ey, upz = uhz + q_p * ez;
    double gammap_sq = 1.0 + upx * upx + upy * upy + upz * upz;
    double taux = q_p * bx, tauy = q_p * by, tauz = q_p * bz;
    double tau_sq = taux * taux + tauy * tauy + tauz * tauz;
    double sigma = gammap_sq - tau_sq;
    double ustar = upx * taux + upy * tauy + upz * tauz;
    double gi = sqrt(sigma * sigma + 4 * (tau_sq + ustar * ustar));
    gi = sqrt(0.5 * (sigma + gi));
    double tx = taux / gi, ty = tauy / gi, tz = tauz / gi;
    double s = 1.0 / (1.0 + tx * tx + ty * ty + tz * tz);
    double udott = ustar / gi;
    double upXt_x = upy * tz - upz * ty, upXt_y = upz * tx - upx * tz, upXt_z = upx * ty - upy * tx;
    double uint_x = s * (upx + udott * tx + upXt_x);
    double uint_y = s * (upy + udott * ty + upXt_y);
    double uint_z = s * (upz + udott * tz + upXt_z);
    vx = uint_x / gi;
    vy = uint_y / gi;
    vz = uint_z / gi;
    x = x + dt * vx;
    y = y + dt * vy;
    z = z + dt * vz;
    gamma = gi;
}

// The six particle boundaries applied to one particle in the reference's
// side order (src/particles/particle_handler.cpp:287-295). A periodic side's
// ghost copy (src/boundaries/b_particles/bc_p_periodic.cpp:52-87) becomes an
// in-place wrap that later sides see, as they see the copy; reflecting folds
// position and velocity (src/boundaries/b_particles/bc_p_reflecting.cpp:43-52);
// absorbing removes the particle. Returns the crossed-side bit mask; bit 6
// set means removed.
__device__ __forceinline__ int apply_bc(const BCTab &bc, double p[3], double v[3]) {
    int mask = 0;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const int d = s >> 1;
        const bool right = s & 1;
        double xmin = bc.xmin[d], xmax = bc.xmax[d];
        bool hit = right ? (p[d] > xmax) : (p[d] < xmin);
        if (!hit) continue;
        mask |= 1 << s;
        int kind = bc.pbc[s];
        if (kind == PBC_PERIODIC) {
            if (right) p[d] -= (xmax - xmin);
            else p[d] += (xmax - xmin);
        } else if (kind == PBC_REFLECTING) {
            p[d] = right ? 2.0 * xmax - p[d] : 2.0 * xmin - p[d];
            v[d] = -v[d];
        } else {
            mask |= 1 << 6;
            break;
        }
    }
    return mask;
}

// Depositor::deposit_particle_J / _Rho (src/particles/deposit.cpp:12-62) for
// one particle at cell (ix,iy,iz): c[0..11] J edge contributions, c[12..19]
// rho vertex contributions, in the reference's order of operations.
__device__ __forceinline__ void deposit_terms(const Geom &g, double uq, double cr, int ix, int iy, int iz, double px,
                                              double py, double pz, double vx, double vy, double vz, bool with_rho,
                                              double c[20]) {
    double r[3];
    r[0] = px - (g.x0[0] + g.d[0] * (ix - g.vshift));
    r[1] = py - (g.x0[1] + g.d[1] * (iy - g.vshift));
    r[2] = pz - (g.x0[2] + g.d[2] * (iz - g.vshift));
    const double *l = g.d;
    double vv[3] = {vx, vy, vz};
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        double cur = uq * vv[i];
        double ratio = ddiv(ddiv(cur, g.vol, g.ivol, g.vol_p2), g.area[i], g.iarea[i], g.area_p2[i]);
        c[4 * i] = ratio * (l[j] - r[j]) * (l[k] - r[k]);
        c[4 * i + 1] = ratio * r[j] * (l[k] - r[k]);
        c[4 * i + 2] = ratio * r[j] * r[k];
        c[4 * i + 3] = ratio * (l[j] - r[j]) * r[k];
    }
    if (with_rho) {
        c[12] = cr * (l[0] - r[0]) * (l[1] - r[1]) * (l[2] - r[2]);
        c[13] = cr * r[0] * (l[1] - r[1]) * (l[2] - r[2]);
        c[14] = cr * r[0] * r[1] * (l[2] - r[2]);
        c[15] = cr * (l[0] - r[0]) * r[1] * (l[2] - r[2]);
        c[16] = cr * (l[0] - r[0]) * r[1] * r[2];
        c[17] = cr * r[0] * r[1] * r[2];
        c[18] = cr * r[0] * (l[1] - r[1]) * r[2];
        c[19] = cr * (l[0] - r[0]) * (l[1] - r[1]) * r[2];
    } else {
#pragma unroll
        for (int q = 12; q < 20; q++) c[q] = 0.0;
    }
}

// Grid point of contribution q of cell o (Grid::addJ with its Jx index as in
// src/grid/oGrid.cpp:98-111, Grid::addRho src/grid/oGrid.cpp:129-136).
__device__ __forceinline__ int64_t deposit_point(const Geom &g, int64_t o, int q) {
    const int64_t sx = g.sx, sy = g.sy;
    switch (q) {
        case 0: return o;
        case 1: return o + sy;
        case 2: return o + sy + 1;
        case 3: return g.vshift ? o + 1 : o + sy;  // reference: Jx[ix][iy+1][iz] (src/grid/oGrid.cpp:101)
        case 4: return o;
        case 5: return o + 1;
        case 6: return o + sx + 1;
        case 7: return o + sx;
        case 8: return o;
        case 9: return o + sx;
        case 10: return o + sx + sy;
        case 11: return o + sy;
        case 12: return o;
        case 13: return o + sx;
        case 14: return o + sx + sy;
        case 15: return o + sy;
        case 16: return o + sy + 1;
        case 17: return o + sx + sy + 1;
        case 18: return o + sx + 1;
        default: return o + 1;
    }
}

// Warp-cooperative commit of the 20 contributions: lanes holding the same
// cell in consecutive positions are summed in a shuffle tree, the first lane
// of each run adds the run total to the grid with FP64 atomics.
__device__ __forceinline__ void commit_deposit(const Geom &g, const DepositPtrs &D, bool active, int64_t cell_o,
                                               double c[20], bool with_rho, int q_first = 0) {
    const int lane = threadIdx.x & 31;
    long long key = active ? (long long)cell_o : -1 - (long long)lane;
    long long prev = __shfl_up_sync(0xffffffffu, key, 1);
    bool head = (lane == 0) || (prev != key);
    unsigned heads = __ballot_sync(0xffffffffu, head);
    int rend = run_end(heads, lane);
    const bool all_single = (heads == 0xffffffffu);
    const int nq = with_rho ? 20 : 12;
    for (int q = q_first; q < nq; q++) {
        double v = c[q];
        if (!all_single) v = run_suffix_sum(v, lane, rend);
        if (head && active) {
            double *base = q < 4 ? D.J[0] : q < 8 ? D.J[1] : q < 12 ? D.J[2] : D.rho;
            atomicAdd(base + deposit_point(g, cell_o, q), v);
        }
    }
}

__device__ __forceinline__ void count_crossings(DevCounters *ctr, int mask) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        unsigned b = __ballot_sync(0xffffffffu, (mask >> s) & 1);
        if (lane == 0 && b) atomicAdd(&ctr->cross[s], (unsigned long long)__popc(b));
    }
}

__device__ __forceinline__ bool alive(double x) { return x == x; }

// emoo_interpolate: per-particle field cache (Particle::field).
__global__ void k_interpolate(Geom g, GatherPtrs P, PState S, int64_t np, int64_t cap, double *fc, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double x = S.x[p], y = S.y[p], z = S.z[p];
    if (!alive(x)) return;
    int ix, iy, iz;
    cell_of(g, x, y, z, ix, iy, iz);
    if (!cell_ok(g, ix, iy, iz)) {
        atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
        return;
    }
    double f[6];
    gather_cell(g, P, ix, iy, iz, x, y, z, f);
#pragma unroll
    for (int q = 0; q < 6; q++) fc[q * cap + p] = f[q];
}

// emoo_push: Particle_Handler::Push with the cached fields.
__global__ void k_push_cached(SpeciesTab st, PState S, int64_t np, int64_t cap, const double *fc, double dt, int rel) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double x = S.x[p], y = S.y[p], z = S.z[p];
    if (!alive(x)) return;
    int s = species_of(st, p);
    double f[6];
#pragma unroll
    for (int q = 0; q < 6; q++) f[q] = fc[q * cap + p];
    double vx = S.vx[p], vy = S.vy[p], vz = S.vz[p];
    if (rel) {
        double ga = S.g[p];
        vay_push(st.qp[s], f, dt, x, y, z, vx, vy, vz, ga);
        S.g[p] = ga;
    } else {
        boris_push(st.qp[s], f, dt, x, y, z, vx, vy, vz);
    }
    S.x[p] = x; S.y[p] = y; S.z[p] = z;
    S.vx[p] = vx; S.vy[p] = vy; S.vz[p] = vz;
}

__global__ void k_particle_bc(BCTab bc, PState S, int64_t np, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int mask = 0;
    if (p < np) {
        double pos[3] = {S.x[p], S.y[p], S.z[p]};
        if (alive(pos[0])) {
            double v[3] = {S.vx[p], S.vy[p], S.vz[p]};
            mask = apply_bc(bc, pos, v);
            if (mask & 64) pos[0] = __longlong_as_double(0x7ff8000000000000LL);
            if (mask) {
                S.x[p] = pos[0]; S.y[p] = pos[1]; S.z[p] = pos[2];
                S.vx[p] = v[0]; S.vy[p] = v[1]; S.vz[p] = v[2];
            }
        }
    }
    count_crossings(ctr, mask);
}

__global__ void k_deposit(Geom g, SpeciesTab st, PState S, int64_t np, DepositPtrs D, int with_rho, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool active = false;
    int64_t o = 0;
    double c[20] = {0.0};
    if (p < np) {
        double x = S.x[p];
        int s = species_of(st, p);
        if (alive(x) && st.deposit[s]) {
            double y = S.y[p], z = S.z[p];
            int ix, iy, iz;
            cell_of(g, x, y, z, ix, iy, iz);
            if (cell_ok(g, ix, iy, iz)) {
                active = true;
                o = gidx(g, ix, iy, iz);
                deposit_terms(g, st.uq[s], st.cr[s], ix, iy, iz, x, y, z, S.vx[p], S.vy[p], S.vz[p], with_rho, c);
            } else {
                atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
            }
        }
    }
    // with_rho: 0 J, 1 J and rho, 2 rho only
    commit_deposit(g, D, active, o, c, with_rho != 0, with_rho == 2 ? 12 : 0);
}

// Villasenor-Buneman current (J. Villasenor and O. Buneman, Comput. Phys.
// Commun. 69 (1992) 306) of a particle moving in a straight line from p0 to
// p1 (unwrapped, at most one cell face per axis), for the corrected policy:
// the path is split at the faces it crosses; a piece with offsets a -> b in a
// cell (cell units, m = (a + b) / 2, D = b - a) adds to the cell's four x
// edges coef dx Dx ((1-my)(1-mz) + Dy Dz / 12), (my (1-mz) - ..),
// ((1-my) mz - ..), (my mz + ..), and likewise for y and z; with the linear
// charge assignment, rho(t + dt) - rho(t) + dt div J = 0 at every point.
// coef = UNIT_RHOJ q / V / dt. Pieces outside the box land in the ghost
// planes, which the periodic fold adds back.
__device__ void vb_deposit(const Geom &g, const DepositPtrs &D, const double p0[3], const double p1[3], double coef) {
    double u0[3], u1[3], ts[5];
    int nt = 0;
    ts[nt++] = 0.0;
    for (int a = 0; a < 3; a++) {
        u0[a] = (p0[a] - g.x0[a]) * g.id[a];
        u1[a] = (p1[a] - g.x0[a]) * g.id[a];
        const double f0 = floor(u0[a]), f1 = floor(u1[a]);
        if (f0 != f1) {
            const double b = f0 > f1 ? f0 : f1;
            ts[nt++] = (b - u0[a]) / (u1[a] - u0[a]);
        }
    }
    ts[nt++] = 1.0;
    for (int i = 2; i < nt - 1; i++)
        for (int j = i; j > 1 && ts[j] < ts[j - 1]; j--) {
            const double t = ts[j];
            ts[j] = ts[j - 1];
            ts[j - 1] = t;
        }
    for (int sgi = 0; sgi + 1 < nt; sgi++) {
        const double ta = ts[sgi], tb = ts[sgi + 1];
        if (!(tb > ta)) continue;
        double m[3], Dd[3];
        int cell[3];
        for (int a = 0; a < 3; a++) {
            const double ua = u0[a] + ta * (u1[a] - u0[a]), ub = u0[a] + tb * (u1[a] - u0[a]);
            cell[a] = (int)floor(0.5 * (ua + ub));
            const double aa = ua - cell[a], bb = ub - cell[a];
            Dd[a] = bb - aa;
            m[a] = 0.5 * (aa + bb);
        }
        // every point of the piece's cell exists: cells -1..n (the path moves less
        // than a cell per axis from a physical position); out of range is recorded
        bool ok = true;
        for (int a = 0; a < 3; a++) ok = ok && cell[a] >= -1 && cell[a] + 2 < g.tot[a];
        if (!ok) continue;
        for (int a = 0; a < 3; a++) {
            const int jb = (a + 1) % 3, kb = (a + 2) % 3;
            const double w = coef * g.d[a] * Dd[a];
            const double cr = Dd[jb] * Dd[kb] / 12.0;
            const double W[4] = {w * ((1.0 - m[jb]) * (1.0 - m[kb]) + cr), w * (m[jb] * (1.0 - m[kb]) - cr),
                                 w * ((1.0 - m[jb]) * m[kb] - cr), w * (m[jb] * m[kb] + cr)};
            for (int e = 0; e < 4; e++) {
                int ii[3] = {cell[0] + 1, cell[1] + 1, cell[2] + 1};
                ii[jb] += e & 1;
                ii[kb] += e >> 1;
                atomicAdd(D.J[a] + gidx(g, ii[0], ii[1], ii[2]), W[e]);
            }
        }
    }
}

// The corrected policy's time-loop kernel: gather at the current position
// (the cell's own vertex), push, the charge-conserving current of the move,
// then the (periodic) boundaries.
// A move that ends beyond an absorbing wall removes the particle; its whole
// charge must cross the wall's vertex plane for continuity to hold there, so
// the path is continued along the wall's normal to the next vertex plane
// beyond the wall (x0 - d or x0 + L + d), a piece inside the ghost cell
// (corrected policy, as the oracle's absorbed_exit).
__device__ void absorbed_exit(const Geom &g, const BCTab &bc, const DepositPtrs &D, const double p1[3],
                              double coef) {
    double a[3] = {p1[0], p1[1], p1[2]};
    for (int d = 0; d < 3; d++) {
        double b[3] = {a[0], a[1], a[2]};
        if (bc.pbc[2 * d] == PBC_ABSORBING && a[d] < bc.xmin[d]) b[d] = bc.xmin[d] - g.d[d];
        else if (bc.pbc[2 * d + 1] == PBC_ABSORBING && a[d] > bc.xmax[d]) b[d] = bc.xmax[d] + g.d[d];
        else continue;
        vb_deposit(g, D, a, b, coef);
        a[d] = b[d];
    }
}

template <bool REL>
__global__ void __launch_bounds__(256) k_fused_vb(Geom g, SpeciesTab st, BCTab bc, GatherPtrs P, PState S, int64_t np,
                                                  DepositPtrs D, double dt, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int mask = 0;
    if (p < np) {
        double x = S.x[p], y = S.y[p], z = S.z[p];
        if (alive(x)) {
            int s = species_of(st, p);
            int ix, iy, iz;
            cell_of(g, x, y, z, ix, iy, iz);
            if (!cell_ok(g, ix, iy, iz)) {
                atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
            } else {
                const double p0[3] = {x, y, z};
                double f[6];
                gather_cell(g, P, ix, iy, iz, x, y, z, f);
                double vx = S.vx[p], vy = S.vy[p], vz = S.vz[p];
                if (REL) {
                    double ga = S.g[p];
                    vay_push(st.qp[s], f, dt, x, y, z, vx, vy, vz, ga);
                    S.g[p] = ga;
                } else {
                    boris_push(st.qp[s], f, dt, x, y, z, vx, vy, vz);
                }
                double pos[3] = {x, y, z}, v[3] = {vx, vy, vz};
                if (st.deposit[s] && dt > 0.0) {
                    vb_deposit(g, D, p0, pos, st.uq[s] / g.vol / dt);
                    absorbed_exit(g, bc, D, pos, st.uq[s] / g.vol / dt);
                }
                mask = apply_bc(bc, pos, v);
                if (mask & 64) pos[0] = __longlong_as_double(0x7ff8000000000000LL);
                S.x[p] = pos[0]; S.y[p] = pos[1]; S.z[p] = pos[2];
                S.vx[p] = v[0]; S.vy[p] = v[1]; S.vz[p] = v[2];
            }
        }
    }
    count_crossings(ctr, mask);
}

// The fused time-loop kernel: gather at the current position (what
// InterpolateEB cached at the end of the previous step), push, the six
// boundaries, then deposit at the new position.
template <bool REL>
__global__ void __launch_bounds__(256) k_fused(Geom g, SpeciesTab st, BCTab bc, GatherPtrs P, PState S, int64_t np,
                                               DepositPtrs D, double dt, int with_rho, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool active = false;
    int64_t o = 0;
    int mask = 0;
    double c[20] = {0.0};
    if (p < np) {
        double x = S.x[p], y = S.y[p], z = S.z[p];
        if (alive(x)) {
            int s = species_of(st, p);
            int ix, iy, iz;
            cell_of(g, x, y, z, ix, iy, iz);
            if (!cell_ok(g, ix, iy, iz)) {
                atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
            } else {
                double f[6];
                gather_cell(g, P, ix, iy, iz, x, y, z, f);
                double vx = S.vx[p], vy = S.vy[p], vz = S.vz[p];
                if (REL) {
                    double ga = S.g[p];
                    vay_push(st.qp[s], f, dt, x, y, z, vx, vy, vz, ga);
                    S.g[p] = ga;
                } else {
                    boris_push(st.qp[s], f, dt, x, y, z, vx, vy, vz);
                }
                double pos[3] = {x, y, z}, v[3] = {vx, vy, vz};
                mask = apply_bc(bc, pos, v);
                if (mask & 64) {
                    pos[0] = __longlong_as_double(0x7ff8000000000000LL);
                } else if (st.deposit[s]) {
                    cell_of(g, pos[0], pos[1], pos[2], ix, iy, iz);
                    if (cell_ok(g, ix, iy, iz)) {
                        active = true;
                        o = gidx(g, ix, iy, iz);
                        deposit_terms(g, st.uq[s], st.cr[s], ix, iy, iz, pos[0], pos[1], pos[2], v[0], v[1], v[2],
                                      with_rho != 0, c);
                    } else {
                        atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
                    }
                }
                S.x[p] = pos[0]; S.y[p] = pos[1]; S.z[p] = pos[2];
                S.vx[p] = v[0]; S.vy[p] = v[1]; S.vz[p] = v[2];
            }
        }
    }
    count_crossings(ctr, mask);
    commit_deposit(g, D, active, o, c, with_rho != 0);
}

// Per-block partial sums of the history's particle terms
// (src/IO/output.cpp:76-87): {sum 1/2 m v^2, sum m vx, sum m vy, sum m vz}.
__global__ void k_moments(SpeciesTab st, PState S, int64_t np, double *part) {
    double acc[4] = {0, 0, 0, 0};
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        double vx = S.vx[p], vy = S.vy[p], vz = S.vz[p];
        if (!alive(S.x[p])) continue;
        double m = st.m[species_of(st, p)];
        acc[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[1] += m * vx;
        acc[2] += m * vy;
        acc[3] += m * vz;
    }
    __shared__ double sh[32][4];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 4; q++) {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) v += sh[ww][threadIdx.x];
        part[blockIdx.x * 4 + threadIdx.x] = v;
    }
}

// Sort keys: species * ncell + reference cellID; removed particles get the
// largest key so they end up behind every live one.
__global__ void k_keys(Geom g, SpeciesTab st, PState S, int64_t np, uint32_t *key, uint32_t dead_key, DevCounters *ctr) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double x = S.x[p];
    if (!alive(x)) {
        key[p] = dead_key;
        return;
    }
    int ix, iy, iz;
    cell_of(g, x, S.y[p], S.z[p], ix, iy, iz);
    if (ix < 0 || iy < 0 || iz < 0 || ix >= g.n[0] + 2 || iy >= g.n[1] + 2 || iz >= g.n[2] + 2) {
        atomicOr(&ctr->err, (unsigned long long)ERR_BOUNDS);
        key[p] = dead_key - 1;
        return;
    }
    int s = species_of(st, p);
    key[p] = (uint32_t)((int64_t)s * g.ncell + cell_id(g, ix, iy, iz));
}

GatherPtrs gather_ptrs(emoo_handle *h) {
    GatherPtrs P;
    for (int c = 0; c < 3; c++) {
        P.E[c] = h->slot[EMOO_EX + c];
        P.B[c] = role_b(h, c);
        P.T[c] = role_t(h, c);
    }
    return P;
}

DepositPtrs deposit_ptrs(emoo_handle *h) {
    DepositPtrs D;
    for (int c = 0; c < 3; c++) D.J[c] = h->slot[EMOO_JX + c];
    D.rho = h->slot[EMOO_RHO];
    return D;
}

PState pstate(emoo_handle *h) { return PState{h->x, h->y, h->z, h->vx, h->vy, h->vz, h->gam}; }

int blocks_for(int64_t n, int t = 256) { return (int)std::max<int64_t>(1, (n + t - 1) / t); }

// ---- sensitivity probe (no reference counterpart) -------------------------

// Uniform in [-1, 1) from (seed, particle or point, component): splitmix64.
__device__ __forceinline__ double unit_noise(uint64_t seed, uint64_t i, uint64_t comp) {
    uint64_t z = seed + (i * 8u + comp + 1u) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 4503599627370496.0) - 1.0;  // 2^-52 steps over [-1, 1)
}

// Every live particle: v *= 1 + rel u, x += rel d u per component (u the
// noise above), a moved position kept only while it stays inside the box.
__global__ void k_perturb_particles(Geom g, PState S, int64_t np, uint64_t seed, double rel) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np || S.x[p] != S.x[p]) return;
    double *pos[3] = {S.x, S.y, S.z}, *vel[3] = {S.vx, S.vy, S.vz};
    for (int c = 0; c < 3; c++) {
        vel[c][p] *= 1.0 + rel * unit_noise(seed, (uint64_t)p, c);
        const double x = pos[c][p] + rel * g.d[c] * unit_noise(seed, (uint64_t)p, 3 + c);
        if (x >= g.x0[c] && x < g.x0[c] + g.n[c] * g.d[c]) pos[c][p] = x;
    }
}

// f *= 1 + rel u at every point of one field (comp tells fields apart).
__global__ void k_perturb_field(double *f, int64_t n, uint64_t seed, uint64_t comp, double rel) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) f[i] *= 1.0 + rel * unit_noise(seed, (uint64_t)i, comp);
}

}  // namespace

void species_tab(emoo_handle *h, double dtp, SpeciesTab &st) {
    st.nspec = h->nspec;
    for (int s = 0; s <= h->nspec; s++) st.off[s] = h->off[s];
    for (int s = h->nspec + 1; s <= EMOO_NSPEC; s++) st.off[s] = h->off[h->nspec];
    const Geom &g = h->g;
    for (int s = 0; s < EMOO_NSPEC; s++) {
        double q = h->info.charge_ratio[s], m = h->info.mass_ratio[s];
        st.q[s] = q;
        st.m[s] = m;
        double qp = (0.5 * dtp * q) / m;
        qp *= UNIT_ACC;
        st.qp[s] = qp;
        st.uq[s] = UNIT_RHOJ * q;
        st.cr[s] = UNIT_RHOJ * (q / g.vol) / g.vol;
        st.deposit[s] = h->info.isTestParticle[s] ? 0 : 1;
    }
}

int interpolate_f64(emoo_handle *h) {
    if (h->np == 0) return EMOO_OK;
    if (!h->fcache) EMOO_CUDA(cudaMalloc(&h->fcache, sizeof(double) * 6 * (size_t)h->cap));
    h->launches++;
    k_interpolate<<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, gather_ptrs(h), pstate(h), h->np, h->cap, h->fcache,
                                                            h->ctr);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int push_cached_f64(emoo_handle *h, double dtp) {
    if (h->np == 0) return EMOO_OK;
    if (!h->fcache) return EMOO_ERR_STATE;
    SpeciesTab st;
    species_tab(h, dtp, st);
    h->launches++;
    k_push_cached<<<blocks_for(h->np), 256, 0, h->stream>>>(st, pstate(h), h->np, h->cap, h->fcache, dtp,
                                                            h->info.relativity != 0);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int particle_bc_f64(emoo_handle *h) {
    if (h->np == 0) return EMOO_OK;
    h->launches++;
    k_particle_bc<<<blocks_for(h->np), 256, 0, h->stream>>>(h->bc, pstate(h), h->np, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int deposit_f64(emoo_handle *h, int with_rho) {
    size_t bytes = sizeof(double) * (size_t)h->g.npts;
    for (int c = 0; c < 3; c++) EMOO_CUDA(cudaMemsetAsync(h->slot[EMOO_JX + c], 0, bytes, h->stream));
    if (with_rho) EMOO_CUDA(cudaMemsetAsync(h->slot[EMOO_RHO], 0, bytes, h->stream));
    if (h->np == 0) return rho_background_f64(h, with_rho);
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    h->launches++;
    k_deposit<<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, pstate(h), h->np, deposit_ptrs(h), with_rho, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    return rho_background_f64(h, with_rho);
}

// rho alone at the particles' current positions (J untouched), plus the
// background: the charge density the loop's last deposit would have left.
int deposit_rho_f64(emoo_handle *h) {
    EMOO_CUDA(cudaMemsetAsync(h->slot[EMOO_RHO], 0, sizeof(double) * (size_t)h->g.npts, h->stream));
    if (h->np > 0) {
        SpeciesTab st;
        species_tab(h, h->dtp, st);
        h->launches++;
        k_deposit<<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, pstate(h), h->np, deposit_ptrs(h), 2, h->ctr);
        EMOO_CUDA(cudaGetLastError());
    }
    return rho_background_f64(h, 1);
}

int fused_step_f64(emoo_handle *h, double dtp, int with_rho) {
    size_t bytes = sizeof(double) * (size_t)h->g.npts;
    for (int c = 0; c < 3; c++) EMOO_CUDA(cudaMemsetAsync(h->slot[EMOO_JX + c], 0, bytes, h->stream));
    if (with_rho) EMOO_CUDA(cudaMemsetAsync(h->slot[EMOO_RHO], 0, bytes, h->stream));
    if (h->np == 0) return rho_background_f64(h, with_rho);
    SpeciesTab st;
    species_tab(h, dtp, st);
    if (h->policy == EMOO_POLICY_CORRECTED) {
        // current along the paths; rho (when asked for) at the new positions
        h->launches++;
        if (h->info.relativity)
            k_fused_vb<true><<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, h->bc, gather_ptrs(h), pstate(h),
                                                                      h->np, deposit_ptrs(h), dtp, h->ctr);
        else
            k_fused_vb<false><<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, h->bc, gather_ptrs(h), pstate(h),
                                                                       h->np, deposit_ptrs(h), dtp, h->ctr);
        EMOO_CUDA(cudaGetLastError());
        if (!with_rho) return EMOO_OK;
        return deposit_rho_f64(h);
    }
    h->launches++;
    if (h->prof_on) EMOO_CUDA(cudaEventRecord(h->prof_ev[0], h->stream));
    if (h->info.relativity)
        k_fused<true><<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, h->bc, gather_ptrs(h), pstate(h), h->np,
                                                                deposit_ptrs(h), dtp, with_rho, h->ctr);
    else
        k_fused<false><<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, h->bc, gather_ptrs(h), pstate(h), h->np,
                                                                 deposit_ptrs(h), dtp, with_rho, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    if (h->prof_on) {
        EMOO_CUDA(cudaEventRecord(h->prof_ev[1], h->stream));
        EMOO_TRY(prof_accumulate(h));
    }
    return rho_background_f64(h, with_rho);
}

int particle_moments_f64(emoo_handle *h, double out4[4]) {
    for (int q = 0; q < 4; q++) out4[q] = 0.0;
    if (h->np == 0) return EMOO_OK;
    int nb = (int)std::min<int64_t>(blocks_for(h->np), 152 * 8);
    if (h->red_cap < (size_t)nb * 4) {
        if (h->red) cudaFree(h->red);
        EMOO_CUDA(cudaMalloc(&h->red, (size_t)nb * 4 * sizeof(double)));
        h->red_cap = (size_t)nb * 4;
    }
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    h->launches++;
    k_moments<<<nb, 256, 0, h->stream>>>(st, pstate(h), h->np, h->red);
    EMOO_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)nb * 4);
    EMOO_CUDA(cudaMemcpyAsync(part.data(), h->red, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 4; q++) out4[q] += part[(size_t)b * 4 + q];
    return EMOO_OK;
}

// Compaction keys: the species index, nspec for removed particles (a stable
// sort by them drops the removed particles and keeps every species' order).
__global__ void k_compact_keys(SpeciesTab st, const double *x, int64_t np, uint32_t *key) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    key[p] = alive(x[p]) ? (uint32_t)species_of(st, p) : (uint32_t)st.nspec;
}

int compact_keys_f64(emoo_handle *h) {
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    h->launches++;
    k_compact_keys<<<blocks_for(h->np), 256, 0, h->stream>>>(st, h->x, h->np, h->key[0]);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

int perturb_f64(emoo_handle *h, uint64_t seed, double rel) {
    if (h->np) {
        h->launches++;
        k_perturb_particles<<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, pstate(h), h->np, seed, rel);
        EMOO_CUDA(cudaGetLastError());
    }
    const int ids[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ, EMOO_BX_TM1, EMOO_BY_TM1, EMOO_BZ_TM1};
    for (int k = 0; k < 9; k++) {
        h->launches++;
        k_perturb_field<<<blocks_for(h->g.npts), 256, 0, h->stream>>>(h->slot[ids[k]], h->g.npts, seed, 8 + k, rel);
        EMOO_CUDA(cudaGetLastError());
    }
    return EMOO_OK;
}

int sort_keys_f64(emoo_handle *h) {
    SpeciesTab st;
    species_tab(h, h->dtp, st);
    uint32_t dead = (uint32_t)((int64_t)h->nspec * h->g.ncell + 1);
    h->launches++;
    k_keys<<<blocks_for(h->np), 256, 0, h->stream>>>(h->g, st, pstate(h), h->np, h->key[0], dead, h->ctr);
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

}  // namespace emoo
