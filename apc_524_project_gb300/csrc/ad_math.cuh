// ad_math.cuh - per-particle arithmetic of the FP64 time step, written once
// for three uses:
//   * templated on the scalar: T = double (the step itself) or T = Dual
//     (value + one directional derivative: the tangent-linear model);
//   * hand-written reverse functions (the adjoint): each takes the forward
//     inputs, recomputes what it needs and maps the adjoints of the outputs
//     to the adjoints of the inputs.
// The operation order follows the FP64 kernels in particles_f64.cu, which
// follow the reference: the gather of src/grid/oGrid.cpp:153-197 with
// src/particles/interpolate.cpp:11-47, Boris::Step src/pusher/boris.cpp:33-85,
// Relativistic_Boris::Step (Vay) src/pusher/relativisticBoris.cpp:53-140, the
// reflecting / periodic boundaries and Depositor::deposit_particle_J
// src/particles/deposit.cpp:12-39.
//
// Differentiation treats the piecewise parts as fixed: the cell a particle
// sits in (and so which grid values it reads and writes) and whether a
// boundary fires are taken from the primal state. The step is smooth in
// between; at a cell face the reference's gather is discontinuous.
//
// Host-compilable (g++) so the reverse functions can be checked against the
// Dual forward without a GPU.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define AD_HD __host__ __device__ __forceinline__
#else
#define AD_HD inline
#endif
// full unrolling of the 3- and 6-long loops on the device (their index
// arithmetic then folds into register names instead of local arrays)
#if defined(__CUDA_ARCH__)
#define AD_UNROLL _Pragma("unroll")
#else
#define AD_UNROLL
#endif

namespace emoo {
namespace ad {

struct Dual {
    double v, d;
};

AD_HD Dual mk(double v, double d = 0.0) { return Dual{v, d}; }
AD_HD double val(double x) { return x; }
AD_HD double val(const Dual &x) { return x.v; }
AD_HD Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
AD_HD Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
AD_HD Dual operator-(Dual a) { return {-a.v, -a.d}; }
AD_HD Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
AD_HD Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
AD_HD Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
AD_HD Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
AD_HD Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
AD_HD Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
AD_HD Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
AD_HD Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
AD_HD Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
AD_HD Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
AD_HD Dual sqrt(Dual a) {
    const double s = ::sqrt(a.v);
    return {s, a.d / (2.0 * s)};
}
AD_HD double sqrt_(double a) { return ::sqrt(a); }
AD_HD Dual sqrt_(Dual a) { return sqrt(a); }

// Geometry of the cell a particle is in: spacings, face areas.
struct CellGeo {
    double d[3];
    double area[3];  // d[j] * d[k]
    double vol;
    // reciprocals for the reverse functions (their products need only be
    // accurate), and the forward divisions' exact shortcut: where d[i] or
    // area[i] is a power of two, x * (1 / d) is x / d to the bit
    double id[3], iarea[3], ivol;
    int p2[3], p2area[3], p2vol;
};

// x / d as the FP64 kernels compute it (multiplication by the exact
// reciprocal when d is a power of two)
template <class T>
AD_HD T divp(const T &x, double d, double id, int p2) {
    return p2 ? x * id : x / d;
}

// The geometry of cells with spacings d0, d1, d2 (host and device).
AD_HD CellGeo make_cell_geo(double d0, double d1, double d2) {
    CellGeo c;
    c.d[0] = d0;
    c.d[1] = d1;
    c.d[2] = d2;
    for (int i = 0; i < 3; i++) c.area[i] = c.d[(i + 1) % 3] * c.d[(i + 2) % 3];
    c.vol = c.d[0] * c.d[1] * c.d[2];
    for (int i = 0; i < 3; i++) {
        c.id[i] = 1.0 / c.d[i];
        c.iarea[i] = 1.0 / c.area[i];
        int e;
        c.p2[i] = frexp(c.d[i], &e) == 0.5;
        c.p2area[i] = frexp(c.area[i], &e) == 0.5;
    }
    c.ivol = 1.0 / c.vol;
    int e;
    c.p2vol = frexp(c.vol, &e) == 0.5;
    return c;
}

// ---- gather ---------------------------------------------------------------
//
// v[0..11]: the 4 edge values of Ex, Ey, Ez in the order the FP64 kernel loads
// them; v[12..17]: the two face values of Bx, By, Bz, each (B + B_tm1) / 2.
// ds: particle minus the cell's vertex (the ghost-offset vertex, so ds is in
// [-d, 0) per axis). out: Ex, Ey, Ez, Bx, By, Bz at the particle.
template <class T>
AD_HD void gather_eval(const CellGeo &c, const T v[18], const T ds[3], T out[6]) {
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = c.d[j], lk = c.d[k], li = c.d[i];
        T e = (lj - ds[j]) * (lk - ds[k]) * v[4 * i];  // 0 + first term: the same value
        e = e + ds[j] * (lk - ds[k]) * v[4 * i + 1];
        e = e + ds[j] * ds[k] * v[4 * i + 2];
        e = e + (lj - ds[j]) * ds[k] * v[4 * i + 3];
        e = divp(e, c.area[i], c.iarea[i], c.p2area[i]);
        T b = (li - ds[i]) * v[12 + 2 * i];
        b = b + ds[i] * v[12 + 2 * i + 1];
        b = divp(b, li, c.id[i], c.p2[i]);
        out[i] = e;
        out[3 + i] = b;
    }
}

// double overload without the Dual seed
AD_HD void gather_eval(const CellGeo &c, const double v[18], const double ds[3], double out[6]) {
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = c.d[j], lk = c.d[k], li = c.d[i];
        double e = 0.0;
        e += (lj - ds[j]) * (lk - ds[k]) * v[4 * i];
        e += ds[j] * (lk - ds[k]) * v[4 * i + 1];
        e += ds[j] * ds[k] * v[4 * i + 2];
        e += (lj - ds[j]) * ds[k] * v[4 * i + 3];
        e = divp(e, c.area[i], c.iarea[i], c.p2area[i]);
        double b = (li - ds[i]) * v[12 + 2 * i];
        b += ds[i] * v[12 + 2 * i + 1];
        b = divp(b, li, c.id[i], c.p2[i]);
        out[i] = e;
        out[3 + i] = b;
    }
}

// Adjoint of gather_eval: adds to lv[18] and lds[3].
AD_HD void gather_rev(const CellGeo &c, const double v[18], const double ds[3], const double lout[6], double lv[18],
                      double lds[3]) {
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = c.d[j], lk = c.d[k], li = c.d[i];
        const double ls = lout[i] * c.iarea[i];
        const double A = lj - ds[j], Bk = lk - ds[k];
        lv[4 * i] += ls * A * Bk;
        lv[4 * i + 1] += ls * ds[j] * Bk;
        lv[4 * i + 2] += ls * ds[j] * ds[k];
        lv[4 * i + 3] += ls * A * ds[k];
        lds[j] += ls * (-Bk * v[4 * i] + Bk * v[4 * i + 1] + ds[k] * v[4 * i + 2] - ds[k] * v[4 * i + 3]);
        lds[k] += ls * (-A * v[4 * i] - ds[j] * v[4 * i + 1] + ds[j] * v[4 * i + 2] + A * v[4 * i + 3]);
        const double lb = lout[3 + i] * c.id[i];
        lv[12 + 2 * i] += lb * (li - ds[i]);
        lv[12 + 2 * i + 1] += lb * ds[i];
        lds[i] += lb * (v[12 + 2 * i + 1] - v[12 + 2 * i]);
    }
}

// ---- pushers --------------------------------------------------------------

template <class T>
AD_HD void boris_eval(double qp, const T f[6], double dt, T x[3], T v[3]) {
    const T ex = f[0], ey = f[1], ez = f[2], bx = f[3], by = f[4], bz = f[5];
    const T tx = qp * bx, ty = qp * by, tz = qp * bz;
    const T bsqr = bx * bx + by * by + bz * bz;
    const T tsqr = 2.0 / (1.0 + qp * qp * bsqr);
    const T sx = tsqr * tx, sy = tsqr * ty, sz = tsqr * tz;
    const T vmx = v[0] + qp * ex, vmy = v[1] + qp * ey, vmz = v[2] + qp * ez;
    const T vix = vmx + vmy * tz - vmz * ty;
    const T viy = vmy + vmz * tx - vmx * tz;
    const T viz = vmz + vmx * ty - vmy * tx;
    const T vpx = vmx + viy * sz - viz * sy;
    const T vpy = vmy + viz * sx - vix * sz;
    const T vpz = vmz + vix * sy - viy * sx;
    v[0] = vpx + qp * ex;
    v[1] = vpy + qp * ey;
    v[2] = vpz + qp * ez;
    for (int a = 0; a < 3; a++) x[a] = x[a] + dt * v[a];
}

template <class R>
AD_HD void cross3t(const R a[3], const R b[3], R o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
AD_HD void cross3(const double a[3], const double b[3], double o[3]) { cross3t(a, b, o); }

// Adjoint of boris_eval at inputs (f, v): lx, lv hold the adjoints of the
// outputs on entry and of the inputs on exit; lf receives the field adjoint.
// R: double (FP64 form) or float (mixed form, with dt = 0 and the position
// adjoint folded into lv by the caller).
template <class R>
AD_HD void boris_rev(R qp, const R f[6], R dt, const R v_in[3], R lx[3], R lv[3], R lf[6]) {
    const R e[3] = {f[0], f[1], f[2]}, b[3] = {f[3], f[4], f[5]};
    R t[3], s[3], vm[3], vi[3];
    for (int a = 0; a < 3; a++) t[a] = qp * b[a];
    const R bsq = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    const R tsq = R(2) / (R(1) + qp * qp * bsq);
    for (int a = 0; a < 3; a++) s[a] = tsq * t[a];
    for (int a = 0; a < 3; a++) vm[a] = v_in[a] + qp * e[a];
    R c[3];
    cross3t(vm, t, c);
    for (int a = 0; a < 3; a++) vi[a] = vm[a] + c[a];
    // x' = x + dt v': the adjoint of v' collects dt lx
    R lvp[3], le[3] = {0, 0, 0}, lb[3] = {0, 0, 0}, lvm[3], lvi[3], ls[3], lt[3];
    for (int a = 0; a < 3; a++) {
        lvp[a] = lv[a] + dt * lx[a];
        le[a] += qp * lvp[a];  // v' = vp + qp e
    }
    // vp = vm + vi x s
    R tmp[3];
    for (int a = 0; a < 3; a++) lvm[a] = lvp[a];
    cross3t(s, lvp, lvi);
    cross3t(lvp, vi, ls);
    // vi = vm + vm x t
    cross3t(t, lvi, tmp);
    for (int a = 0; a < 3; a++) lvm[a] += lvi[a] + tmp[a];
    cross3t(lvi, vm, lt);
    // vm = v + qp e
    for (int a = 0; a < 3; a++) {
        lv[a] = lvm[a];
        le[a] += qp * lvm[a];
    }
    // s = tsq t
    const R ltsq = ls[0] * t[0] + ls[1] * t[1] + ls[2] * t[2];
    for (int a = 0; a < 3; a++) lt[a] += tsq * ls[a];
    // tsq = 2 / (1 + qp^2 bsq)
    const R lbsq = ltsq * (R(-0.5) * tsq * tsq * qp * qp);
    for (int a = 0; a < 3; a++) lb[a] += R(2) * b[a] * lbsq + qp * lt[a];
    for (int a = 0; a < 3; a++) {
        lf[a] += le[a];
        lf[3 + a] += lb[a];
    }
    // lx passes through unchanged (x' = x + ...)
}

template <class T>
AD_HD void vay_eval(double qp, const T f[6], double dt, T x[3], T v[3], T &gamma) {
    const T ex = f[0], ey = f[1], ez = f[2], bx = f[3], by = f[4], bz = f[5];
    const T vXbx = v[1] * bz - v[2] * by, vXby = v[2] * bx - v[0] * bz, vXbz = v[0] * by - v[1] * bx;
    const T uhx = gamma * v[0] + qp * (ex + vXbx);
    const T uhy = gamma * v[1] + qp * (ey + vXby);
    const T uhz = gamma * v[2] + qp * (ez + vXbz);
    const T upx = uhx + qp * ex, upy = uhy + qp * ey, upz = uhz + qp * ez;
    const T gammap_sq = 1.0 + upx * upx + upy * upy + upz * upz;
    const T taux = qp * bx, tauy = qp * by, tauz = qp * bz;
    const T tau_sq = taux * taux + tauy * tauy + tauz * tauz;
    const T sigma = gammap_sq - tau_sq;
    const T ustar = upx * taux + upy * tauy + upz * tauz;
    T gi = sqrt_(sigma * sigma + 4.0 * (tau_sq + ustar * ustar));
    gi = sqrt_(0.5 * (sigma + gi));
    const T tx = taux / gi, ty = tauy / gi, tz = tauz / gi;
    const T s = 1.0 / (1.0 + tx * tx + ty * ty + tz * tz);
    const T udott = ustar / gi;
    const T cx = upy * tz - upz * ty, cy = upz * tx - upx * tz, cz = upx * ty - upy * tx;
    const T ux = s * (upx + udott * tx + cx);
    const T uy = s * (upy + udott * ty + cy);
    const T uz = s * (upz + udott * tz + cz);
    v[0] = ux / gi;
    v[1] = uy / gi;
    v[2] = uz / gi;
    for (int a = 0; a < 3; a++) x[a] = x[a] + dt * v[a];
    gamma = gi;
}

// The intermediates of one Vay step, for its reverse.
struct VayTape {
    double up[3], tau[3], tsq, sigma, ustar, gi1, gi, tt[3], s, udott, w[3], vout[3];
};

// vay_eval<double> keeping its intermediates: the same operations in the
// same order (bit-identical x, v, gamma).
AD_HD void vay_fwd(double qp, const double f[6], double dt, double x[3], double v[3], double &gamma, VayTape &T) {
    const double e[3] = {f[0], f[1], f[2]}, b[3] = {f[3], f[4], f[5]};
    double vXb[3];
    cross3(v, b, vXb);
    AD_UNROLL
    for (int a = 0; a < 3; a++) T.up[a] = gamma * v[a] + qp * (e[a] + vXb[a]) + qp * e[a];
    const double gps = 1.0 + T.up[0] * T.up[0] + T.up[1] * T.up[1] + T.up[2] * T.up[2];
    AD_UNROLL
    for (int a = 0; a < 3; a++) T.tau[a] = qp * b[a];
    T.tsq = T.tau[0] * T.tau[0] + T.tau[1] * T.tau[1] + T.tau[2] * T.tau[2];
    T.sigma = gps - T.tsq;
    T.ustar = T.up[0] * T.tau[0] + T.up[1] * T.tau[1] + T.up[2] * T.tau[2];
    T.gi1 = ::sqrt(T.sigma * T.sigma + 4.0 * (T.tsq + T.ustar * T.ustar));
    T.gi = ::sqrt(0.5 * (T.sigma + T.gi1));
    AD_UNROLL
    for (int a = 0; a < 3; a++) T.tt[a] = T.tau[a] / T.gi;
    T.s = 1.0 / (1.0 + T.tt[0] * T.tt[0] + T.tt[1] * T.tt[1] + T.tt[2] * T.tt[2]);
    T.udott = T.ustar / T.gi;
    double cr[3];
    cross3(T.up, T.tt, cr);
    AD_UNROLL
    for (int a = 0; a < 3; a++) T.w[a] = T.up[a] + T.udott * T.tt[a] + cr[a];
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        T.vout[a] = T.s * T.w[a] / T.gi;
        v[a] = T.vout[a];
        x[a] = x[a] + dt * v[a];
    }
    gamma = T.gi;
}

// Adjoint of vay_eval from its tape (inputs v_in, g_in, fields f): lx, lv,
// lg hold the output adjoints on entry and the input adjoints on exit; lf
// receives the field adjoint. Divisions by gi and gi1 are products with
// their reciprocals.
AD_HD void vay_rev_tape(const VayTape &T, double qp, const double f[6], double dt, const double v_in[3], double g_in,
                        double lx[3], double lv[3], double &lg, double lf[6]) {
    const double b[3] = {f[3], f[4], f[5]};
    const double igi = 1.0 / T.gi, igi1 = 1.0 / T.gi1;
    const double *up = T.up, *tau = T.tau, *tt = T.tt, *w = T.w, *vout = T.vout;
    const double gi = T.gi, gi1 = T.gi1, s = T.s, udott = T.udott, sigma = T.sigma, ustar = T.ustar;
    double lvo[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lvo[a] = lv[a] + dt * lx[a];
    double lgi = lg;
    double luint[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) luint[a] = lvo[a] * igi;
    lgi += -(vout[0] * lvo[0] + vout[1] * lvo[1] + vout[2] * lvo[2]) * igi;
    // uint = s w
    const double ls = w[0] * luint[0] + w[1] * luint[1] + w[2] * luint[2];
    double lw[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lw[a] = s * luint[a];
    double lup[3], ltt[3], tmp[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lup[a] = lw[a];
    const double ludott = tt[0] * lw[0] + tt[1] * lw[1] + tt[2] * lw[2];
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltt[a] = udott * lw[a];
    cross3(tt, lw, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lup[a] += tmp[a];
    cross3(lw, up, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltt[a] += tmp[a];
    // udott = ustar / gi
    double lustar = ludott * igi;
    lgi += -udott * ludott * igi;
    // s = 1 / (1 + tt.tt)
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltt[a] += -2.0 * s * s * ls * tt[a];
    // tt = tau / gi
    double ltau[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltau[a] = ltt[a] * igi;
    lgi += -(tt[0] * ltt[0] + tt[1] * ltt[1] + tt[2] * ltt[2]) * igi;
    // gi = sqrt(0.5 (sigma + gi1))
    double lsigma = 0.25 * lgi * igi;
    const double lgi1 = 0.25 * lgi * igi;
    // gi1 = sqrt(sigma^2 + 4 tsq + 4 ustar^2)
    lsigma += lgi1 * sigma * igi1;
    double ltsq = 2.0 * lgi1 * igi1;
    lustar += 4.0 * ustar * lgi1 * igi1;
    // ustar = up . tau
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lup[a] += tau[a] * lustar;
        ltau[a] += up[a] * lustar;
    }
    // sigma = gps - tsq
    const double lgps = lsigma;
    ltsq -= lsigma;
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltau[a] += 2.0 * tau[a] * ltsq;
    // gps = 1 + up.up
    AD_UNROLL
    for (int a = 0; a < 3; a++) lup[a] += 2.0 * up[a] * lgps;
    // up = g v + qp (e + v x b) + qp e
    double lb[3], le[3], lvxb[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lb[a] = qp * ltau[a];
        le[a] = 2.0 * qp * lup[a];
        lvxb[a] = qp * lup[a];
    }
    lg = v_in[0] * lup[0] + v_in[1] * lup[1] + v_in[2] * lup[2];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lv[a] = g_in * lup[a];
    cross3(b, lvxb, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lv[a] += tmp[a];
    cross3(lvxb, v_in, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lb[a] += tmp[a];
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lf[a] += le[a];
        lf[3 + a] += lb[a];
    }
    (void)gi;
    (void)gi1;
}

// Adjoint of vay_eval at inputs (f, v, gamma): lx, lv, lg hold the output
// adjoints on entry and the input adjoints on exit; lf receives the field
// adjoint.
AD_HD void vay_rev(double qp, const double f[6], double dt, const double v_in[3], double g_in, double lx[3],
                   double lv[3], double &lg, double lf[6]) {
    VayTape T;
    double x[3] = {0.0, 0.0, 0.0}, v[3] = {v_in[0], v_in[1], v_in[2]}, g = g_in;
    vay_fwd(qp, f, dt, x, v, g, T);
    vay_rev_tape(T, qp, f, dt, v_in, g_in, lx, lv, lg, lf);
}

// ---- current deposit ----------------------------------------------------
//
// The 12 J edge contributions of a particle at offset r from its cell's
// vertex with velocity vv; uq = UNIT_RHOJ q.
template <class T>
AD_HD void jterms_eval(const CellGeo &c, double uq, const T r[3], const T vv[3], T out[12]) {
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = c.d[j], lk = c.d[k];
        const T cur = uq * vv[i];
        const T ratio = divp(divp(cur, c.vol, c.ivol, c.p2vol), c.area[i], c.iarea[i], c.p2area[i]);
        out[4 * i] = ratio * (lj - r[j]) * (lk - r[k]);
        out[4 * i + 1] = ratio * r[j] * (lk - r[k]);
        out[4 * i + 2] = ratio * r[j] * r[k];
        out[4 * i + 3] = ratio * (lj - r[j]) * r[k];
    }
}

// Adjoint of jterms_eval: the adjoint of each contribution is the adjoint of
// the grid point it lands on (a gather); adds to lr[3] and lvv[3].
AD_HD void jterms_rev(const CellGeo &c, double uq, const double r[3], const double vv[3], const double lout[12],
                      double lr[3], double lvv[3]) {
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const double lj = c.d[j], lk = c.d[k];
        const double ratio = uq * vv[i] * c.ivol * c.iarea[i];
        const double A = lj - r[j], Bk = lk - r[k];
        const double l0 = lout[4 * i], l1 = lout[4 * i + 1], l2 = lout[4 * i + 2], l3 = lout[4 * i + 3];
        const double lratio = l0 * A * Bk + l1 * r[j] * Bk + l2 * r[j] * r[k] + l3 * A * r[k];
        lvv[i] += lratio * uq * c.ivol * c.iarea[i];
        lr[j] += ratio * (-l0 * Bk + l1 * Bk + l2 * r[k] - l3 * r[k]);
        lr[k] += ratio * (-l0 * A - l1 * r[j] + l2 * r[j] + l3 * A);
    }
}


// ---- charge-conserving current (corrected policy) --------------------------
//
// Villasenor and Buneman's current of a straight move p0 -> p1 (vb_deposit in
// particles_f64.cu, same operations in the same order): the path, in cell
// units u = (p - x0) / d, is split where it crosses a face (at most once per
// axis); piece k with ends ua, ub in cell c = floor((ua + ub) / 2), offsets
// aa = ua - c, bb = ub - c, extent D = bb - aa and mid m = (aa + bb) / 2 adds
// to axis a's four edges coef d_a D_a ((1-m_j)(1-m_k) + D_j D_k / 12,
// m_j (1-m_k) - .., (1-m_j) m_k - .., m_j m_k + ..) (edges at j, j+1 / k,
// k+1). Which faces are crossed and which cell a piece is in are decided on
// the primal values; the piece ends and weights carry the derivative.
struct VbGeo {
    double x0[3], id[3], d[3];
};

template <class T>
struct VbPiece {
    int cell[3];
    T W[12];  // 4 a + e: axis a, edge e (bit 0: +1 along j, bit 1: +1 along k)
};

AD_HD double cst(double v, const double *) { return v; }
AD_HD Dual cst(double v, const Dual *) { return mk(v); }

template <class T>
AD_HD int vb_eval(const VbGeo &g, const T p0[3], const T p1[3], double coef, VbPiece<T> out[4]) {
    const T *tag = nullptr;
    T u0[3], u1[3], ts[5];
    int nt = 0;
    ts[nt++] = cst(0.0, tag);
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        u0[a] = (p0[a] - g.x0[a]) * g.id[a];
        u1[a] = (p1[a] - g.x0[a]) * g.id[a];
        const double f0 = floor(val(u0[a])), f1 = floor(val(u1[a]));
        if (f0 != f1) {
            const double b = f0 > f1 ? f0 : f1;
            ts[nt++] = (b - u0[a]) / (u1[a] - u0[a]);
        }
    }
    ts[nt++] = cst(1.0, tag);
    for (int i = 2; i < nt - 1; i++)
        for (int j = i; j > 1 && val(ts[j]) < val(ts[j - 1]); j--) {
            const T t = ts[j];
            ts[j] = ts[j - 1];
            ts[j - 1] = t;
        }
    int n = 0;
    for (int sgi = 0; sgi + 1 < nt; sgi++) {
        const T ta = ts[sgi], tb = ts[sgi + 1];
        if (!(val(tb) > val(ta))) continue;
        T m[3], D[3];
        VbPiece<T> &pc = out[n++];
        AD_UNROLL
        for (int a = 0; a < 3; a++) {
            const T ua = u0[a] + ta * (u1[a] - u0[a]), ub = u0[a] + tb * (u1[a] - u0[a]);
            pc.cell[a] = (int)floor(0.5 * (val(ua) + val(ub)));
            const T aa = ua - (double)pc.cell[a], bb = ub - (double)pc.cell[a];
            D[a] = bb - aa;
            m[a] = 0.5 * (aa + bb);
        }
        AD_UNROLL
        for (int a = 0; a < 3; a++) {
            const int jb = (a + 1) % 3, kb = (a + 2) % 3;
            const T w = coef * g.d[a] * D[a];
            const T cr = D[jb] * D[kb] / 12.0;
            pc.W[4 * a + 0] = w * ((1.0 - m[jb]) * (1.0 - m[kb]) + cr);
            pc.W[4 * a + 1] = w * (m[jb] * (1.0 - m[kb]) - cr);
            pc.W[4 * a + 2] = w * ((1.0 - m[jb]) * m[kb] - cr);
            pc.W[4 * a + 3] = w * (m[jb] * m[kb] + cr);
        }
    }
    return n;
}

// Adjoint of vb_eval, written out by hand (one pass instead of six dual
// ones). lw(piece, cell, a, e) returns the adjoint of piece `piece`'s weight
// W[4 a + e] (the adjoint of the grid point it lands on; 0 for a piece the
// deposit skips); the derivatives of p0 and p1 are added to lp0 and lp1.
// Per piece, with l_e the four adjoints of axis a (j, k the other two axes):
//   W_e = w (P_e +- cr), w = coef d_a D_a, cr = D_j D_k / 12,
//   P = ((1-m_j)(1-m_k), m_j (1-m_k), (1-m_j) m_k, m_j m_k);
// then D = ub - ua, m = (ua + ub) / 2 - cell, ua = u0 + ta (u1 - u0) (ub with
// tb), a crossing t = (b - u0) / (u1 - u0) of its axis, u = (p - x0) / d.
template <class LW>
AD_HD void vb_rev(const VbGeo &g, const double p0[3], const double p1[3], double coef, LW lw, double lp0[3],
                  double lp1[3]) {
    double u0[3], u1[3], ts[5];
    int ax[5];
    int nt = 0;
    ts[nt] = 0.0;
    ax[nt++] = -1;
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        u0[a] = (p0[a] - g.x0[a]) * g.id[a];
        u1[a] = (p1[a] - g.x0[a]) * g.id[a];
        const double f0 = floor(u0[a]), f1 = floor(u1[a]);
        if (f0 != f1) {
            const double b = f0 > f1 ? f0 : f1;
            ts[nt] = (b - u0[a]) / (u1[a] - u0[a]);
            ax[nt++] = a;
        }
    }
    ts[nt] = 1.0;
    ax[nt++] = -1;
    for (int i = 2; i < nt - 1; i++)
        for (int j = i; j > 1 && ts[j] < ts[j - 1]; j--) {
            const double t = ts[j];
            ts[j] = ts[j - 1];
            ts[j - 1] = t;
            const int q = ax[j];
            ax[j] = ax[j - 1];
            ax[j - 1] = q;
        }
    double lts[5] = {0, 0, 0, 0, 0}, lu0[3] = {0, 0, 0}, lu1[3] = {0, 0, 0};
    int n = 0;
    for (int sgi = 0; sgi + 1 < nt; sgi++) {
        const double ta = ts[sgi], tb = ts[sgi + 1];
        if (!(tb > ta)) continue;
        double m[3], D[3], du[3];
        int cell[3];
        AD_UNROLL
        for (int a = 0; a < 3; a++) {
            du[a] = u1[a] - u0[a];
            const double ua = u0[a] + ta * du[a], ub = u0[a] + tb * du[a];
            cell[a] = (int)floor(0.5 * (ua + ub));
            const double aa = ua - (double)cell[a], bb = ub - (double)cell[a];
            D[a] = bb - aa;
            m[a] = 0.5 * (aa + bb);
        }
        double lD[3] = {0, 0, 0}, lm[3] = {0, 0, 0};
        AD_UNROLL
        for (int a = 0; a < 3; a++) {
            const int jb = (a + 1) % 3, kb = (a + 2) % 3;
            const double l0 = lw(n, cell, a, 0), l1 = lw(n, cell, a, 1), l2 = lw(n, cell, a, 2), l3 = lw(n, cell, a, 3);
            const double w = coef * g.d[a] * D[a];
            const double cr = D[jb] * D[kb] * (1.0 / 12.0);
            const double mj = m[jb], mk = m[kb];
            const double lwa = l0 * ((1.0 - mj) * (1.0 - mk) + cr) + l1 * (mj * (1.0 - mk) - cr) +
                               l2 * ((1.0 - mj) * mk - cr) + l3 * (mj * mk + cr);
            const double lcr = w * (l0 - l1 - l2 + l3);
            lm[jb] += w * (-l0 * (1.0 - mk) + l1 * (1.0 - mk) - l2 * mk + l3 * mk);
            lm[kb] += w * (-l0 * (1.0 - mj) - l1 * mj + l2 * (1.0 - mj) + l3 * mj);
            lD[a] += coef * g.d[a] * lwa;
            lD[jb] += lcr * D[kb] * (1.0 / 12.0);
            lD[kb] += lcr * D[jb] * (1.0 / 12.0);
        }
        AD_UNROLL
        for (int a = 0; a < 3; a++) {
            const double lua = -lD[a] + 0.5 * lm[a], lub = lD[a] + 0.5 * lm[a];
            lu0[a] += lua * (1.0 - ta) + lub * (1.0 - tb);
            lu1[a] += lua * ta + lub * tb;
            lts[sgi] += lua * du[a];
            lts[sgi + 1] += lub * du[a];
        }
        n++;
    }
    for (int i = 1; i + 1 < nt; i++) {
        const int a = ax[i];
        const double idu = 1.0 / (u1[a] - u0[a]), t = ts[i];
        lu0[a] += lts[i] * (t - 1.0) * idu;
        lu1[a] += lts[i] * (-t * idu);
    }
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lp0[a] += lu0[a] * g.id[a];
        lp1[a] += lu1[a] * g.id[a];
    }
}

}  // namespace ad
}  // namespace emoo
