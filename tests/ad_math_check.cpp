// Host check of apc_524_project_gb300/csrc/ad_math.cuh and ad_mixed.cuh
// (built by tests/test_ad_math.py with g++): for the gather, both pushers and
// the current terms of the FP64 form, and the pack gather, the u-form Vay
// pusher and the cell-unit current terms of the mixed form, on seeded random
// inputs,
//   * the Dual (tangent-linear) derivative matches a central difference of
//     the double evaluation;
//   * the reverse (adjoint) function is the transpose of the Dual one:
//     <lambda, J delta> == <J^T lambda, delta> to rounding.
// Prints one line per check and exits non-zero if any fails.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "ad_math.cuh"
#include "ad_mixed.cuh"

using namespace emoo::ad;

static std::mt19937_64 rng(20240404);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

static int failures = 0;
static void report(const char *what, double got, double want, double tol) {
    double err = std::fabs(got - want) / std::fmax(std::fabs(want), 1e-300);
    bool ok = err <= tol;
    if (!ok) failures++;
    std::printf("%-28s %s  got % .16e want % .16e rel %.2e\n", what, ok ? "ok  " : "FAIL", got, want, err);
}

static CellGeo geo() {
    const double d0 = U(0.5, 1.5), d1 = U(0.5, 1.5), d2 = U(0.5, 1.5);
    return make_cell_geo(d0, d1, d2);
}

// generic check of a map R^n -> R^m given as double and Dual evaluations
template <class FD, class FDual, class FRev>
static void check(const char *name, int n, int m, const double *x0, FD fd, FDual fdual, FRev frev, double fd_tol) {
    std::vector<double> dir(n), lam(m), y(m), yp(m), ym(m), xp(n), xm(n), jd(m), jtl(n, 0.0);
    for (int i = 0; i < n; i++) dir[i] = U(-1, 1);
    for (int i = 0; i < m; i++) lam[i] = U(-1, 1);
    // Dual directional derivative
    fdual(x0, dir.data(), jd.data());
    // central difference
    const double h = 1e-6;
    for (int i = 0; i < n; i++) {
        xp[i] = x0[i] + h * dir[i];
        xm[i] = x0[i] - h * dir[i];
    }
    fd(xp.data(), yp.data());
    fd(xm.data(), ym.data());
    double num = 0, den = 0;
    for (int i = 0; i < m; i++) {
        double c = (yp[i] - ym[i]) / (2 * h);
        num += (c - jd[i]) * (c - jd[i]);
        den += jd[i] * jd[i];
    }
    char buf[96];
    const double rel = std::sqrt(num / den);
    const bool fd_ok = rel <= fd_tol;
    if (!fd_ok) failures++;
    std::printf("%-28s %s  relative L2 %.2e (bar %.0e)\n", (std::string(name) + " tangent vs FD").c_str(),
                fd_ok ? "ok  " : "FAIL", rel, fd_tol);
    // adjoint: J^T lam
    frev(x0, lam.data(), jtl.data());
    double lhs = 0, rhs = 0;
    for (int i = 0; i < m; i++) lhs += lam[i] * jd[i];
    for (int i = 0; i < n; i++) rhs += jtl[i] * dir[i];
    std::snprintf(buf, sizeof buf, "%s <l,Jd> = <J'l,d>", name);
    report(buf, rhs, lhs, 1e-12);
}

int main() {
    for (int trial = 0; trial < 5; trial++) {
        const CellGeo c = geo();
        // ---- gather: inputs v[18], ds[3] -> out[6]
        {
            double x0[21];
            for (int i = 0; i < 18; i++) x0[i] = U(-1, 1);
            for (int a = 0; a < 3; a++) x0[18 + a] = -U(0.0, 1.0) * c.d[a];
            auto fd = [&](const double *x, double *y) { gather_eval(c, x, x + 18, y); };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual v[18], ds[3], o[6];
                for (int i = 0; i < 18; i++) v[i] = mk(x[i], d[i]);
                for (int a = 0; a < 3; a++) ds[a] = mk(x[18 + a], d[18 + a]);
                gather_eval(c, v, ds, o);
                for (int i = 0; i < 6; i++) jd[i] = o[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                gather_rev(c, x, x + 18, l, jt, jt + 18);
            };
            check("gather", 21, 6, x0, fd, fdual, frev, 1e-7);
        }
        // ---- Boris: inputs f[6], x[3], v[3] -> x'[3], v'[3]
        {
            const double qp = U(-0.3, 0.3), dt = 0.5;
            double x0[12];
            for (int i = 0; i < 6; i++) x0[i] = U(-1, 1);
            for (int i = 6; i < 9; i++) x0[i] = U(0, 10);
            for (int i = 9; i < 12; i++) x0[i] = U(-0.5, 0.5);
            auto fd = [&](const double *x, double *y) {
                double xx[3] = {x[6], x[7], x[8]}, vv[3] = {x[9], x[10], x[11]};
                boris_eval(qp, x, dt, xx, vv);
                for (int a = 0; a < 3; a++) { y[a] = xx[a]; y[3 + a] = vv[a]; }
            };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual f[6], xx[3], vv[3];
                for (int i = 0; i < 6; i++) f[i] = mk(x[i], d[i]);
                for (int a = 0; a < 3; a++) { xx[a] = mk(x[6 + a], d[6 + a]); vv[a] = mk(x[9 + a], d[9 + a]); }
                boris_eval(qp, f, dt, xx, vv);
                for (int a = 0; a < 3; a++) { jd[a] = xx[a].d; jd[3 + a] = vv[a].d; }
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                double lx[3] = {l[0], l[1], l[2]}, lv[3] = {l[3], l[4], l[5]}, lf[6] = {0, 0, 0, 0, 0, 0};
                boris_rev(qp, x, dt, x + 9, lx, lv, lf);
                for (int i = 0; i < 6; i++) jt[i] = lf[i];
                for (int a = 0; a < 3; a++) { jt[6 + a] = lx[a]; jt[9 + a] = lv[a]; }
            };
            check("boris", 12, 6, x0, fd, fdual, frev, 1e-7);
        }
        // ---- Vay: inputs f[6], x[3], v[3], gamma -> x'[3], v'[3], gamma'
        {
            const double qp = U(-0.3, 0.3), dt = 0.5;
            double x0[13];
            for (int i = 0; i < 6; i++) x0[i] = U(-1, 1);
            for (int i = 6; i < 9; i++) x0[i] = U(0, 10);
            for (int i = 9; i < 12; i++) x0[i] = U(-0.5, 0.5);
            x0[12] = 1.0 / std::sqrt(1.0 - (x0[9] * x0[9] + x0[10] * x0[10] + x0[11] * x0[11]));
            auto fd = [&](const double *x, double *y) {
                double xx[3] = {x[6], x[7], x[8]}, vv[3] = {x[9], x[10], x[11]}, g = x[12];
                vay_eval(qp, x, dt, xx, vv, g);
                for (int a = 0; a < 3; a++) { y[a] = xx[a]; y[3 + a] = vv[a]; }
                y[6] = g;
            };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual f[6], xx[3], vv[3], g = mk(x[12], d[12]);
                for (int i = 0; i < 6; i++) f[i] = mk(x[i], d[i]);
                for (int a = 0; a < 3; a++) { xx[a] = mk(x[6 + a], d[6 + a]); vv[a] = mk(x[9 + a], d[9 + a]); }
                vay_eval(qp, f, dt, xx, vv, g);
                for (int a = 0; a < 3; a++) { jd[a] = xx[a].d; jd[3 + a] = vv[a].d; }
                jd[6] = g.d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                double lx[3] = {l[0], l[1], l[2]}, lv[3] = {l[3], l[4], l[5]}, lg = l[6], lf[6] = {0, 0, 0, 0, 0, 0};
                vay_rev(qp, x, dt, x + 9, x[12], lx, lv, lg, lf);
                for (int i = 0; i < 6; i++) jt[i] = lf[i];
                for (int a = 0; a < 3; a++) { jt[6 + a] = lx[a]; jt[9 + a] = lv[a]; }
                jt[12] = lg;
            };
            check("vay", 13, 7, x0, fd, fdual, frev, 1e-7);
        }
        // ---- J terms: inputs r[3], v[3] -> 12 contributions
        {
            const double uq = U(-2, 2);
            double x0[6];
            for (int a = 0; a < 3; a++) x0[a] = -U(0.0, 1.0) * c.d[a];
            for (int a = 3; a < 6; a++) x0[a] = U(-0.5, 0.5);
            auto fd = [&](const double *x, double *y) { jterms_eval(c, uq, x, x + 3, y); };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual r[3], vv[3], o[12];
                for (int a = 0; a < 3; a++) { r[a] = mk(x[a], d[a]); vv[a] = mk(x[3 + a], d[3 + a]); }
                jterms_eval(c, uq, r, vv, o);
                for (int i = 0; i < 12; i++) jd[i] = o[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) { jterms_rev(c, uq, x, x + 3, l, jt, jt + 3); };
            check("jterms", 6, 12, x0, fd, fdual, frev, 1e-7);
        }
        // ---- mixed pack gather: inputs F[12] (E edge values), S[6] (B + B_tm1
        // face values), o[3] -> f[6], through the pack coefficients
        {
            double x0[21];
            for (int i = 0; i < 18; i++) x0[i] = U(-1, 1);
            for (int a = 0; a < 3; a++) x0[18 + a] = U(0.0, 1.0);
            auto pack = [](const auto *x, auto *pk) {
                for (int i = 0; i < 3; i++) {  // edge_coef of (F00, F10, F11, F01)
                    const auto f00 = x[4 * i], f10 = x[4 * i + 1], f11 = x[4 * i + 2], f01 = x[4 * i + 3];
                    pk[4 * i] = (4.0 * f00 - 2.0 * f01) + (f11 - 2.0 * f10);
                    pk[4 * i + 1] = (2.0 * f10 - 2.0 * f00) + (f01 - f11);
                    pk[4 * i + 2] = (2.0 * f01 - 2.0 * f00) + (f10 - f11);
                    pk[4 * i + 3] = (f00 - f10) + (f11 - f01);
                    const auto s0 = x[12 + 2 * i], s1 = x[12 + 2 * i + 1];
                    pk[12 + 2 * i] = s0 - 0.5 * s1;
                    pk[12 + 2 * i + 1] = 0.5 * (s1 - s0);
                }
            };
            auto fd = [&](const double *x, double *y) {
                double pk[18];
                pack(x, pk);
                gather_m_eval(pk, x + 18, y);
            };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual xx[21], pk[18], o[6];
                for (int i = 0; i < 21; i++) xx[i] = mk(x[i], d[i]);
                pack(xx, pk);
                gather_m_eval(pk, xx + 18, o);
                for (int i = 0; i < 6; i++) jd[i] = o[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                double pk[18], we[12], wb[6];
                pack(x, pk);
                gather_m_weights(x + 18, we, wb);
                for (int k = 0; k < 12; k++) jt[k] = we[k] * l[k >> 2];
                for (int k = 0; k < 6; k++) jt[12 + k] = wb[k] * l[3 + (k >> 1)];
                for (int a = 0; a < 3; a++) jt[18 + a] = 0.0;
                gather_m_rev_offsets(pk, x + 18, l, jt + 18);
            };
            check("mixed gather", 21, 6, x0, fd, fdual, frev, 1e-7);
        }
        // ---- mixed Vay: inputs f[6], u[3] -> u'[3], v'[3]
        {
            const double qp = U(-0.3, 0.3);
            double x0[9];
            for (int i = 0; i < 6; i++) x0[i] = U(-1, 1);
            for (int i = 6; i < 9; i++) x0[i] = U(-2, 2);
            auto fd = [&](const double *x, double *y) {
                double u[3] = {x[6], x[7], x[8]}, v[3];
                vay_u_eval(qp, x, u, v);
                for (int a = 0; a < 3; a++) { y[a] = u[a]; y[3 + a] = v[a]; }
            };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual f[6], u[3], v[3];
                for (int i = 0; i < 6; i++) f[i] = mk(x[i], d[i]);
                for (int a = 0; a < 3; a++) u[a] = mk(x[6 + a], d[6 + a]);
                vay_u_eval(qp, f, u, v);
                for (int a = 0; a < 3; a++) { jd[a] = u[a].d; jd[3 + a] = v[a].d; }
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                double lu[3] = {l[0], l[1], l[2]}, lv[3] = {l[3], l[4], l[5]}, lf[6] = {0, 0, 0, 0, 0, 0};
                vay_u_rev(qp, x, x + 6, lu, lv, lf);
                for (int i = 0; i < 6; i++) jt[i] = lf[i];
                for (int a = 0; a < 3; a++) jt[6 + a] = lu[a];
            };
            check("mixed vay", 9, 6, x0, fd, fdual, frev, 1e-7);
        }
        // ---- mixed J terms: inputs o[3], v[3] -> 12 contributions
        {
            const double qd = U(-2, 2);
            double x0[6];
            for (int a = 0; a < 3; a++) x0[a] = U(0.0, 1.0);
            for (int a = 3; a < 6; a++) x0[a] = U(-0.5, 0.5);
            auto fd = [&](const double *x, double *y) { jterms_m_eval(qd, x, x + 3, y); };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual o[3], vv[3], out[12];
                for (int a = 0; a < 3; a++) { o[a] = mk(x[a], d[a]); vv[a] = mk(x[3 + a], d[3 + a]); }
                jterms_m_eval(qd, o, vv, out);
                for (int i = 0; i < 12; i++) jd[i] = out[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                for (int i = 0; i < 6; i++) jt[i] = 0.0;
                jterms_m_rev(qd, x, x + 3, l, jt, jt + 3);
            };
            check("mixed jterms", 6, 12, x0, fd, fdual, frev, 1e-7);
        }
        // ---- Villasenor-Buneman current: inputs p0[3], p1[3] -> the weights of
        // up to 4 pieces (zero-padded); the ends stay clear of the cell faces so
        // the central difference sees the same pieces
        for (int sub = 0; sub < 4; sub++) {
            VbGeo vg;
            for (int a = 0; a < 3; a++) {
                vg.d[a] = c.d[a];
                vg.id[a] = 1.0 / c.d[a];
                vg.x0[a] = U(-2, 2);
            }
            const double coef = U(-2, 2);
            double x0[6];
            for (int a = 0; a < 3; a++) {
                const double u0 = std::floor(U(0, 8)) + U(0.05, 0.95);
                double u1 = u0 + U(-0.9, 0.9);
                while (u1 - std::floor(u1) < 0.05 || u1 - std::floor(u1) > 0.95) u1 = u0 + U(-0.9, 0.9);
                x0[a] = vg.x0[a] + u0 * vg.d[a];
                x0[3 + a] = vg.x0[a] + u1 * vg.d[a];
            }
            auto fd = [&](const double *x, double *y) {
                VbPiece<double> pc[4];
                for (int i = 0; i < 48; i++) y[i] = 0.0;
                const int n = vb_eval(vg, x, x + 3, coef, pc);
                for (int k = 0; k < n; k++)
                    for (int i = 0; i < 12; i++) y[12 * k + i] = pc[k].W[i];
            };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual a[3], b[3];
                VbPiece<Dual> pc[4];
                for (int i = 0; i < 3; i++) { a[i] = mk(x[i], d[i]); b[i] = mk(x[3 + i], d[3 + i]); }
                for (int i = 0; i < 48; i++) jd[i] = 0.0;
                const int n = vb_eval(vg, a, b, coef, pc);
                for (int k = 0; k < n; k++)
                    for (int i = 0; i < 12; i++) jd[12 * k + i] = pc[k].W[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                for (int i = 0; i < 6; i++) jt[i] = 0.0;
                auto lw = [&](int k, const int *, int a, int e) { return l[12 * k + 4 * a + e]; };
                vb_rev(vg, x, x + 3, coef, lw, jt, jt + 3);
            };
            check("vb current", 6, 48, x0, fd, fdual, frev, 1e-7);
        }
        // ---- the mixed form's piece terms: inputs ua[3], ub[3] -> 12 terms
        {
            const double qd = U(-2, 2), ddt[3] = {U(0.5, 3), U(0.5, 3), U(0.5, 3)};
            const int cs[3] = {-1, 0, 1};
            double x0[6];
            for (int a = 0; a < 3; a++) {
                x0[a] = U(-0.9, 1.9);
                x0[3 + a] = U(-0.9, 1.9);
            }
            auto fd = [&](const double *x, double *y) { vb_piece_m_eval(x, x + 3, qd, ddt, cs, y); };
            auto fdual = [&](const double *x, const double *d, double *jd) {
                Dual a[3], b[3], W[12];
                for (int i = 0; i < 3; i++) { a[i] = mk(x[i], d[i]); b[i] = mk(x[3 + i], d[3 + i]); }
                vb_piece_m_eval(a, b, qd, ddt, cs, W);
                for (int i = 0; i < 12; i++) jd[i] = W[i].d;
            };
            auto frev = [&](const double *x, const double *l, double *jt) {
                for (int i = 0; i < 6; i++) jt[i] = 0.0;
                vb_piece_m_rev(x, x + 3, qd, ddt, cs, l, jt, jt + 3);
            };
            check("mixed vb piece", 6, 12, x0, fd, fdual, frev, 1e-7);
        }
    }
    std::printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
    return failures ? 1 : 0;
}
