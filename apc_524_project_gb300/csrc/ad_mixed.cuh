// ad_mixed.cuh - per-particle arithmetic of the mixed-precision step in the
// form its adjoint needs, written once for the host check (double, Dual)
// and the device (float):
//   * the gather from the per-cell interpolation pack: each E component a
//     bilinear polynomial c0 + ct t + cr r + ctr t r of the two transverse
//     in-cell offsets, each B component d0 + d1 s of its own axis offset;
//     its field weights are the reference's (2 - o, o - 1) products
//     (src/grid/oGrid.cpp:153-197 with src/particles/interpolate.cpp:11-47);
//   * Vay's pusher on u = gamma v (src/pusher/relativisticBoris.cpp:53-140)
//     and Boris's (src/pusher/boris.cpp:33-85, ad_math.cuh's boris_rev);
//   * the 12 current terms in fixed-point units per in-cell offset
//     (src/particles/deposit.cpp:12-39 in cell units).
// The reverse functions take the forward inputs, recompute what they need
// and map output adjoints to input adjoints; decisions (cell, boundary
// events) are held at their primal values, as in ad_math.cuh.
#pragma once

#include "ad_math.cuh"

namespace emoo {
namespace ad {

AD_HD float sqrt_(float a) { return ::sqrtf(a); }

// 1 / x and 1 / sqrt(x): the hardware approximations for float on the device
// (relative error a few 2^-24, the mixed form's own accuracy), exact
// arithmetic for double and on the host.
AD_HD float rcp_(float x) {
#if defined(__CUDA_ARCH__)
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}
AD_HD float rsq_(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / ::sqrtf(x);
#endif
}
AD_HD double rcp_(double x) { return 1.0 / x; }
AD_HD double rsq_(double x) { return 1.0 / ::sqrt(x); }

// ---- gather from the pack ------------------------------------------------
//
// pk[18]: Ex (c0 ct cr ctr; t = y, r = z), Ey (t = z, r = x), Ez (t = x,
// r = y), then Bx (d0 d1), By (d0 d1), Bz (d0 d1). o: in-cell offsets.
template <class T, class P>
AD_HD void gather_m_eval(const P pk[18], const T o[3], T f[6]) {
    AD_UNROLL
    for (int i = 0; i < 3; i++) {
        const T &t = o[(i + 1) % 3], &r = o[(i + 2) % 3];
        f[i] = t * (r * pk[4 * i + 3] + pk[4 * i + 1]) + (r * pk[4 * i + 2] + pk[4 * i]);
        f[3 + i] = o[i] * pk[12 + 2 * i + 1] + pk[12 + 2 * i];
    }
}

// Adjoint with respect to the offsets: lo += (df/do)^T lf.
template <class R>
AD_HD void gather_m_rev_offsets(const R pk[18], const R o[3], const R lf[6], R lo[3]) {
    AD_UNROLL
    for (int i = 0; i < 3; i++) {
        const int jt = (i + 1) % 3, jr = (i + 2) % 3;
        lo[jt] += lf[i] * (pk[4 * i + 1] + pk[4 * i + 3] * o[jr]);
        lo[jr] += lf[i] * (pk[4 * i + 2] + pk[4 * i + 3] * o[jt]);
        lo[i] += lf[3 + i] * pk[12 + 2 * i + 1];
    }
}

// Field weights of the gather: E component i reads its 4 edge points
// (F00, F10, F11, F01 over (t, r)) with (a_t a_r, b_t a_r, b_t b_r, a_t b_r),
// B component i its 2 face points of B + B_tm1 with (a_i / 2, b_i / 2);
// a = 2 - o, b = o - 1 (the ghost-offset vertex), or with corr (the corrected
// policy's true vertex) a = 1 - o, b = o.
template <class R>
AD_HD void gather_m_weights(const R o[3], R we[12], R wb[6], bool corr = false) {
    R a[3], b[3];
    AD_UNROLL
    for (int k = 0; k < 3; k++) {
        a[k] = corr ? R(1) - o[k] : R(2) - o[k];
        b[k] = corr ? o[k] : o[k] - R(1);
    }
    AD_UNROLL
    for (int i = 0; i < 3; i++) {
        const int jt = (i + 1) % 3, jr = (i + 2) % 3;
        we[4 * i] = a[jt] * a[jr];
        we[4 * i + 1] = b[jt] * a[jr];
        we[4 * i + 2] = b[jt] * b[jr];
        we[4 * i + 3] = a[jt] * b[jr];
        wb[2 * i] = R(0.5) * a[i];
        wb[2 * i + 1] = R(0.5) * b[i];
    }
}

// ---- Vay on u = gamma v ----------------------------------------------------
//
// u: momentum per mass in (updated in place); v: the new velocity u' / gamma'.
template <class T>
AD_HD void vay_u_eval(double qp, const T f[6], T u[3], T v[3]) {
    const T g0 = sqrt_(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const T v0[3] = {u[0] / g0, u[1] / g0, u[2] / g0};
    const T bx = f[3], by = f[4], bz = f[5];
    const T vxb[3] = {v0[1] * bz - v0[2] * by, v0[2] * bx - v0[0] * bz, v0[0] * by - v0[1] * bx};
    T up[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) up[a] = u[a] + qp * (f[a] + vxb[a]) + qp * f[a];
    const T gps = 1.0 + up[0] * up[0] + up[1] * up[1] + up[2] * up[2];
    const T tau[3] = {qp * bx, qp * by, qp * bz};
    const T tau2 = tau[0] * tau[0] + tau[1] * tau[1] + tau[2] * tau[2];
    const T sigma = gps - tau2;
    const T ust = up[0] * tau[0] + up[1] * tau[1] + up[2] * tau[2];
    const T gi = sqrt_(0.5 * (sigma + sqrt_(sigma * sigma + 4.0 * (tau2 + ust * ust))));
    const T t[3] = {tau[0] / gi, tau[1] / gi, tau[2] / gi};
    const T s = 1.0 / (1.0 + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const T ud = ust / gi;
    const T c[3] = {up[1] * t[2] - up[2] * t[1], up[2] * t[0] - up[0] * t[2], up[0] * t[1] - up[1] * t[0]};
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        u[a] = s * (up[a] + ud * t[a] + c[a]);
        v[a] = u[a] / gi;
    }
}

// Adjoint of vay_u_eval at (f, u_in): lu holds the adjoint of u' on entry
// and of u_in on exit, lv the adjoint of v'; lf receives the field adjoint.
template <class R>
AD_HD void vay_u_rev(R qp, const R f[6], const R u_in[3], R lu[3], const R lv[3], R lf[6]) {
    const R e[3] = {f[0], f[1], f[2]}, b[3] = {f[3], f[4], f[5]};
    const R ig0 = rsq_(R(1) + u_in[0] * u_in[0] + u_in[1] * u_in[1] + u_in[2] * u_in[2]);  // 1 / gamma_in
    R v0[3], vxb[3], up[3], tau[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) v0[a] = u_in[a] * ig0;
    cross3t(v0, b, vxb);
    AD_UNROLL
    for (int a = 0; a < 3; a++) up[a] = u_in[a] + qp * (e[a] + vxb[a]) + qp * e[a];
    const R gps = R(1) + up[0] * up[0] + up[1] * up[1] + up[2] * up[2];
    AD_UNROLL
    for (int a = 0; a < 3; a++) tau[a] = qp * b[a];
    const R tau2 = tau[0] * tau[0] + tau[1] * tau[1] + tau[2] * tau[2];
    const R sigma = gps - tau2;
    const R ust = up[0] * tau[0] + up[1] * tau[1] + up[2] * tau[2];
    const R rad = sigma * sigma + R(4) * (tau2 + ust * ust);
    const R ig1 = rsq_(rad), g1 = rad * ig1;
    const R hg = R(0.5) * (sigma + g1);
    const R igi = rsq_(hg);  // 1 / gamma'
    R t[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) t[a] = tau[a] * igi;
    const R s = rcp_(R(1) + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const R ud = ust * igi;
    R c[3], w[3], uo[3];
    cross3t(up, t, c);
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        w[a] = up[a] + ud * t[a] + c[a];
        uo[a] = s * w[a];
    }
    // v' = u' / gi
    R luo[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) luo[a] = lu[a] + lv[a] * igi;
    R lgi = -(uo[0] * lv[0] + uo[1] * lv[1] + uo[2] * lv[2]) * (igi * igi);
    // u' = s w
    const R ls = w[0] * luo[0] + w[1] * luo[1] + w[2] * luo[2];
    R lw[3], lup[3], lt[3], tmp[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lw[a] = s * luo[a];
    // w = up + ud t + up x t
    AD_UNROLL
    for (int a = 0; a < 3; a++) lup[a] = lw[a];
    cross3t(t, lw, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lup[a] += tmp[a];
    const R lud = t[0] * lw[0] + t[1] * lw[1] + t[2] * lw[2];
    AD_UNROLL
    for (int a = 0; a < 3; a++) lt[a] = ud * lw[a];
    cross3t(lw, up, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lt[a] += tmp[a];
    // ud = ust / gi
    R lust = lud * igi;
    lgi += -ud * lud * igi;
    // s = 1 / (1 + t.t)
    AD_UNROLL
    for (int a = 0; a < 3; a++) lt[a] += R(-2) * s * s * ls * t[a];
    // t = tau / gi
    R ltau[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) ltau[a] = lt[a] * igi;
    lgi += -(t[0] * lt[0] + t[1] * lt[1] + t[2] * lt[2]) * igi;
    // gi = sqrt(0.5 (sigma + g1)), g1 = sqrt(sigma^2 + 4 tau2 + 4 ust^2)
    R lsigma = R(0.25) * lgi * igi;
    const R lg1 = R(0.25) * lgi * igi;
    lsigma += lg1 * sigma * ig1;
    R ltau2 = R(2) * lg1 * ig1;
    lust += R(4) * ust * lg1 * ig1;
    // ust = up . tau
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lup[a] += tau[a] * lust;
        ltau[a] += up[a] * lust;
    }
    // sigma = gps - tau2; tau2 = tau.tau; gps = 1 + up.up
    ltau2 -= lsigma;
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        ltau[a] += R(2) * tau[a] * ltau2;
        lup[a] += R(2) * up[a] * lsigma;
    }
    // up = u + qp (e + v0 x b) + qp e; tau = qp b
    R lvxb[3], lv0[3], lb[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lvxb[a] = qp * lup[a];
        lb[a] = qp * ltau[a];
        lf[a] += R(2) * qp * lup[a];
    }
    cross3t(b, lvxb, lv0);
    cross3t(lvxb, v0, tmp);
    AD_UNROLL
    for (int a = 0; a < 3; a++) lb[a] += tmp[a];
    // v0 = u / g0, g0 = sqrt(1 + u.u)
    const R uv = u_in[0] * lv0[0] + u_in[1] * lv0[1] + u_in[2] * lv0[2];
    const R ig03 = ig0 * ig0 * ig0;
    AD_UNROLL
    for (int a = 0; a < 3; a++) lu[a] = lup[a] + lv0[a] * ig0 - u_in[a] * uv * ig03;
    AD_UNROLL
    for (int a = 0; a < 3; a++) lf[3 + a] += lb[a];
}

// ---- current terms in fixed-point units ------------------------------------
//
// out[4 i .. 4 i + 3] = qd v_i (a_j a_k, b_j a_k, b_j b_k, a_j b_k), j = i + 1,
// k = i + 2 (mod 3), a = 2 - o, b = o - 1.
template <class T>
AD_HD void jterms_m_eval(double qd, const T o[3], const T v[3], T out[12]) {
    AD_UNROLL
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const T J = qd * v[i];
        const T aj = 2.0 - o[j], ak = 2.0 - o[k], bj = o[j] - 1.0, bk = o[k] - 1.0;
        out[4 * i] = J * aj * ak;
        out[4 * i + 1] = J * bj * ak;
        out[4 * i + 2] = J * bj * bk;
        out[4 * i + 3] = J * aj * bk;
    }
}

// Adjoint of jterms_m_eval: adds to lo[3] and lv[3].
template <class R>
AD_HD void jterms_m_rev(R qd, const R o[3], const R v[3], const R l[12], R lo[3], R lv[3]) {
    AD_UNROLL
    for (int i = 0; i < 3; i++) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        const R J = qd * v[i];
        const R aj = R(2) - o[j], ak = R(2) - o[k], bj = o[j] - R(1), bk = o[k] - R(1);
        const R l0 = l[4 * i], l1 = l[4 * i + 1], l2 = l[4 * i + 2], l3 = l[4 * i + 3];
        lv[i] += qd * (l0 * aj * ak + l1 * bj * ak + l2 * bj * bk + l3 * aj * bk);
        lo[j] += J * (-l0 * ak + l1 * ak + l2 * bk - l3 * bk);
        lo[k] += J * (-l0 * aj - l1 * bj + l2 * bj + l3 * aj);
    }
}

// ---- charge-conserving current, one straight piece (corrected policy) ------
//
// The twelve terms of a piece ua -> ub (old-cell units) lying in the cell
// shifted by c (per axis -1, 0 or 1, decided from the mid-point and held), as
// vb_piece in particles_mixed.cu: m = (ua + ub) / 2 - c, D = ub - ua, and for
// axis a with transverse axes j, k:
//   W[4a .. 4a+3] = qd D_a ddt_a ((1-m_j)(1-m_k) + cr, m_j (1-m_k) - cr,
//                                 m_j m_k + cr, (1-m_j) m_k - cr),
// cr = D_j D_k / 12.
template <class T, class R>
AD_HD void vb_piece_m_eval(const T ua[3], const T ub[3], R qd, const R ddt[3], const int c[3], T W[12]) {
    T m[3], D[3];
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        m[a] = R(0.5) * (ua[a] + ub[a]) - R(c[a]);
        D[a] = ub[a] - ua[a];
    }
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        const int jb = (a + 1) % 3, kb = (a + 2) % 3;
        const T wa = qd * D[a] * ddt[a];
        const T cr = D[jb] * D[kb] * R(1.0 / 12.0);
        W[4 * a + 0] = wa * ((R(1) - m[jb]) * (R(1) - m[kb]) + cr);
        W[4 * a + 1] = wa * (m[jb] * (R(1) - m[kb]) - cr);
        W[4 * a + 2] = wa * (m[jb] * m[kb] + cr);
        W[4 * a + 3] = wa * ((R(1) - m[jb]) * m[kb] - cr);
    }
}

// Adjoint of vb_piece_m_eval: l[12] the adjoints of the terms; adds the
// derivatives with respect to the piece's ends to lua and lub.
template <class R>
AD_HD void vb_piece_m_rev(const R ua[3], const R ub[3], R qd, const R ddt[3], const int c[3], const R l[12],
                          R lua[3], R lub[3]) {
    R m[3], D[3], lD[3] = {R(0), R(0), R(0)}, lm[3] = {R(0), R(0), R(0)};
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        m[a] = R(0.5) * (ua[a] + ub[a]) - R(c[a]);
        D[a] = ub[a] - ua[a];
    }
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        const int jb = (a + 1) % 3, kb = (a + 2) % 3;
        const R l0 = l[4 * a], l1 = l[4 * a + 1], l2 = l[4 * a + 2], l3 = l[4 * a + 3];
        const R wa = qd * D[a] * ddt[a];
        const R cr = D[jb] * D[kb] * R(1.0 / 12.0);
        const R mj = m[jb], mk = m[kb];
        const R lwa = l0 * ((R(1) - mj) * (R(1) - mk) + cr) + l1 * (mj * (R(1) - mk) - cr) + l2 * (mj * mk + cr) +
                      l3 * ((R(1) - mj) * mk - cr);
        const R lcr = wa * (l0 - l1 + l2 - l3);
        lm[jb] += wa * (-l0 * (R(1) - mk) + l1 * (R(1) - mk) + l2 * mk - l3 * mk);
        lm[kb] += wa * (-l0 * (R(1) - mj) - l1 * mj + l2 * mj + l3 * (R(1) - mj));
        lD[a] += qd * ddt[a] * lwa;
        lD[jb] += lcr * D[kb] * R(1.0 / 12.0);
        lD[kb] += lcr * D[jb] * R(1.0 / 12.0);
    }
    AD_UNROLL
    for (int a = 0; a < 3; a++) {
        lua[a] += -lD[a] + R(0.5) * lm[a];
        lub[a] += lD[a] + R(0.5) * lm[a];
    }
}

}  // namespace ad
}  // namespace emoo
