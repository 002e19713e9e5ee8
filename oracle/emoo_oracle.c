/*
 * emoo_oracle.c - CPU restatement (plain C, FP64, one thread) of the EMOOPIC
 * per-timestep PIC loop, used ONLY as the checker of the GPU library.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm load this library. The product never calls it.
 *
 * It restates the reference serial build's arithmetic in the same evaluation
 * order (compile with -ffp-contract=off so no multiply-add is fused), so that
 * on identical inputs it reproduces the reference bit for bit wherever the
 * reference's order of operations is defined. Each function cites the
 * reference file:line it follows (paths inside DenSto/APC_524_Project).
 *
 * It is pinned against the compiled reference (oracle/ref) through the golden
 * fixtures in tests/golden/.
 *
 * Reference behaviours reproduced on purpose (all verified against the
 * compiled reference):
 *  (a) the cell "vertex" handed to interpolation and deposition includes the
 *      ghost offset, so in-cell offsets lie in [-dx, 0) and the weights are
 *      linear extrapolations (src/grid/oGrid.cpp:160-162, 239-241);
 *  (b) Grid::addJ puts the 4th x-edge weight on Jx[i][j+1][k] instead of
 *      Jx[i][j][k+1] (src/grid/oGrid.cpp:101);
 *  (c) ghost planes are refreshed over the physical transverse range only,
 *      edge and corner ghost lines keep stale values (src/grid/spookyGrid.cpp:318-341);
 *  (d) the periodic J/rho fold moves only the two transverse J components and
 *      rho of the far ghost plane (src/grid/spookyGrid.cpp:21-26);
 *  (e) the gather uses B averaged over the two stored time levels
 *      (src/grid/oGrid.cpp:183-192);
 *  (f) evolveFields swaps the B / B_tm1 member pointers but not the field
 *      pointer table (src/grid/oGrid.cpp:18-20 vs src/grid/grid.cpp:321-342):
 *      ghost fills, getFieldPtr and the history read fixed storage slots, the
 *      Yee update, LightBC and the gather read the swapped roles;
 *  (g) Poisson_Solver::run_poisson_solver_ swaps its local pointer copies
 *      only, so phiToE / AToB always read phi1 / A1 (src/poisson/poisson.cpp:285);
 *  (h) AToB differences the same A component twice (src/poisson/convertFields.cpp:131-150);
 *  (i) periodic particle boundaries create ghost copies that later sides test
 *      again, and clearGhosts swaps each ghost with the vector's last element
 *      (src/boundaries/b_particles/bc_p_periodic.cpp:44-87,
 *      src/particles/particle_handler.cpp:271-284), which fixes the particle
 *      order and hence the current summation order.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/emoo.h"
/* The input generator of the CPU legs: the seeded per-particle sampler the
 * library compiles into its host and device loaders (the same inline code,
 * separately rounded basic operations only), so the CPU baseline and the
 * reference arm generate their particles without loading the product. */
#include "../apc_524_project_gb300/csrc/loader_common.h"

#define UNIT_ACC 0.58668774          /* src/globals.hpp:12 */
#define UNIT_RHOJ 4.80320427e-13     /* src/globals.hpp:16 */
#define PI_D 3.14159265358979323846  /* M_PI */
#define ITER_MAX 10000               /* src/poisson/poisson.cpp:14 */
#define CONV_CRIT 1e-12              /* src/poisson/poisson.cpp:12 */
#define CONV_RATIO 1e-9              /* src/poisson/poisson.cpp:13 */

enum { BC_PERIODIC = 0, BC_REFLECTING = 1, BC_ABSORBING = 2, BC_EXTERNAL = 3 };

typedef struct {
    int nw;
    double amp[EMOO_NWAVE], omg[EMOO_NWAVE], pha[EMOO_NWAVE], del[EMOO_NWAVE], iw[EMOO_NWAVE];
    int wid[EMOO_NWAVE]; /* input index of each wave */
} pulses_t;

typedef struct {
    emoo_input_info info;
    int n[3];    /* physical cells */
    int tot[3];  /* n + 3 points per dimension */
    long npts;
    double x0[3], L[3], d[3], id[3];
    double *slot[EMOO_NFIELDS]; /* storage slots, indexed like the reference fieldPtr_ */
    int bswap;                  /* 1 when the B / B_tm1 roles are exchanged (f) */
    int poisson;
    int pbc[6], fbc[6];
    pulses_t pulse[6][3]; /* LightBC: per side, per polarisation */
    double conv_phi, conv_A;
    /* particles */
    long np, cap;
    double *x, *y, *z, *vx, *vy, *vz, *g;
    double *fe1, *fe2, *fe3, *fb1, *fb2, *fb3;
    int *type;
    long *pid;
    short *ghost;
    double dt, t0;
    double t, dtp; /* the reference's globals time_phys and dt_phys */
    long next_hist;
    double rho_bg; /* immobile uniform background charge density (no reference counterpart) */
    int rho_bg_i0; /* first physical x index it covers */
    /* shaped injected waves (no reference counterpart): shape per wave, and
     * per side and E component the spot's factors along the plane's two
     * transverse axes (NULL: no spot) */
    emoo_wave_shape wshape[EMOO_NWAVE];
    int wshaped[EMOO_NWAVE];
    double *spot[6][3][2];
    /* 1: the corrected-physics policy (no reference counterpart; see
     * orc_set_policy), 0: the reference's arithmetic */
    int policy;
    /* field start solver: 0 the reference's Jacobi, 1 the exact discrete
     * solution (see orc_set_poisson_solver) */
    int poisson_solver;
    double poisson_rtol;
} orc_t;

/* ------------------------------------------------------------------ */
/* helpers                                                              */

static inline long IDX(const orc_t *c, int i, int j, int k) {
    return ((long)i * c->tot[1] + j) * c->tot[2] + k;
}

/* Member-role pointers (Ex_, Bx_, Bx_tm1_ ...) versus the fixed slots. */
static double *role_B(orc_t *c, int comp) { return c->bswap ? c->slot[EMOO_BX_TM1 + comp] : c->slot[EMOO_BX + comp]; }
static double *role_Btm1(orc_t *c, int comp) { return c->bswap ? c->slot[EMOO_BX + comp] : c->slot[EMOO_BX_TM1 + comp]; }

static int bc_code(const char *s, int field) {
    if (strcmp(s, "periodic") == 0) return BC_PERIODIC;
    if (field) return strcmp(s, "external") == 0 ? BC_EXTERNAL : -1;
    if (strcmp(s, "reflecting") == 0) return BC_REFLECTING;
    if (strcmp(s, "absorbing") == 0) return BC_ABSORBING;
    return -1;
}

static int grow(orc_t *c, long need) {
    if (need <= c->cap) return 0;
    long nc = c->cap ? c->cap : 1024;
    while (nc < need) nc *= 2;
#define RE(p, T)                                      \
    do {                                              \
        void *q = realloc(c->p, sizeof(T) * (size_t)nc); \
        if (!q) return -1;                            \
        c->p = (T *)q;                                \
    } while (0)
    RE(x, double); RE(y, double); RE(z, double);
    RE(vx, double); RE(vy, double); RE(vz, double); RE(g, double);
    RE(fe1, double); RE(fe2, double); RE(fe3, double);
    RE(fb1, double); RE(fb2, double); RE(fb3, double);
    RE(type, int); RE(pid, long); RE(ghost, short);
#undef RE
    c->cap = nc;
    return 0;
}

static void copy_particle(orc_t *c, long dst, long src) {
    c->x[dst] = c->x[src]; c->y[dst] = c->y[src]; c->z[dst] = c->z[src];
    c->vx[dst] = c->vx[src]; c->vy[dst] = c->vy[src]; c->vz[dst] = c->vz[src];
    c->g[dst] = c->g[src];
    c->fe1[dst] = c->fe1[src]; c->fe2[dst] = c->fe2[src]; c->fe3[dst] = c->fe3[src];
    c->fb1[dst] = c->fb1[src]; c->fb2[dst] = c->fb2[src]; c->fb3[dst] = c->fb3[src];
    c->type[dst] = c->type[src]; c->pid[dst] = c->pid[src]; c->ghost[dst] = c->ghost[src];
}

static void swap_particle(orc_t *c, long a, long b) {
#define SW(p, T) do { T t_ = c->p[a]; c->p[a] = c->p[b]; c->p[b] = t_; } while (0)
    SW(x, double); SW(y, double); SW(z, double);
    SW(vx, double); SW(vy, double); SW(vz, double); SW(g, double);
    SW(fe1, double); SW(fe2, double); SW(fe3, double);
    SW(fb1, double); SW(fb2, double); SW(fb3, double);
    SW(type, int); SW(pid, long); SW(ghost, short);
#undef SW
}

static double *pos_of(orc_t *c, int d) { return d == 0 ? c->x : (d == 1 ? c->y : c->z); }
static double *vel_of(orc_t *c, int d) { return d == 0 ? c->vx : (d == 1 ? c->vy : c->vz); }

/* ------------------------------------------------------------------ */
/* construction                                                         */

/* LightBC constructor: waves registered per side and E polarisation in input
 * order (src/grid/lightBC.cpp:22-68). */
static void setup_pulses(orc_t *c) {
    const emoo_input_info *in = &c->info;
    for (int s = 0; s < 6; s++) {
        int side = (s % 2 == 0) ? -(s / 2 + 1) : (s / 2 + 1);
        for (int p = 0; p < 3; p++) c->pulse[s][p].nw = 0;
        for (int w = 0; w < in->nwaves; w++) {
            if (in->inSide[w] != side) continue;
            int pid = in->inPolE[w] - 1;
            if (pid < 0 || pid > 2) continue;
            pulses_t *P = &c->pulse[s][pid];
            P->amp[P->nw] = in->peakamps[w];
            P->omg[P->nw] = in->omegas[w];
            P->pha[P->nw] = in->phases[w];
            P->del[P->nw] = in->delays[w];
            P->iw[P->nw] = in->invWidths[w];
            P->wid[P->nw] = w;
            P->nw++;
        }
    }
}

void *orc_create(const emoo_input_info *in, double dt, double t0) {
    orc_t *c = (orc_t *)calloc(1, sizeof(orc_t));
    if (!c) return NULL;
    c->info = *in;
    for (int d = 0; d < 3; d++) {
        c->n[d] = in->nCell[d];
        c->tot[d] = in->nCell[d] + 3;
        c->x0[d] = in->xyz0[d];
        c->L[d] = in->Lxyz[d];
        c->d[d] = in->Lxyz[d] / in->nCell[d]; /* src/grid/grid.cpp:37-42 */
        c->id[d] = 1.0 / c->d[d];
    }
    c->npts = (long)c->tot[0] * c->tot[1] * c->tot[2];
    for (int f = 0; f < EMOO_NFIELDS; f++) {
        c->slot[f] = (double *)calloc((size_t)c->npts, sizeof(double));
        if (!c->slot[f]) return NULL;
    }
    c->poisson = (in->restart == 0 && strcmp(in->fields_init, "poisson") == 0);
    for (int s = 0; s < 6; s++) {
        c->pbc[s] = bc_code(in->parts_bound[s], 0);
        c->fbc[s] = bc_code(in->fields_bound[s], 1);
        if (c->pbc[s] < 0 || c->fbc[s] < 0) {
            fprintf(stderr, "oracle: unknown boundary on side %d\n", s);
            return NULL;
        }
    }
    setup_pulses(c);
    /* src/poisson/poisson.cpp:135-154 */
    double vmax = in->bound_phi[0], vmin = in->bound_phi[0];
    for (int i = 0; i < 6; i++) {
        if (in->bound_phi[i] > vmax) vmax = in->bound_phi[i];
        if (in->bound_phi[i] < vmin) vmin = in->bound_phi[i];
    }
    c->conv_phi = vmax - vmin;
    vmax = vmin = in->bound_Ax[0];
    for (int i = 0; i < 6; i++) {
        double a[3] = {in->bound_Ax[i], in->bound_Ay[i], in->bound_Az[i]};
        for (int q = 0; q < 3; q++) {
            if (a[q] > vmax) vmax = a[q];
            if (a[q] < vmin) vmin = a[q];
        }
    }
    c->conv_A = vmax - vmin;
    c->dt = dt;
    c->t0 = t0;
    c->t = 0.0;
    c->dtp = 0.0;
    c->next_hist = 0;
    return c;
}

void orc_destroy(void *h) {
    orc_t *c = (orc_t *)h;
    if (!c) return;
    for (int f = 0; f < EMOO_NFIELDS; f++) free(c->slot[f]);
    free(c->x); free(c->y); free(c->z); free(c->vx); free(c->vy); free(c->vz); free(c->g);
    free(c->fe1); free(c->fe2); free(c->fe3); free(c->fb1); free(c->fb2); free(c->fb3);
    free(c->type); free(c->pid); free(c->ghost);
    for (int s = 0; s < 6; s++)
        for (int p = 0; p < 3; p++) { free(c->spot[s][p][0]); free(c->spot[s][p][1]); }
    free(c);
}

long orc_npoints(void *h) { return ((orc_t *)h)->npts; }

int orc_add_particles(void *h, long n, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, const double *gamma,
                      const int *type, const long *id) {
    orc_t *c = (orc_t *)h;
    if (grow(c, c->np + n)) return -2;
    for (long i = 0; i < n; i++) {
        long p = c->np + i;
        c->x[p] = x[i]; c->y[p] = y[i]; c->z[p] = z[i];
        c->vx[p] = vx[i]; c->vy[p] = vy[i]; c->vz[p] = vz[i];
        c->g[p] = gamma ? gamma[i] : 0.0;
        c->fe1[p] = c->fe2[p] = c->fe3[p] = c->fb1[p] = c->fb2[p] = c->fb3[p] = 0.0;
        c->type[p] = type[i];
        c->pid[p] = id ? id[i] : p;
        c->ghost[p] = 0;
    }
    c->np += n;
    return 0;
}

long orc_num_particles(void *h) { return ((orc_t *)h)->np; }

int orc_get_particles(void *h, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                      double *gamma, int *type, long *id) {
    orc_t *c = (orc_t *)h;
    for (long i = 0; i < c->np; i++) {
        x[i] = c->x[i]; y[i] = c->y[i]; z[i] = c->z[i];
        vx[i] = c->vx[i]; vy[i] = c->vy[i]; vz[i] = c->vz[i];
        gamma[i] = c->g[i]; type[i] = c->type[i]; id[i] = c->pid[i];
    }
    return 0;
}

int orc_get_particle_fields(void *h, double *e1, double *e2, double *e3, double *b1, double *b2, double *b3) {
    orc_t *c = (orc_t *)h;
    for (long i = 0; i < c->np; i++) {
        e1[i] = c->fe1[i]; e2[i] = c->fe2[i]; e3[i] = c->fe3[i];
        b1[i] = c->fb1[i]; b2[i] = c->fb2[i]; b3[i] = c->fb3[i];
    }
    return 0;
}

/* getFieldPtr()[id] semantics: fixed storage slots (f). */
int orc_get_field(void *h, int id, double *out) {
    orc_t *c = (orc_t *)h;
    if (id < 0 || id >= EMOO_NFIELDS) return -1;
    memcpy(out, c->slot[id], sizeof(double) * (size_t)c->npts);
    return 0;
}

int orc_set_field(void *h, int id, const double *in) {
    orc_t *c = (orc_t *)h;
    if (id < 0 || id >= EMOO_NFIELDS) return -1;
    memcpy(c->slot[id], in, sizeof(double) * (size_t)c->npts);
    return 0;
}

/* Grid::getCellID, src/grid/oGrid.cpp:208-227 (C truncation, ghost offset +1,
 * linear index over the (n+2)^3 cell array). */
static inline int cell_id(const orc_t *c, double x, double y, double z, int *ix, int *iy, int *iz) {
    int i = (int)((x - c->x0[0]) * c->id[0]) + 1;
    int j = (int)((y - c->x0[1]) * c->id[1]) + 1;
    int k = (int)((z - c->x0[2]) * c->id[2]) + 1;
    if (ix) { *ix = i; *iy = j; *iz = k; }
    int ny = c->n[1] + 2, nz = c->n[2] + 2;
    return (ny * nz) * i + nz * j + k;
}

int orc_cell_id(void *h, double x, double y, double z) { return cell_id((orc_t *)h, x, y, z, NULL, NULL, NULL); }

/* cellID -> (ix,iy,iz), src/grid/oGrid.cpp:155-157 */
static inline void cell_split(const orc_t *c, int cid, int *ix, int *iy, int *iz) {
    int ny = c->n[1] + 2, nz = c->n[2] + 2;
    int k = cid % nz;
    int j = ((cid - k) / nz) % ny;
    int i = (((cid - k) / nz) - j) / ny;
    *ix = i; *iy = j; *iz = k;
}

/* ------------------------------------------------------------------ */
/* field boundaries                                                     */

/* Plane copy / sum over the physical transverse range [1,n]x[1,n]
 * (sliceMatToVec_ / unsliceMatToVec_, src/grid/spookyGrid.cpp:286-425). */
static void plane_op(orc_t *c, double *f, int dim, int src, int dst, int sum) {
    int o1 = (dim == 0) ? 1 : 0; /* outer transverse dim */
    int o2 = (dim == 2) ? 1 : 2; /* inner transverse dim */
    for (int p = 1; p <= c->n[o1]; p++) {
        for (int q = 1; q <= c->n[o2]; q++) {
            int is[3], id_[3];
            is[dim] = src; id_[dim] = dst;
            is[o1] = id_[o1] = p;
            is[o2] = id_[o2] = q;
            long s = IDX(c, is[0], is[1], is[2]);
            long t = IDX(c, id_[0], id_[1], id_[2]);
            if (sum) f[t] += f[s];
            else f[t] = f[s];
        }
    }
}

/* setFieldInPlane, src/grid/oGrid.cpp:446-476 (whole plane incl. ghosts). */
static void plane_set(orc_t *c, double *f, int dim, int idx, double v) {
    int o1 = (dim == 0) ? 1 : 0;
    int o2 = (dim == 2) ? 1 : 2;
    for (int p = 0; p < c->tot[o1]; p++)
        for (int q = 0; q < c->tot[o2]; q++) {
            int ii[3];
            ii[dim] = idx; ii[o1] = p; ii[o2] = q;
            f[IDX(c, ii[0], ii[1], ii[2])] = v;
        }
}

/* Sine-series envelope of a shaped wave (no reference counterpart):
 * sum_k coef[k-1] sin(k pi a), a = (t - t_start) / window, inside the window,
 * 0 outside. */
static double sine_envelope(const emoo_wave_shape *sh, double t) {
    if (!(t >= sh->t_start && t <= sh->t_start + sh->window)) return 0.0;
    double a = (t - sh->t_start) / sh->window;
    double e = 0.0;
    for (int k = 1; k <= sh->ncoef; k++) e += sh->coef[k - 1] * sin(k * PI_D * a);
    return e;
}

/* GaussianPulses, src/utils/evaluateGaussianPulse.cpp:7-30. A shaped wave
 * takes its sine-series envelope in place of the Gaussian; terms of waves
 * with a transverse spot go to *spot, the rest to the return value. */
static double gaussian_pulses(const orc_t *c, double t, double dt, const pulses_t *P, double *spot) {
    double val = 0.0, sv = 0.0;
    for (int i = 0; i < P->nw; i++) {
        const emoo_wave_shape *sh = c->wshaped[P->wid[i]] ? &c->wshape[P->wid[i]] : NULL;
        double tmp = P->amp[i] * cos(P->omg[i] * (t + dt) + P->pha[i] * PI_D / 180.0);
        double env = (sh && sh->ncoef > 0) ? sine_envelope(sh, t) : exp(-pow((t - P->del[i]) * P->iw[i], 2));
        if (sh && sh->waist > 0) sv += tmp * env;
        else val += tmp * env;
    }
    *spot = sv;
    return val;
}

/* Plane set with a transverse spot: v + (vs t1[p]) t2[q]. */
static void plane_set_spot(orc_t *c, double *f, int dim, int idx, double v, double vs, const double *t1,
                           const double *t2) {
    if (!t1) { plane_set(c, f, dim, idx, v); return; }
    int o1 = (dim == 0) ? 1 : 0;
    int o2 = (dim == 2) ? 1 : 2;
    for (int p = 0; p < c->tot[o1]; p++)
        for (int q = 0; q < c->tot[o2]; q++) {
            int ii[3];
            ii[dim] = idx; ii[o1] = p; ii[o2] = q;
            f[IDX(c, ii[0], ii[1], ii[2])] = v + vs * t1[p] * t2[q];
        }
}

/* Shape of wave w (NULL: plain). Spots of one side and E component must
 * share waist and centre (else -1 and nothing changes). The spot factor
 * along transverse axis a of the plane at grid index j is
 * exp(-(r r)), r = (xyz0 + (j - 1 + h) d - center) / waist, h = 1/2 along
 * the wave's E polarisation, 0 across it. */
int orc_set_wave_shape(void *h, int w, const emoo_wave_shape *sh) {
    orc_t *c = (orc_t *)h;
    if (w < 0 || w >= c->info.nwaves || w >= EMOO_NWAVE) return -1;
    emoo_wave_shape old = c->wshape[w];
    int old_on = c->wshaped[w];
    if (sh) { c->wshape[w] = *sh; c->wshaped[w] = 1; }
    else { memset(&c->wshape[w], 0, sizeof(emoo_wave_shape)); c->wshaped[w] = 0; }
    int owner[6][3];
    for (int s = 0; s < 6; s++) for (int p = 0; p < 3; p++) owner[s][p] = -1;
    for (int v = 0; v < c->info.nwaves && v < EMOO_NWAVE; v++) {
        if (!c->wshaped[v] || !(c->wshape[v].waist > 0)) continue;
        int side = c->info.inSide[v], p = c->info.inPolE[v] - 1;
        if (side == 0 || side < -3 || side > 3 || p < 0 || p > 2) continue;
        int s = 2 * (abs(side) - 1) + (side > 0 ? 1 : 0);
        int o = owner[s][p];
        if (o >= 0) {
            const emoo_wave_shape *a = &c->wshape[o], *b = &c->wshape[v];
            if (a->waist != b->waist || a->center[0] != b->center[0] || a->center[1] != b->center[1]) {
                c->wshape[w] = old;
                c->wshaped[w] = old_on;
                return -1;
            }
        } else {
            owner[s][p] = v;
        }
    }
    for (int s = 0; s < 6; s++) {
        int d = s / 2, ax[2] = {(d == 0) ? 1 : 0, (d == 2) ? 1 : 2};
        for (int p = 0; p < 3; p++)
            for (int a = 0; a < 2; a++) {
                free(c->spot[s][p][a]);
                c->spot[s][p][a] = NULL;
                if (owner[s][p] < 0) continue;
                const emoo_wave_shape *ws = &c->wshape[owner[s][p]];
                int n = c->tot[ax[a]];
                double hh = ax[a] == p ? 0.5 : 0.0;
                double *t = (double *)malloc(sizeof(double) * n);
                for (int j = 0; j < n; j++) {
                    double pos = c->x0[ax[a]] + (j - 1 + hh) * c->d[ax[a]];
                    double r = (pos - ws->center[a]) / ws->waist;
                    t[j] = exp(-(r * r));
                }
                c->spot[s][p][a] = t;
            }
    }
    return 0;
}

/* setFieldAlongEdge plane index, src/grid/oGrid.cpp:291-431: left = first
 * physical (1); right = n for an E component along dim or a B component
 * across it, n+1 otherwise. */
static int edge_plane(const orc_t *c, int isB, int comp, int dim, int right) {
    if (!right) return 1;
    int along = (comp == dim);
    if (!isB) return along ? c->n[dim] : c->n[dim] + 1;
    return along ? c->n[dim] + 1 : c->n[dim];
}

/* LightBC::applyBCs, src/grid/lightBC.cpp:165-200. Uses the member roles (f). */
static void light_bc(orc_t *c, int s, double t, double dt) {
    int dim = s / 2, right = s % 2, sign = right ? 1 : -1;
    static const int EPOL[3][3] = {{1, 2, 0}, {2, 0, 1}, {0, 1, 2}};
    static const int BPOL[3][3] = {{2, 1, 0}, {0, 2, 1}, {1, 0, 2}};
    double E1[3], B1[3];
    for (int i = 0; i < 3; i++) {
        E1[i] = c->info.E0[i];
        B1[i] = c->info.B0[i];
    }
    double dx = c->d[dim];
    double bphase = (dx + sign * dt) / 2;
    for (int i = 0; i < 3; i++) {
        int eid = EPOL[dim][i], bid = BPOL[dim][i];
        double es = 0.0, bs = 0.0;
        if (c->pulse[s][eid].nw > 0 && eid != dim) {
            double ev = gaussian_pulses(c, t, 0.0, &c->pulse[s][eid], &es);
            E1[eid] += ev;
            int bsign = sign * (int)pow(-1, i + 1);
            double bsp;
            double bv = bsign * gaussian_pulses(c, t, bphase, &c->pulse[s][eid], &bsp);
            B1[bid] += bv;
            bs = bsign * bsp;
        }
        /* the B component paired with E component eid sits at the same
         * transverse offsets: both take the spot of (s, eid) */
        const double *t1 = eid != dim ? c->spot[s][eid][0] : NULL;
        const double *t2 = eid != dim ? c->spot[s][eid][1] : NULL;
        plane_set_spot(c, c->slot[EMOO_EX + eid], dim, edge_plane(c, 0, eid, dim, right), E1[eid], es, t1, t2);
        plane_set_spot(c, role_B(c, bid), dim, edge_plane(c, 1, bid, dim, right), B1[bid], bs, t1, t2);
    }
}

/* PoissonBC::applyBCs, src/poisson/poissonBC.cpp:164-234: Dirichlet value on
 * the first physical (left) or the ghost (right) plane. */
static void poisson_bc(orc_t *c, int s, int id) {
    int dim = s / 2, right = s % 2;
    int fid;
    if (id == EMOO_PHI1 || id == EMOO_PHI2) fid = 0;
    else if (id == EMOO_AX1 || id == EMOO_AX2) fid = 1;
    else if (id == EMOO_AY1 || id == EMOO_AY2) fid = 2;
    else if (id == EMOO_AZ1 || id == EMOO_AZ2) fid = 3;
    else return;
    double v = fid == 0 ? c->info.bound_phi[s] : fid == 1 ? c->info.bound_Ax[s]
                        : fid == 2 ? c->info.bound_Ay[s] : c->info.bound_Az[s];
    int off = right ? 1 + c->n[dim] : 1;
    plane_set(c, c->slot[id], dim, off, v);
}

/* Grid::executeBC(sendID), src/grid/grid.cpp:577-585, dispatching to
 * BC_F_Periodic::completeBC (src/boundaries/b_fields/bc_f_periodic.cpp:34-57)
 * and BC_F_External::completeBC (src/boundaries/b_fields/bc_f_external.cpp:45-58). */
static void full_plane(orc_t *c, double *f, int dim, int src, int dst, int sum);
static void corrected_fold(orc_t *c);
static void corrected_ghosts(orc_t *c);
static void corrected_e_bounds(orc_t *c);

int orc_execute_bc(void *h, int send_id) {
    orc_t *c = (orc_t *)h;
    if (c->policy && send_id == EMOO_SEND_JRHO) {
        corrected_fold(c);
        return 0;
    }
    if (c->policy && send_id == EMOO_SEND_EB) {
        corrected_ghosts(c);
        return 0;
    }
    for (int dim = 0; dim < 3; dim++) {
        for (int r = 0; r < 2; r++) {
            int s = 2 * dim + r;
            int n = c->n[dim];
            if (c->fbc[s] == BC_PERIODIC) {
                if (send_id == EMOO_SEND_JRHO) {
                    if (r == 0) {
                        /* far ghost plane n+1 summed into first physical plane 1 */
                        int f0 = (dim == 0) ? EMOO_JY : EMOO_JX;
                        int f1 = (dim == 2) ? EMOO_JY : EMOO_JZ;
                        plane_op(c, c->slot[f0], dim, n + 1, 1, 1);
                        plane_op(c, c->slot[f1], dim, n + 1, 1, 1);
                        plane_op(c, c->slot[EMOO_RHO], dim, n + 1, 1, 1);
                    }
                } else {
                    int src = r == 0 ? n : 1, dst = r == 0 ? 0 : n + 1;
                    if (send_id == EMOO_SEND_EB) {
                        for (int f = EMOO_EX; f <= EMOO_BZ; f++) plane_op(c, c->slot[f], dim, src, dst, 0);
                    } else {
                        plane_op(c, c->slot[send_id], dim, src, dst, 0);
                    }
                }
            } else { /* external */
                if (send_id == EMOO_SEND_EB) light_bc(c, s, c->t, c->dtp);
                else if (c->poisson && send_id > 0) poisson_bc(c, s, send_id);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* particles                                                            */

/* Grid::getFieldInterpolatorVec (src/grid/oGrid.cpp:153-197) followed by
 * Interpolator::interpolate_fields (src/particles/interpolate.cpp:11-47). */
static void gather(orc_t *c, double px, double py, double pz, double out[6]) {
    int ix, iy, iz;
    int cid = cell_id(c, px, py, pz, NULL, NULL, NULL);
    cell_split(c, cid, &ix, &iy, &iz);
    double v[21];
    /* the reference's ghost-offset vertex (a); the corrected policy's is the
     * cell's own lower corner, grid point i at x0 + (i - 1) d */
    const int vs = c->policy;
    v[0] = c->x0[0] + c->d[0] * (ix - vs);
    v[1] = c->x0[1] + c->d[1] * (iy - vs);
    v[2] = c->x0[2] + c->d[2] * (iz - vs);
    const double *Ex = c->slot[EMOO_EX], *Ey = c->slot[EMOO_EY], *Ez = c->slot[EMOO_EZ];
    v[3] = Ex[IDX(c, ix, iy, iz)];
    v[4] = Ex[IDX(c, ix, iy + 1, iz)];
    v[5] = Ex[IDX(c, ix, iy + 1, iz + 1)];
    v[6] = Ex[IDX(c, ix, iy, iz + 1)];
    v[7] = Ey[IDX(c, ix, iy, iz)];
    v[8] = Ey[IDX(c, ix, iy, iz + 1)];
    v[9] = Ey[IDX(c, ix + 1, iy, iz + 1)];
    v[10] = Ey[IDX(c, ix + 1, iy, iz)];
    v[11] = Ez[IDX(c, ix, iy, iz)];
    v[12] = Ez[IDX(c, ix + 1, iy, iz)];
    v[13] = Ez[IDX(c, ix + 1, iy + 1, iz)];
    v[14] = Ez[IDX(c, ix, iy + 1, iz)];
    const double *Bx = role_B(c, 0), *By = role_B(c, 1), *Bz = role_B(c, 2);
    const double *Tx = role_Btm1(c, 0), *Ty = role_Btm1(c, 1), *Tz = role_Btm1(c, 2);
    v[15] = (Tx[IDX(c, ix, iy, iz)] + Bx[IDX(c, ix, iy, iz)]) / 2;
    v[16] = (Tx[IDX(c, ix + 1, iy, iz)] + Bx[IDX(c, ix + 1, iy, iz)]) / 2;
    v[17] = (Ty[IDX(c, ix, iy, iz)] + By[IDX(c, ix, iy, iz)]) / 2;
    v[18] = (Ty[IDX(c, ix, iy + 1, iz)] + By[IDX(c, ix, iy + 1, iz)]) / 2;
    v[19] = (Tz[IDX(c, ix, iy, iz)] + Bz[IDX(c, ix, iy, iz)]) / 2;
    v[20] = (Tz[IDX(c, ix, iy, iz + 1)] + Bz[IDX(c, ix, iy, iz + 1)]) / 2;
    double pos[3] = {px, py, pz}, ds[3];
    const double *l = c->d;
    for (int i = 0; i < 3; i++) ds[i] = pos[i] - v[i];
    for (int i = 0; i < 3; i++) {
        int j = (i + 1) % 3, k = (i + 2) % 3;
        double e = 0;
        e += (l[j] - ds[j]) * (l[k] - ds[k]) * v[3 + 4 * i];
        e += ds[j] * (l[k] - ds[k]) * v[3 + 4 * i + 1];
        e += ds[j] * ds[k] * v[3 + 4 * i + 2];
        e += (l[j] - ds[j]) * ds[k] * v[3 + 4 * i + 3];
        e /= l[j] * l[k];
        double b = 0;
        b += (l[i] - ds[i]) * v[3 + 12 + 2 * i];
        b += ds[i] * v[3 + 12 + 2 * i + 1];
        b /= l[i];
        out[i] = e;
        out[3 + i] = b;
    }
}

int orc_interpolate(void *h) {
    orc_t *c = (orc_t *)h;
    for (long p = 0; p < c->np; p++) {
        double f[6];
        gather(c, c->x[p], c->y[p], c->z[p], f);
        c->fe1[p] = f[0]; c->fe2[p] = f[1]; c->fe3[p] = f[2];
        c->fb1[p] = f[3]; c->fb2[p] = f[4]; c->fb3[p] = f[5];
    }
    return 0;
}

/* Boris::Step, src/pusher/boris.cpp:12-111. st = {x,y,z,vx,vy,vz,gamma}. */
static void boris(double *st, double q, double m, const double *f, double dt) {
    double x = st[0], y = st[1], z = st[2], vx = st[3], vy = st[4], vz = st[5];
    double q_p = (0.5 * dt * q) / m;
    q_p *= UNIT_ACC;
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
    double vxn = v_px + q_p * ex, vyn = v_py + q_p * ey, vzn = v_pz + q_p * ez;
    st[0] = x + dt * vxn;
    st[1] = y + dt * vyn;
    st[2] = z + dt * vzn;
    st[3] = vxn; st[4] = vyn; st[5] = vzn;
}

/* Relativistic_Boris::Step (Vay 2008), src/pusher/relativisticBoris.cpp:28-143. */
static void vay(double *st, double q, double m, const double *f, double dt) {
    double x = st[0], y = st[1], z = st[2], vx = st[3], vy = st[4], vz = st[5], gamma = st[6];
    double q_p = (0.5 * dt * q) / m;
    q_p *= UNIT_ACC;
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
    double gamma_int = sqrt(sigma * sigma + 4 * (tau_sq + ustar * ustar));
    gamma_int = sqrt(0.5 * (sigma + gamma_int));
    double tx = taux / gamma_int, ty = tauy / gamma_int, tz = tauz / gamma_int;
    double s = 1.0 / (1.0 + tx * tx + ty * ty + tz * tz);
    double udott = ustar / gamma_int;
    double upXt_x = upy * tz - upz * ty, upXt_y = upz * tx - upx * tz, upXt_z = upx * ty - upy * tx;
    double uint_x = s * (upx + udott * tx + upXt_x);
    double uint_y = s * (upy + udott * ty + upXt_y);
    double uint_z = s * (upz + udott * tz + upXt_z);
    double vxn = uint_x / gamma_int, vyn = uint_y / gamma_int, vzn = uint_z / gamma_int;
    st[0] = x + dt * vxn;
    st[1] = y + dt * vyn;
    st[2] = z + dt * vzn;
    st[3] = vxn; st[4] = vyn; st[5] = vzn;
    st[6] = gamma_int;
}

int orc_pusher_steps(int relativistic, double *state, const double *field, double dt, long nsteps) {
    for (long s = 0; s < nsteps; s++) {
        if (relativistic) vay(state, state[7], state[8], field, dt);
        else boris(state, state[7], state[8], field, dt);
    }
    return 0;
}

/* Particle_Handler::Push, src/particles/particle_handler.cpp:124-128 */
static void push_all(orc_t *c, double dt) {
    for (long p = 0; p < c->np; p++) {
        int s = c->type[p];
        double st[7] = {c->x[p], c->y[p], c->z[p], c->vx[p], c->vy[p], c->vz[p], c->g[p]};
        double f[6] = {c->fe1[p], c->fe2[p], c->fe3[p], c->fb1[p], c->fb2[p], c->fb3[p]};
        if (c->info.relativity == 0) boris(st, c->info.charge_ratio[s], c->info.mass_ratio[s], f, dt);
        else vay(st, c->info.charge_ratio[s], c->info.mass_ratio[s], f, dt);
        c->x[p] = st[0]; c->y[p] = st[1]; c->z[p] = st[2];
        c->vx[p] = st[3]; c->vy[p] = st[4]; c->vz[p] = st[5]; c->g[p] = st[6];
    }
}

int orc_push(void *h) {
    orc_t *c = (orc_t *)h;
    push_all(c, c->dt);
    return 0;
}

/* executeParticleBoundaryConditions, src/particles/particle_handler.cpp:287-295:
 * six sides in order; periodic sides append ghost copies that later sides see
 * (bc_p_periodic.cpp:44-87), reflecting sides fold in place
 * (bc_p_reflecting.cpp:43-52), absorbing sides (no reference counterpart)
 * only mark the particle for removal. */
int orc_particle_bc(void *h, long *counts6) {
    orc_t *c = (orc_t *)h;
    for (int s = 0; s < 6; s++) {
        int d = s / 2, right = s % 2;
        double xmin = c->x0[d], xmax = xmin + c->L[d];
        long cnt = 0;
        if (c->pbc[s] == BC_PERIODIC) {
            long cur = c->np, nb = 0;
            for (long p = 0; p < cur; p++) {
                if (c->ghost[p]) continue;
                double xp = pos_of(c, d)[p];
                int hit = (!right && xp < xmin) || (right && xp > xmax);
                if (!hit) continue;
                if (grow(c, cur + nb + 1)) return -2;
                long q = cur + nb;
                copy_particle(c, q, p);
                c->ghost[q] = 0;
                if (!right) pos_of(c, d)[q] += (xmax - xmin);
                else pos_of(c, d)[q] -= (xmax - xmin);
                c->ghost[p] = 1;
                nb++;
            }
            c->np = cur + nb;
            cnt = nb;
        } else {
            for (long p = 0; p < c->np; p++) {
                if (c->ghost[p]) continue;
                double *xp = &pos_of(c, d)[p];
                if (right && *xp > xmax) {
                    cnt++;
                    if (c->pbc[s] == BC_REFLECTING) {
                        *xp = 2.0 * xmax - *xp;
                        vel_of(c, d)[p] = -vel_of(c, d)[p];
                    } else {
                        c->ghost[p] = 1;
                    }
                } else if (!right && *xp < xmin) {
                    cnt++;
                    if (c->pbc[s] == BC_REFLECTING) {
                        *xp = 2.0 * xmin - *xp;
                        vel_of(c, d)[p] = -vel_of(c, d)[p];
                    } else {
                        c->ghost[p] = 1;
                    }
                }
            }
        }
        if (counts6) counts6[s] = cnt;
    }
    return 0;
}

/* clearGhosts, src/particles/particle_handler.cpp:271-284 */
int orc_clear_ghosts(void *h) {
    orc_t *c = (orc_t *)h;
    long i = 0;
    while (i < c->np) {
        if (c->ghost[i]) {
            swap_particle(c, i, c->np - 1);
            c->np--;
        } else {
            i++;
        }
    }
    return 0;
}

/* Grid::addJ with its Jx index quirk (b), src/grid/oGrid.cpp:91-114 */
static void add_j(orc_t *c, int cid, const double *J) {
    int ix, iy, iz;
    cell_split(c, cid, &ix, &iy, &iz);
    double *Jx = c->slot[EMOO_JX], *Jy = c->slot[EMOO_JY], *Jz = c->slot[EMOO_JZ];
    Jx[IDX(c, ix, iy, iz)] += J[0];
    Jx[IDX(c, ix, iy + 1, iz)] += J[1];
    Jx[IDX(c, ix, iy + 1, iz + 1)] += J[2];
    if (c->policy) Jx[IDX(c, ix, iy, iz + 1)] += J[3]; /* corrected: the cell's own 4th x-edge */
    else Jx[IDX(c, ix, iy + 1, iz)] += J[3];
    Jy[IDX(c, ix, iy, iz)] += J[4];
    Jy[IDX(c, ix, iy, iz + 1)] += J[5];
    Jy[IDX(c, ix + 1, iy, iz + 1)] += J[6];
    Jy[IDX(c, ix + 1, iy, iz)] += J[7];
    Jz[IDX(c, ix, iy, iz)] += J[8];
    Jz[IDX(c, ix + 1, iy, iz)] += J[9];
    Jz[IDX(c, ix + 1, iy + 1, iz)] += J[10];
    Jz[IDX(c, ix, iy + 1, iz)] += J[11];
}

/* Grid::addRho, src/grid/oGrid.cpp:122-139 */
static void add_rho(orc_t *c, int cid, const double *R) {
    int ix, iy, iz;
    cell_split(c, cid, &ix, &iy, &iz);
    double *rho = c->slot[EMOO_RHO];
    rho[IDX(c, ix, iy, iz)] += R[0];
    rho[IDX(c, ix + 1, iy, iz)] += R[1];
    rho[IDX(c, ix + 1, iy + 1, iz)] += R[2];
    rho[IDX(c, ix, iy + 1, iz)] += R[3];
    rho[IDX(c, ix, iy + 1, iz + 1)] += R[4];
    rho[IDX(c, ix + 1, iy + 1, iz + 1)] += R[5];
    rho[IDX(c, ix + 1, iy, iz + 1)] += R[6];
    rho[IDX(c, ix, iy, iz + 1)] += R[7];
}

/* Particle_Handler::depositRhoJ (src/particles/particle_handler.cpp:185-239)
 * with Depositor::deposit_particle_J / _Rho (src/particles/deposit.cpp:12-62):
 * contributions accumulate per run of equal cell IDs and are flushed on a
 * cell change. The uniform background (orc_set_rho_background) is added afterwards. */
static void deposit(orc_t *c, int with_rho) {
    long npts = c->npts;
    memset(c->slot[EMOO_JX], 0, sizeof(double) * (size_t)npts);
    memset(c->slot[EMOO_JY], 0, sizeof(double) * (size_t)npts);
    memset(c->slot[EMOO_JZ], 0, sizeof(double) * (size_t)npts);
    if (with_rho) memset(c->slot[EMOO_RHO], 0, sizeof(double) * (size_t)npts);
    const double *l = c->d;
    double vol = l[0] * l[1] * l[2];
    long cellID = -1;
    double JObj[12] = {0}, RhoObj[8] = {0}, verts[3] = {0, 0, 0};
    for (long p = 0; p < c->np; p++) {
        int s = c->type[p];
        if (c->ghost[p] || c->info.isTestParticle[s]) continue;
        int tmp = cell_id(c, c->x[p], c->y[p], c->z[p], NULL, NULL, NULL);
        if (tmp != cellID) {
            if (cellID != -1) {
                add_j(c, (int)cellID, JObj);
                if (with_rho) add_rho(c, (int)cellID, RhoObj);
                for (int k = 0; k < 12; k++) JObj[k] = 0;
                if (with_rho)
                    for (int k = 0; k < 8; k++) RhoObj[k] = 0;
            }
            cellID = tmp;
            int ix, iy, iz;
            cell_split(c, tmp, &ix, &iy, &iz);
            verts[0] = c->x0[0] + c->d[0] * (ix - c->policy);
            verts[1] = c->x0[1] + c->d[1] * (iy - c->policy);
            verts[2] = c->x0[2] + c->d[2] * (iz - c->policy);
        }
        double q = c->info.charge_ratio[s];
        double xp[3] = {c->x[p], c->y[p], c->z[p]};
        double vp[3] = {c->vx[p], c->vy[p], c->vz[p]};
        double r[3];
        for (int i = 0; i < 3; i++) r[i] = xp[i] - verts[i];
        for (int i = 0; i < 3; i++) {
            int j = (i + 1) % 3, k = (i + 2) % 3;
            double area = l[j] * l[k];
            double cur = UNIT_RHOJ * q * vp[i];
            double ratio = (cur / vol) / area;
            JObj[4 * i] += ratio * (l[j] - r[j]) * (l[k] - r[k]);
            JObj[4 * i + 1] += ratio * r[j] * (l[k] - r[k]);
            JObj[4 * i + 2] += ratio * r[j] * r[k];
            JObj[4 * i + 3] += ratio * (l[j] - r[j]) * r[k];
        }
        if (with_rho) {
            double cr = UNIT_RHOJ * (q / vol) / vol;
            RhoObj[0] += cr * (l[0] - r[0]) * (l[1] - r[1]) * (l[2] - r[2]);
            RhoObj[1] += cr * r[0] * (l[1] - r[1]) * (l[2] - r[2]);
            RhoObj[2] += cr * r[0] * r[1] * (l[2] - r[2]);
            RhoObj[3] += cr * (l[0] - r[0]) * r[1] * (l[2] - r[2]);
            RhoObj[4] += cr * (l[0] - r[0]) * r[1] * r[2];
            RhoObj[5] += cr * r[0] * r[1] * r[2];
            RhoObj[6] += cr * r[0] * (l[1] - r[1]) * r[2];
            RhoObj[7] += cr * (l[0] - r[0]) * (l[1] - r[1]) * r[2];
        }
    }
    if (cellID != -1) {
        add_j(c, (int)cellID, JObj);
        if (with_rho) add_rho(c, (int)cellID, RhoObj);
    }
    if (with_rho && c->rho_bg != 0.0) {
        /* the immobile background sits on the physical points */
        double *rho = c->slot[EMOO_RHO];
        for (int i = c->rho_bg_i0 > 1 ? c->rho_bg_i0 : 1; i <= c->n[0]; i++)
            for (int j = 1; j <= c->n[1]; j++)
                for (int k = 1; k <= c->n[2]; k++) rho[IDX(c, i, j, k)] += c->rho_bg;
    }
}

/* Uniform immobile background charge density added to rho at every deposit
 * (the neutralising ions of the two-stream and laser-plasma workloads; the reference has none). */
void orc_set_rho_background(void *h, double v) { ((orc_t *)h)->rho_bg = v; }

/* Restricts the background to the physical points with x >= xmin (grid point
 * x index i at xyz0 + (i - 1) dx). */
void orc_set_rho_background_xmin(void *h, double xmin) {
    orc_t *c = (orc_t *)h;
    c->rho_bg_i0 = c->n[0] + 1;
    for (int i = 1; i <= c->n[0]; i++)
        if (c->x0[0] + (i - 1) * c->d[0] >= xmin) { c->rho_bg_i0 = i; break; }
}

int orc_deposit(void *h, int with_rho) {
    deposit((orc_t *)h, with_rho);
    return 0;
}

/* Stable counting sort by (species, cellID), ascending: the sort order of the
 * GPU library (the reference sorts descending with an unstable std::sort,
 * src/particles/particle_handler.cpp:180-183, particle_utils.hpp:31-51). */
int orc_sort(void *h) {
    orc_t *c = (orc_t *)h;
    long ncell = (long)(c->n[0] + 2) * (c->n[1] + 2) * (c->n[2] + 2);
    long nkey = ncell * c->info.nspecies;
    long *cnt = (long *)calloc((size_t)nkey + 1, sizeof(long));
    long *key = (long *)malloc(sizeof(long) * (size_t)(c->np ? c->np : 1));
    long *perm = (long *)malloc(sizeof(long) * (size_t)(c->np ? c->np : 1));
    if (!cnt || !key || !perm) return -2;
    for (long p = 0; p < c->np; p++) {
        key[p] = (long)c->type[p] * ncell + cell_id(c, c->x[p], c->y[p], c->z[p], NULL, NULL, NULL);
        cnt[key[p] + 1]++;
    }
    for (long k = 0; k < nkey; k++) cnt[k + 1] += cnt[k];
    for (long p = 0; p < c->np; p++) perm[cnt[key[p]]++] = p;
    /* apply the permutation through a scratch copy at the end of the arrays */
    if (grow(c, 2 * c->np)) return -2;
    for (long i = 0; i < c->np; i++) copy_particle(c, c->np + i, perm[i]);
    for (long i = 0; i < c->np; i++) copy_particle(c, i, c->np + i);
    free(cnt); free(key); free(perm);
    return 0;
}

/* ------------------------------------------------------------------ */
/* fields                                                               */

/* Grid::evolveFields, src/grid/oGrid.cpp:15-60 (role swap first, (f)). */
static void evolve(orc_t *c, double dt) {
    c->bswap ^= 1;
    double *Ex = c->slot[EMOO_EX], *Ey = c->slot[EMOO_EY], *Ez = c->slot[EMOO_EZ];
    double *Jx = c->slot[EMOO_JX], *Jy = c->slot[EMOO_JY], *Jz = c->slot[EMOO_JZ];
    double *Bx = role_B(c, 0), *By = role_B(c, 1), *Bz = role_B(c, 2);
    double *Tx = role_Btm1(c, 0), *Ty = role_Btm1(c, 1), *Tz = role_Btm1(c, 2);
    double dx = c->d[0], dy = c->d[1], dz = c->d[2];
    int nx = c->n[0], ny = c->n[1], nz = c->n[2];
    for (int i = 1; i <= nx; i++)
        for (int j = 1; j <= ny; j++)
            for (int k = 1; k <= nz; k++) {
                long o = IDX(c, i, j, k);
                Ex[o] = Ex[o] - dt * ((Ty[o] - Ty[IDX(c, i, j, k - 1)]) / dz - (Tz[o] - Tz[IDX(c, i, j - 1, k)]) / dy +
                                      4 * PI_D * Jx[o]);
                Ey[o] = Ey[o] - dt * ((Tz[o] - Tz[IDX(c, i - 1, j, k)]) / dx - (Tx[o] - Tx[IDX(c, i, j, k - 1)]) / dz +
                                      4 * PI_D * Jy[o]);
                Ez[o] = Ez[o] - dt * ((Tx[o] - Tx[IDX(c, i, j - 1, k)]) / dy - (Ty[o] - Ty[IDX(c, i - 1, j, k)]) / dx +
                                      4 * PI_D * Jz[o]);
            }
    /* corrected policy: the B half below reads E at plane n+1 and at the
     * boundary planes, so E's periodic images and LightBC planes are set
     * first (time-centred leapfrog at the wrap and at external sides) */
    if (c->policy) corrected_e_bounds(c);
    for (int i = 1; i <= nx; i++)
        for (int j = 1; j <= ny; j++)
            for (int k = 1; k <= nz; k++) {
                long o = IDX(c, i, j, k);
                Bx[o] = Tx[o] + dt * ((Ey[IDX(c, i, j, k + 1)] - Ey[o]) / dz - (Ez[IDX(c, i, j + 1, k)] - Ez[o]) / dy);
                By[o] = Ty[o] + dt * ((Ez[IDX(c, i + 1, j, k)] - Ez[o]) / dx - (Ex[IDX(c, i, j, k + 1)] - Ex[o]) / dz);
                Bz[o] = Tz[o] + dt * ((Ex[IDX(c, i, j + 1, k)] - Ex[o]) / dy - (Ey[IDX(c, i + 1, j, k)] - Ey[o]) / dx);
            }
}

/* Grid::evolveFieldsES, src/grid/oGrid.cpp:67-81 */
static void evolve_es(orc_t *c, double dt) {
    double *Ex = c->slot[EMOO_EX], *Ey = c->slot[EMOO_EY], *Ez = c->slot[EMOO_EZ];
    double *Jx = c->slot[EMOO_JX], *Jy = c->slot[EMOO_JY], *Jz = c->slot[EMOO_JZ];
    for (int i = 1; i <= c->n[0]; i++)
        for (int j = 1; j <= c->n[1]; j++)
            for (int k = 1; k <= c->n[2]; k++) {
                long o = IDX(c, i, j, k);
                Ex[o] = -dt * (4 * PI_D * Jx[o]);
                Ey[o] = -dt * (4 * PI_D * Jy[o]);
                Ez[o] = -dt * (4 * PI_D * Jz[o]);
            }
}

int orc_evolve(void *h, int electrostatic) {
    orc_t *c = (orc_t *)h;
    if (electrostatic) evolve_es(c, c->dt);
    else evolve(c, c->dt);
    return 0;
}

/* Poisson_Solver::run_poisson_solver_, src/poisson/poisson.cpp:172-287.
 * Returns the last iteration index; *conv = 1 if it met the tolerance. */
static int jacobi(orc_t *c, int id1, int id2, const double *R, double tol, double mult, int *conv) {
    double dx = c->d[0], dy = c->d[1], dz = c->d[2];
    double celldist2 = pow(dx, 2.0) * pow(dy, 2.0) + pow(dy, 2.0) * pow(dz, 2.0) + pow(dx, 2.0) * pow(dz, 2.0);
    double ax = pow(dy, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    double ay = pow(dx, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    double az = pow(dx, 2.0) * pow(dy, 2.0) / (2.0 * celldist2);
    double af = pow(dx, 2.0) * pow(dy, 2.0) * pow(dz, 2.0) / (2.0 * celldist2);
    double *u1 = c->slot[id1], *u2 = c->slot[id2];
    orc_execute_bc(c, id1);
    int iternum = -1, converged = 0;
    double maxDiff;
    do {
        iternum++;
        maxDiff = 0.0;
        double *src = (iternum % 2 == 0) ? u1 : u2;
        double *dst = (iternum % 2 == 0) ? u2 : u1;
        for (int i = 1; i <= c->n[0]; i++)
            for (int j = 1; j <= c->n[1]; j++)
                for (int k = 1; k <= c->n[2]; k++) {
                    long o = IDX(c, i, j, k);
                    dst[o] = ax * (src[IDX(c, i - 1, j, k)] + src[IDX(c, i + 1, j, k)]) +
                             ay * (src[IDX(c, i, j - 1, k)] + src[IDX(c, i, j + 1, k)]) +
                             az * (src[IDX(c, i, j, k - 1)] + src[IDX(c, i, j, k + 1)]) - af * R[o] * mult;
                }
        orc_execute_bc(c, (iternum % 2 == 0) ? id2 : id1);
        for (int i = 1; i <= c->n[0]; i++)
            for (int j = 1; j <= c->n[1]; j++)
                for (int k = 1; k <= c->n[2]; k++) {
                    long o = IDX(c, i, j, k);
                    double a = fabs(u2[o] - u1[o]);
                    if (a > maxDiff) maxDiff = a;
                }
        if (maxDiff < tol) converged = 1;
    } while (!converged && iternum < ITER_MAX);
    *conv = iternum < ITER_MAX;
    return iternum;
}

/* The discrete problem the Jacobi iteration of run_poisson_solver_
 * (src/poisson/poisson.cpp:216-241) has as its fixed point, solved outright:
 * at every unknown point the 7-point Laplacian of u equals mult R, where a
 * dimension with periodic field boundaries wraps (unknowns 1..n) and one with
 * external boundaries holds the PoissonBC values on planes 1 and n + 1
 * (unknowns 2..n). Conjugate gradients on -Laplacian (symmetric positive
 * semi-definite), to |r| <= rtol |b| in the 2-norm; with every dimension
 * periodic the right side's mean is removed first (the system is singular
 * and consistent only then) and the solution's mean set to zero, which the
 * field differences of phiToE / AToB do not see. The result goes to id1,
 * ghost planes by the same boundary fill as the Jacobi, and a copy to id2.
 * Returns the iteration count, or -1 when a side's field boundary is neither
 * periodic nor external or the two sides of a dimension differ. *conv = 1
 * when the tolerance was met within the iteration cap. */
static int exact_poisson(orc_t *c, int id1, int id2, const double *R, double mult, double rtol, int *conv) {
    int per[3], lo[3], hi[3], m[3];
    *conv = 0;
    for (int d = 0; d < 3; d++) {
        int a = c->fbc[2 * d], b = c->fbc[2 * d + 1];
        if (a != b || (a != BC_PERIODIC && a != BC_EXTERNAL)) return -1;
        per[d] = a == BC_PERIODIC;
        lo[d] = per[d] ? 1 : 2;
        hi[d] = c->n[d];
        m[d] = hi[d] - lo[d] + 1;
    }
    double *u = c->slot[id1];
    for (long o = 0; o < c->npts; o++) u[o] = 0.0;
    orc_execute_bc(c, id1); /* the Dirichlet planes */
    if (m[0] < 1 || m[1] < 1 || m[2] < 1) { /* no unknowns: the boundary planes are the solution */
        memcpy(c->slot[id2], u, sizeof(double) * c->npts);
        *conv = 1;
        return 0;
    }
    long nu = (long)m[0] * m[1] * m[2];
    double *x = calloc(nu, sizeof(double)), *r = malloc(nu * sizeof(double));
    double *p = malloc(nu * sizeof(double)), *q = malloc(nu * sizeof(double));
    double cd[3];
    for (int d = 0; d < 3; d++) cd[d] = 1.0 / (c->d[d] * c->d[d]);
#define UIDX(a, b, e) (((long)(a) * m[1] + (b)) * m[2] + (e))
    /* b = -mult R + (boundary neighbours' values) / h^2 */
    for (int a = 0; a < m[0]; a++)
        for (int b = 0; b < m[1]; b++)
            for (int e = 0; e < m[2]; e++) {
                int ii[3] = {a + lo[0], b + lo[1], e + lo[2]};
                double v = -mult * R[IDX(c, ii[0], ii[1], ii[2])];
                for (int d = 0; d < 3; d++) {
                    if (per[d]) continue;
                    int jj[3] = {ii[0], ii[1], ii[2]};
                    if (ii[d] == lo[d]) {
                        jj[d] = 1;
                        v += cd[d] * u[IDX(c, jj[0], jj[1], jj[2])];
                    }
                    if (ii[d] == hi[d]) {
                        jj[d] = c->n[d] + 1;
                        v += cd[d] * u[IDX(c, jj[0], jj[1], jj[2])];
                    }
                }
                r[UIDX(a, b, e)] = v;
            }
    int allper = per[0] && per[1] && per[2];
    if (allper) {
        double mean = 0.0;
        for (long t = 0; t < nu; t++) mean += r[t];
        mean /= (double)nu;
        for (long t = 0; t < nu; t++) r[t] -= mean;
    }
    double bn = 0.0;
    for (long t = 0; t < nu; t++) bn += r[t] * r[t];
    bn = sqrt(bn);
    double rr = bn * bn;
    for (long t = 0; t < nu; t++) p[t] = r[t];
    int it = 0;
    const int cap = 100000;
    while (sqrt(rr) > rtol * bn && it < cap) {
        /* q = -Laplacian(p), homogeneous boundaries */
        double pq = 0.0;
        for (int a = 0; a < m[0]; a++)
            for (int b = 0; b < m[1]; b++)
                for (int e = 0; e < m[2]; e++) {
                    int ii[3] = {a, b, e};
                    double v = 2.0 * (cd[0] + cd[1] + cd[2]) * p[UIDX(a, b, e)];
                    for (int d = 0; d < 3; d++)
                        for (int sgn = -1; sgn <= 1; sgn += 2) {
                            int jj[3] = {ii[0], ii[1], ii[2]};
                            jj[d] += sgn;
                            if (jj[d] < 0 || jj[d] >= m[d]) {
                                if (!per[d]) continue;
                                jj[d] = (jj[d] + m[d]) % m[d];
                            }
                            v -= cd[d] * p[UIDX(jj[0], jj[1], jj[2])];
                        }
                    q[UIDX(a, b, e)] = v;
                    pq += v * p[UIDX(a, b, e)];
                }
        double alpha = rr / pq;
        double rr1 = 0.0;
        for (long t = 0; t < nu; t++) {
            x[t] += alpha * p[t];
            r[t] -= alpha * q[t];
            rr1 += r[t] * r[t];
        }
        double beta = rr1 / rr;
        rr = rr1;
        for (long t = 0; t < nu; t++) p[t] = r[t] + beta * p[t];
        it++;
    }
    *conv = sqrt(rr) <= rtol * bn;
    if (allper) {
        double mean = 0.0;
        for (long t = 0; t < nu; t++) mean += x[t];
        mean /= (double)nu;
        for (long t = 0; t < nu; t++) x[t] -= mean;
    }
    for (int a = 0; a < m[0]; a++)
        for (int b = 0; b < m[1]; b++)
            for (int e = 0; e < m[2]; e++) u[IDX(c, a + lo[0], b + lo[1], e + lo[2])] = x[UIDX(a, b, e)];
#undef UIDX
    orc_execute_bc(c, id1);
    memcpy(c->slot[id2], u, sizeof(double) * c->npts);
    free(x);
    free(r);
    free(p);
    free(q);
    return it;
}

int orc_set_poisson_solver(void *h, int solver, double rtol) {
    orc_t *c = (orc_t *)h;
    if (solver != 0 && solver != 1) return -1;
    c->poisson_solver = solver;
    c->poisson_rtol = rtol > 0 ? rtol : 1e-13;
    return 0;
}

/* phiToE, src/poisson/convertFields.cpp:10-68 (reads phi1, (g)) */
static void phi_to_e(orc_t *c) {
    const double *phi = c->slot[EMOO_PHI1];
    for (int dir = 0; dir < 3; dir++) {
        double *E = c->slot[EMOO_EX + dir];
        double h = c->d[dir];
        for (int i = 1; i <= c->n[0]; i++)
            for (int j = 1; j <= c->n[1]; j++)
                for (int k = 1; k <= c->n[2]; k++) {
                    long nxt = dir == 0 ? IDX(c, i + 1, j, k) : dir == 1 ? IDX(c, i, j + 1, k) : IDX(c, i, j, k + 1);
                    long o = IDX(c, i, j, k);
                    E[o] = -(phi[nxt] - phi[o]) / h;
                }
    }
}

/* AToB, src/poisson/convertFields.cpp:73-154 (quirk (h): both differences
 * taken of Ak; B written through the fixed slots). */
static void a_to_b(orc_t *c) {
    for (int dir = 0; dir < 3; dir++) {
        double *B = c->slot[EMOO_BX + dir];
        const double *Ak, *Aj;
        double hk, hj;
        if (dir == 0) { Ak = c->slot[EMOO_AZ1]; hk = c->d[2]; Aj = c->slot[EMOO_AY1]; hj = c->d[1]; }
        else if (dir == 1) { Ak = c->slot[EMOO_AX1]; hk = c->d[0]; Aj = c->slot[EMOO_AZ1]; hj = c->d[2]; }
        else { Ak = c->slot[EMOO_AY1]; hk = c->d[1]; Aj = c->slot[EMOO_AX1]; hj = c->d[0]; }
        for (int i = 1; i <= c->n[0]; i++)
            for (int j = 1; j <= c->n[1]; j++)
                for (int k = 1; k <= c->n[2]; k++) {
                    long nk, nj;
                    if (dir == 0) { nk = IDX(c, i, j + 1, k); nj = IDX(c, i, j, k + 1); }
                    else if (dir == 1) { nk = IDX(c, i, j, k + 1); nj = IDX(c, i + 1, j, k); }
                    else { nk = IDX(c, i + 1, j, k); nj = IDX(c, i, j + 1, k); }
                    long o = IDX(c, i, j, k);
                    B[o] = (Ak[nk] - Ak[o]) / hj + (Ak[nj] - Aj[o]) / hk;
                }
    }
}

/* Poisson_Solver::InitializeFields, src/poisson/poisson.cpp:143-170.
 * iters[4] receives the last iteration index of the phi, Ax, Ay, Az solves.
 * Returns 1 when every solve converged. */
static int poisson_init(orc_t *c, int *iters) {
    double mult = -4 * PI_D;
    if (c->poisson_solver == 1) {
        int ok = 1, cv;
        for (int q = 0; q < 4; q++) {
            int it = exact_poisson(c, q == 0 ? EMOO_PHI1 : EMOO_AX1 + (q - 1), q == 0 ? EMOO_PHI2 : EMOO_AX2 + (q - 1),
                                   c->slot[q == 0 ? EMOO_RHO : EMOO_JX + (q - 1)], mult, c->poisson_rtol, &cv);
            if (it < 0) return -1;
            ok &= cv;
            if (iters) iters[q] = it;
            if (q == 0) phi_to_e(c);
        }
        a_to_b(c);
        orc_execute_bc(c, EMOO_SEND_EB);
        return ok;
    }
    double a = c->conv_phi * CONV_RATIO;
    double tol = a < CONV_CRIT ? CONV_CRIT : a;
    int ok = 1, cv;
    int it = jacobi(c, EMOO_PHI1, EMOO_PHI2, c->slot[EMOO_RHO], tol, mult, &cv);
    ok &= cv;
    if (iters) iters[0] = it;
    phi_to_e(c);
    a = c->conv_A * CONV_RATIO;
    tol = a < CONV_CRIT ? CONV_CRIT : a;
    for (int q = 0; q < 3; q++) {
        it = jacobi(c, EMOO_AX1 + q, EMOO_AX2 + q, c->slot[EMOO_JX + q], tol, mult, &cv);
        ok &= cv;
        if (iters) iters[1 + q] = it;
    }
    a_to_b(c);
    orc_execute_bc(c, EMOO_SEND_EB);
    return ok;
}

/* Grid::InitializeFields for the non-Poisson path, src/grid/grid.cpp:554-574 */
static void const_init(orc_t *c) {
    const emoo_input_info *in = &c->info;
    long n = c->npts;
    int cst = (in->restart == 0 && strcmp(in->fields_init, "constant") == 0);
    if (!cst) {
        memset(c->slot[EMOO_JX], 0, sizeof(double) * n);
        memset(c->slot[EMOO_JY], 0, sizeof(double) * n);
        memset(c->slot[EMOO_JZ], 0, sizeof(double) * n);
    }
    for (int q = 0; q < 3; q++) {
        for (long o = 0; o < n; o++) c->slot[EMOO_EX + q][o] = in->E0[q];
        for (long o = 0; o < n; o++) c->slot[EMOO_BX + q][o] = in->B0[q];
        for (long o = 0; o < n; o++) c->slot[EMOO_BX_TM1 + q][o] = in->B0[q];
    }
    if (!cst) memset(c->slot[EMOO_RHO], 0, sizeof(double) * n);
}

int orc_initialize_fields_only(void *h, int *iters) {
    orc_t *c = (orc_t *)h;
    c->t = 0.0;
    c->dtp = 0.0;
    int ok = 1;
    if (c->poisson) ok = poisson_init(c, iters);
    else const_init(c);
    c->t = c->t0;
    c->dtp = c->dt;
    return ok < 0 ? -1 : ok ? 0 : -3;
}

/* src/main.cpp:159-179 */
int orc_init_fields(void *h, int *iters) {
    orc_t *c = (orc_t *)h;
    c->t = 0.0;
    c->dtp = 0.0;
    int ok = 1;
    if (c->poisson) {
        deposit(c, 1);
        orc_execute_bc(c, EMOO_SEND_JRHO);
        ok = poisson_init(c, iters);
    } else {
        const_init(c);
    }
    orc_interpolate(c);
    c->t = c->t0;
    c->dtp = c->dt;
    return ok < 0 ? -1 : ok ? 0 : -3;
}

void orc_set_time(void *h, double t, double dtp) {
    orc_t *c = (orc_t *)h;
    c->t = t;
    c->dtp = dtp;
}

double orc_time(void *h) { return ((orc_t *)h)->t; }

/* OutputBoxQuantities::output, src/IO/output.cpp:52-123 (fixed slots for B,
 * (f); SQR(x) expands to x*x without parentheses, hence ((0.5*s)*0.5)*s). */
int orc_history(void *h, double t, double *out8) {
    orc_t *c = (orc_t *)h;
    double pEn = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
    for (long p = 0; p < c->np; p++) {
        double m = c->info.mass_ratio[c->type[p]];
        double vx = c->vx[p], vy = c->vy[p], vz = c->vz[p];
        pEn += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        mx += m * vx;
        my += m * vy;
        mz += m * vz;
    }
    double vol = c->d[0] * c->d[1] * c->d[2];
    double e[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 1; i <= c->n[0]; i++)
        for (int j = 1; j <= c->n[1]; j++)
            for (int k = 1; k <= c->n[2]; k++) {
                long o = IDX(c, i, j, k);
                long nx_ = IDX(c, i + 1, j, k), ny_ = IDX(c, i, j + 1, k), nz_ = IDX(c, i, j, k + 1);
                long nb[3] = {nx_, ny_, nz_};
                for (int q = 0; q < 3; q++) {
                    double s = c->slot[EMOO_EX + q][o] + c->slot[EMOO_EX + q][nb[q]];
                    e[q] += 0.5 * vol * (0.5 * s * 0.5 * s);
                }
                for (int q = 0; q < 3; q++) {
                    double s = c->slot[EMOO_BX + q][o] + c->slot[EMOO_BX + q][nb[q]];
                    e[3 + q] += 0.5 * vol * (0.5 * s * 0.5 * s);
                }
            }
    double B_en = e[3] + e[4] + e[5];
    double E_en = e[0] + e[1] + e[2];
    out8[0] = t;
    out8[1] = mx;
    out8[2] = my;
    out8[3] = mz;
    out8[4] = pEn;
    out8[5] = B_en;
    out8[6] = E_en;
    out8[7] = B_en + E_en + pEn;
    return 0;
}

/* Gauss-law residual div E - 4 pi rho over physical vertices (no reference
 * counterpart): out2 = {max |r|, sqrt(sum r^2)}. */
int orc_gauss_residual(void *h, double *out2) {
    orc_t *c = (orc_t *)h;
    const double *Ex = c->slot[EMOO_EX], *Ey = c->slot[EMOO_EY], *Ez = c->slot[EMOO_EZ], *rho = c->slot[EMOO_RHO];
    double mx = 0.0, s2 = 0.0;
    for (int i = 1; i <= c->n[0]; i++)
        for (int j = 1; j <= c->n[1]; j++)
            for (int k = 1; k <= c->n[2]; k++) {
                long o = IDX(c, i, j, k);
                double dv = (Ex[o] - Ex[IDX(c, i - 1, j, k)]) / c->d[0] + (Ey[o] - Ey[IDX(c, i, j - 1, k)]) / c->d[1] +
                            (Ez[o] - Ez[IDX(c, i, j, k - 1)]) / c->d[2];
                double r = dv - 4 * PI_D * rho[o];
                double a = fabs(r);
                if (a > mx) mx = a;
                s2 += r * r;
            }
    out2[0] = mx;
    out2[1] = sqrt(s2);
    return 0;
}

/* ------------------------------------------------------------------ */
/* the corrected-physics policy (no reference counterpart)              */

/* Selects the corrected-physics policy (1) or the reference's arithmetic
 * (0). Under the corrected policy every dimension is either periodic
 * (particle and field sides) or walled (particle sides reflecting or
 * absorbing, field sides external; -1 otherwise): gather and deposit use the
 * cell's own lower corner as vertex, the current comes from Villasenor and
 * Buneman's charge-conserving deposit along each particle's straight path,
 * periodic ghost copies and folds cover the whole transverse range of every
 * component, the current a reflected particle deposited beyond its wall is
 * mirrored back (mirror_fold), and E's boundary values - periodic images or
 * LightBC planes - are set between the two halves of the Yee update. */
int orc_set_policy(void *h, int policy) {
    orc_t *c = (orc_t *)h;
    if (policy != 0 && policy != 1) return -1;
    if (policy)
        for (int d = 0; d < 3; d++) {
            const int pl = c->pbc[2 * d], pr = c->pbc[2 * d + 1], fl = c->fbc[2 * d], fr = c->fbc[2 * d + 1];
            const int periodic = pl == BC_PERIODIC && pr == BC_PERIODIC && fl == BC_PERIODIC && fr == BC_PERIODIC;
            const int walled = pl != BC_PERIODIC && pr != BC_PERIODIC && fl == BC_EXTERNAL && fr == BC_EXTERNAL;
            if (!periodic && !walled) return -1;
        }
    c->policy = policy;
    return 0;
}

/* Villasenor-Buneman current (J. Villasenor and O. Buneman, Comput. Phys.
 * Commun. 69 (1992) 306) of one particle moving in a straight line from p0
 * to p1 (unwrapped, at most one cell face per axis): the path is split at
 * the faces it crosses; a piece with offsets a -> b inside a cell (cell
 * units, m = (a + b) / 2, D = b - a) adds to the cell's four x edges
 * coef dx Dx ((1-my)(1-mz) + Dy Dz / 12), (my (1-mz) - ..), ((1-my) mz - ..),
 * (my mz + ..) (edges at y, y+1 / z, z+1), and likewise for y and z. With the
 * linear charge assignment this makes rho(t + dt) - rho(t) + dt div J = 0
 * exactly at every point. coef = UNIT_RHOJ q / V / dt. */
static void vb_deposit(orc_t *c, const double p0[3], const double p1[3], double coef) {
    double u0[3], u1[3], ts[5];
    int nt = 0;
    ts[nt++] = 0.0;
    for (int a = 0; a < 3; a++) {
        u0[a] = (p0[a] - c->x0[a]) * c->id[a];
        u1[a] = (p1[a] - c->x0[a]) * c->id[a];
        double f0 = floor(u0[a]), f1 = floor(u1[a]);
        if (f0 != f1) {
            double b = f0 > f1 ? f0 : f1;
            ts[nt++] = (b - u0[a]) / (u1[a] - u0[a]);
        }
    }
    ts[nt++] = 1.0;
    for (int i = 2; i < nt - 1; i++) /* insertion sort of the crossings */
        for (int j = i; j > 1 && ts[j] < ts[j - 1]; j--) {
            double t = ts[j]; ts[j] = ts[j - 1]; ts[j - 1] = t;
        }
    double *J[3] = {c->slot[EMOO_JX], c->slot[EMOO_JY], c->slot[EMOO_JZ]};
    for (int sgi = 0; sgi + 1 < nt; sgi++) {
        double ta = ts[sgi], tb = ts[sgi + 1];
        if (!(tb > ta)) continue;
        double a_[3], b_[3], m[3], D[3];
        int cell[3];
        for (int a = 0; a < 3; a++) {
            double ua = u0[a] + ta * (u1[a] - u0[a]), ub = u0[a] + tb * (u1[a] - u0[a]);
            cell[a] = (int)floor(0.5 * (ua + ub));
            a_[a] = ua - cell[a];
            b_[a] = ub - cell[a];
            D[a] = b_[a] - a_[a];
            m[a] = 0.5 * (a_[a] + b_[a]);
        }
        for (int a = 0; a < 3; a++) {
            int jb = (a + 1) % 3, kb = (a + 2) % 3;
            double w = coef * c->d[a] * D[a];
            double cr = D[jb] * D[kb] / 12.0;
            double W[4] = {w * ((1.0 - m[jb]) * (1.0 - m[kb]) + cr), w * (m[jb] * (1.0 - m[kb]) - cr),
                           w * ((1.0 - m[jb]) * m[kb] - cr), w * (m[jb] * m[kb] + cr)};
            for (int e = 0; e < 4; e++) {
                int ii[3] = {cell[0] + 1, cell[1] + 1, cell[2] + 1};
                ii[jb] += e & 1;
                ii[kb] += e >> 1;
                J[a][IDX(c, ii[0], ii[1], ii[2])] += W[e];
            }
        }
    }
}

/* A particle whose move ends beyond an absorbing wall leaves the domain in
 * this step (the particle boundaries remove it). Its whole charge must cross
 * the wall's vertex plane for the continuity equation to hold there, so the
 * path is continued along the wall's normal to the next vertex plane beyond
 * the wall (x0 - d, or x0 + L + d): that piece, inside the ghost cell, adds
 * the flux of the charge the move's end point still left on the wall plane.
 * (Corrected policy, no reference counterpart.) */
static void absorbed_exit(orc_t *c, const double p1[3], double coef) {
    double a[3] = {p1[0], p1[1], p1[2]};
    for (int d = 0; d < 3; d++) {
        const double xmin = c->x0[d], xmax = xmin + c->L[d];  /* the particle boundaries' limits */
        double b[3] = {a[0], a[1], a[2]};
        if (c->pbc[2 * d] == BC_ABSORBING && a[d] < xmin) b[d] = xmin - c->d[d];
        else if (c->pbc[2 * d + 1] == BC_ABSORBING && a[d] > xmax) b[d] = xmax + c->d[d];
        else continue;
        vb_deposit(c, a, b, coef);
        a[d] = b[d];
    }
}

/* Push with the cached fields and the charge-conserving current of the
 * move (before the boundaries wrap the particle). */
static void push_vb(orc_t *c, double dt) {
    long npts = c->npts;
    for (int a = 0; a < 3; a++) memset(c->slot[EMOO_JX + a], 0, sizeof(double) * (size_t)npts);
    double vol = c->d[0] * c->d[1] * c->d[2];
    for (long p = 0; p < c->np; p++) {
        int s = c->type[p];
        double p0[3] = {c->x[p], c->y[p], c->z[p]};
        double st[7] = {c->x[p], c->y[p], c->z[p], c->vx[p], c->vy[p], c->vz[p], c->g[p]};
        double f[6] = {c->fe1[p], c->fe2[p], c->fe3[p], c->fb1[p], c->fb2[p], c->fb3[p]};
        if (c->info.relativity == 0) boris(st, c->info.charge_ratio[s], c->info.mass_ratio[s], f, dt);
        else vay(st, c->info.charge_ratio[s], c->info.mass_ratio[s], f, dt);
        c->x[p] = st[0]; c->y[p] = st[1]; c->z[p] = st[2];
        c->vx[p] = st[3]; c->vy[p] = st[4]; c->vz[p] = st[5]; c->g[p] = st[6];
        if (c->info.isTestParticle[s] || !(dt > 0)) continue;
        double p1[3] = {st[0], st[1], st[2]};
        const double coef = UNIT_RHOJ * c->info.charge_ratio[s] / vol / dt;
        vb_deposit(c, p0, p1, coef);
        absorbed_exit(c, p1, coef);
    }
}

/* rho alone at the particles' positions (the deposit's charge part). */
static void deposit_rho_only(orc_t *c) {
    double *save[3];
    double *tmp = (double *)malloc(sizeof(double) * 3 * (size_t)c->npts);
    for (int a = 0; a < 3; a++) {
        save[a] = c->slot[EMOO_JX + a];
        c->slot[EMOO_JX + a] = tmp + (size_t)a * c->npts;
    }
    deposit(c, 1);
    for (int a = 0; a < 3; a++) c->slot[EMOO_JX + a] = save[a];
    free(tmp);
}

/* Periodic copies and folds over the whole transverse range, dimension by
 * dimension (so edge and corner lines follow): the ghost planes 0, n+1, n+2
 * are the images of n, 1, 2. */
static void full_plane(orc_t *c, double *f, int dim, int src, int dst, int sum) {
    int o1 = (dim == 0) ? 1 : 0;
    int o2 = (dim == 2) ? 1 : 2;
    for (int p = 0; p < c->tot[o1]; p++)
        for (int q = 0; q < c->tot[o2]; q++) {
            int is[3], id_[3];
            is[dim] = src; id_[dim] = dst;
            is[o1] = id_[o1] = p;
            is[o2] = id_[o2] = q;
            if (sum) f[IDX(c, id_[0], id_[1], id_[2])] += f[IDX(c, is[0], is[1], is[2])];
            else f[IDX(c, id_[0], id_[1], id_[2])] = f[IDX(c, is[0], is[1], is[2])];
        }
}

/* Mirror fold at a reflecting wall (corrected policy; no reference
 * counterpart). A particle that crossed the wall during the push is
 * reflected (x -> 2 x_wall - x, v_n -> -v_n, src/boundaries/b_particles/
 * bc_p_reflecting.cpp:43-52), so it moved along the mirror image of the part
 * of its straight path that lies beyond the wall. The Villasenor-Buneman
 * current that part deposited in the ghost layer therefore belongs to the
 * mirrored points inside: the component normal to the wall with its sign
 * reversed, the transverse ones unchanged, and charge stays conserved at
 * every point. Left wall (vertex plane 1): normal edge 0 -> edge 1,
 * transverse plane 0 -> plane 2; right wall (plane n+1): normal edge n+1 ->
 * edge n, transverse plane n+2 -> plane n. The ghost values are cleared.
 * Whole transverse range, so corners follow the other dimensions' folds. */
static void mirror_fold(orc_t *c, int dim, int right) {
    const int n = c->n[dim];
    const int o1 = (dim == 0) ? 1 : 0, o2 = (dim == 2) ? 1 : 2;
    for (int a = 0; a < 3; a++) {
        double *f = c->slot[EMOO_JX + a];
        const int normal = a == dim;
        const int src = normal ? (right ? n + 1 : 0) : (right ? n + 2 : 0);
        const int dst = normal ? (right ? n : 1) : (right ? n : 2);
        for (int p = 0; p < c->tot[o1]; p++)
            for (int q = 0; q < c->tot[o2]; q++) {
                int is[3], id_[3];
                is[dim] = src; id_[dim] = dst;
                is[o1] = id_[o1] = p;
                is[o2] = id_[o2] = q;
                long ks = IDX(c, is[0], is[1], is[2]), kd = IDX(c, id_[0], id_[1], id_[2]);
                if (normal) f[kd] -= f[ks];
                else f[kd] += f[ks];
                f[ks] = 0.0;
            }
    }
}

static int dim_periodic(const orc_t *c, int dim) { return c->fbc[2 * dim] == BC_PERIODIC; }

/* Folds of the corrected policy: periodic dimensions as images over the
 * whole range; a reflecting wall mirrors its ghost current back; at an
 * absorbing wall the current of the path beyond it stays in the ghost layer
 * (it carried the charge out: continuity holds there too). */
static void corrected_fold(orc_t *c) {
    const int ids[4] = {EMOO_JX, EMOO_JY, EMOO_JZ, EMOO_RHO};
    for (int dim = 0; dim < 3; dim++) {
        int n = c->n[dim];
        if (!dim_periodic(c, dim)) {
            for (int r = 0; r < 2; r++)
                if (c->pbc[2 * dim + r] == BC_REFLECTING) mirror_fold(c, dim, r);
            continue;
        }
        for (int k = 0; k < 4; k++) {
            double *f = c->slot[ids[k]];
            full_plane(c, f, dim, 0, n, 1);
            full_plane(c, f, dim, n + 1, 1, 1);
            full_plane(c, f, dim, n + 2, 2, 1);
        }
    }
}

/* E's boundary values of the corrected policy: periodic images over the
 * whole range, LightBC planes on external sides (the latter at the step's
 * time, as the loop's executeBC(-1) sets them). */
static void corrected_e_bounds(orc_t *c) {
    for (int dim = 0; dim < 3; dim++) {
        if (!dim_periodic(c, dim)) continue;
        for (int a = 0; a < 3; a++) {
            double *f = c->slot[EMOO_EX + a];
            full_plane(c, f, dim, c->n[dim], 0, 0);
            full_plane(c, f, dim, 1, c->n[dim] + 1, 0);
            full_plane(c, f, dim, 2, c->n[dim] + 2, 0);
        }
    }
    for (int s = 0; s < 6; s++)
        if (c->fbc[s] == BC_EXTERNAL) light_bc(c, s, c->t, c->dtp);
}

static void corrected_ghosts(orc_t *c) {
    const int ids[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ, EMOO_BX_TM1, EMOO_BY_TM1, EMOO_BZ_TM1};
    for (int dim = 0; dim < 3; dim++) {
        int n = c->n[dim];
        if (!dim_periodic(c, dim)) continue;
        for (int k = 0; k < 9; k++) {
            double *f = c->slot[ids[k]];
            full_plane(c, f, dim, n, 0, 0);
            full_plane(c, f, dim, 1, n + 1, 0);
            full_plane(c, f, dim, 2, n + 2, 0);
        }
    }
    for (int s = 0; s < 6; s++)
        if (c->fbc[s] == BC_EXTERNAL) light_bc(c, s, c->t, c->dtp);
}

/* One pass of the driver loop, src/main.cpp:221-287 (history cadence of
 * src/IO/output.cpp:46,68-71: every 10 steps from step 0). */
int orc_step(void *h, int ti, long *counts6, double *hist8, int *hist_written) {
    orc_t *c = (orc_t *)h;
    if (c->policy) {
        if (c->info.nstep_sort > 0 && ti % c->info.nstep_sort == 0) orc_sort(c);
        *hist_written = 0;
        if (ti >= c->next_hist) {
            orc_history(c, c->t, hist8);
            c->next_hist += 10;
            *hist_written = 1;
        }
        push_vb(c, c->dtp);
        if (orc_particle_bc(c, counts6)) return -2;
        orc_clear_ghosts(c);
        deposit_rho_only(c);
        corrected_fold(c);
        if (c->info.electrostatic == 1) evolve_es(c, c->dtp);
        else evolve(c, c->dtp);
        corrected_ghosts(c);
        orc_interpolate(c);
        c->t += c->dtp;
        return 0;
    }
    if (c->info.nstep_sort > 0 && ti % c->info.nstep_sort == 0) orc_sort(c);
    *hist_written = 0;
    if (ti >= c->next_hist) {
        orc_history(c, c->t, hist8);
        c->next_hist += 10;
        *hist_written = 1;
    }
    push_all(c, c->dtp);
    if (orc_particle_bc(c, counts6)) return -2;
    orc_clear_ghosts(c);
    deposit(c, 1);
    orc_execute_bc(c, EMOO_SEND_JRHO);
    if (c->info.electrostatic == 1) evolve_es(c, c->dtp);
    else evolve(c, c->dtp);
    orc_execute_bc(c, EMOO_SEND_EB);
    orc_interpolate(c);
    c->t += c->dtp;
    return 0;
}

/* Particles [first, first + n) of the sampler stream g into caller arrays
 * (gamma may be null): bit-identical to the library's emoo_generate_host. */
int orc_generate(const emoo_gen_params *g, int64_t first, int64_t n, double *x, double *y, double *z, double *vx,
                 double *vy, double *vz, double *gamma) {
    if (!g || n < 0 || (n > 0 && (!x || !y || !z || !vx || !vy || !vz))) return EMOO_ERR_ARG;
    for (int64_t i = 0; i < n; i++) {
        double o[7];
        emoo_sample_particle(g, first + i, o);
        x[i] = o[0];
        y[i] = o[1];
        z[i] = o[2];
        vx[i] = o[3];
        vy[i] = o[4];
        vz[i] = o[5];
        if (gamma) gamma[i] = o[6];
    }
    return EMOO_OK;
}
