// api.cpp - the C ABI (include/emoo.h): handle lifecycle, particle upload and
// readback, boundary dispatch in the reference's order, and the time loop.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "emoo.h"
#include "emoo_internal.h"

using namespace emoo;

namespace emoo {

int cuda_status(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) return EMOO_ERR_OOM;
    fprintf(stderr, "emoo: CUDA error %d (%s)\n", (int)e, cudaGetErrorString(e));
    return EMOO_ERR_CUDA;
}

static bool is_pow2(double v) {
    int e;
    double m = frexp(v, &e);
    return m == 0.5;
}

void make_geom(const emoo_input_info &in, Geom &g) {
    for (int d = 0; d < 3; d++) {
        g.n[d] = in.nCell[d];
        g.tot[d] = in.nCell[d] + 3;
        g.x0[d] = in.xyz0[d];
        g.L[d] = in.Lxyz[d];
        g.d[d] = in.Lxyz[d] / in.nCell[d];  // src/grid/grid.cpp:37-39
        g.id[d] = 1.0 / g.d[d];             // src/grid/grid.cpp:40-42
        g.p2[d] = is_pow2(g.d[d]);
    }
    g.sy = g.tot[2];
    g.sx = (int64_t)g.tot[1] * g.tot[2];
    g.npts = (int64_t)g.tot[0] * g.sx;
    g.cnz = g.n[2] + 2;
    g.cny = (g.n[1] + 2) * (g.n[2] + 2);
    g.ncell = (int64_t)(g.n[0] + 2) * g.cny;
    g.vol = g.d[0] * g.d[1] * g.d[2];  // src/particles/deposit.cpp:20
    g.vol_p2 = is_pow2(g.vol);
    g.ivol = 1.0 / g.vol;
    for (int i = 0; i < 3; i++) {
        int j = (i + 1) % 3, k = (i + 2) % 3;
        g.area[i] = g.d[j] * g.d[k];
        g.area_p2[i] = is_pow2(g.area[i]);
        g.iarea[i] = 1.0 / g.area[i];
    }
}

// Queues the (start, stop) event pair of the timed kernel and takes a fresh
// pair for the next launch; the pairs are read by emoo_stats.
int prof_accumulate(emoo_handle *h) {
    h->prof_pending.push_back(h->prof_ev[0]);
    h->prof_pending.push_back(h->prof_ev[1]);
    for (int i = 0; i < 2; i++) {
        if (!h->prof_pool.empty()) {
            h->prof_ev[i] = h->prof_pool.back();
            h->prof_pool.pop_back();
        } else {
            EMOO_CUDA(cudaEventCreate(&h->prof_ev[i]));
        }
    }
    return EMOO_OK;
}

int read_err(emoo_handle *h) {
    DevCounters c;
    EMOO_CUDA(cudaMemcpyAsync(&c, h->ctr, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    unsigned long long zero = 0;
    EMOO_CUDA(cudaMemcpyAsync(&h->ctr->err, &zero, sizeof(zero), cudaMemcpyHostToDevice, h->stream));
    if (c.err & ERR_FIXED_OVERFLOW) return EMOO_ERR_FIXED_OVERFLOW;
    if (c.err & ERR_BOUNDS) return EMOO_ERR_BOUNDS;
    return EMOO_OK;
}

}  // namespace emoo

namespace {

struct Pulses {
    int nw;
    double amp[EMOO_NWAVE], omg[EMOO_NWAVE], pha[EMOO_NWAVE], del[EMOO_NWAVE], iw[EMOO_NWAVE];
    int wid[EMOO_NWAVE];  // input index of each wave
};

// LightBC host state per handle (src/grid/lightBC.cpp:10-142), computed on
// the host with the same libm calls as the reference.
struct LightState {
    Pulses p[6][3];
};

std::vector<std::pair<emoo_handle *, LightState>> &light_registry() {
    static std::vector<std::pair<emoo_handle *, LightState>> r;
    return r;
}

LightState *light_of(emoo_handle *h) {
    for (auto &e : light_registry())
        if (e.first == h) return &e.second;
    return nullptr;
}

// Sine-series envelope of a shaped wave: sum_k coef[k-1] sin(k pi a),
// a = (t - t_start) / window, inside the window and 0 outside.
double sine_envelope(const emoo_wave_shape &sh, double t) {
    if (!(t >= sh.t_start && t <= sh.t_start + sh.window)) return 0.0;
    const double a = (t - sh.t_start) / sh.window;
    double e = 0.0;
    for (int k = 1; k <= sh.ncoef; k++) e += sh.coef[k - 1] * sin(k * PI_D * a);
    return e;
}

const emoo_wave_shape *shape_of(const emoo_handle *h, int w) { return h->wshaped[w] ? &h->wshape[w] : nullptr; }

// GaussianPulses, src/utils/evaluateGaussianPulse.cpp:7-30, over the waves of
// one side and polarisation; a shaped wave takes its sine-series envelope in
// place of the Gaussian. Terms of waves with a transverse spot are summed
// into *spot, the others into the return value (so that without spots the
// sum is the reference's, term by term).
double light_sum(const emoo_handle *h, const Pulses &P, double t, double dt, double *spot) {
    double val = 0.0, sv = 0.0;
    for (int i = 0; i < P.nw; i++) {
        const emoo_wave_shape *sh = shape_of(h, P.wid[i]);
        double tmp = P.amp[i] * cos(P.omg[i] * (t + dt) + P.pha[i] * PI_D / 180.0);
        const double env = (sh && sh->ncoef > 0) ? sine_envelope(*sh, t) : exp(-pow((t - P.del[i]) * P.iw[i], 2));
        if (sh && sh->waist > 0) sv += tmp * env;
        else val += tmp * env;
    }
    *spot = sv;
    return val;
}

// Spot factor tables of side s, E component p (null when it has no spot).
const double *spot_table(const emoo_handle *h, int s, int p, int a) {
    return h->wspot[s][p] ? h->wprof + (size_t)((3 * s + p) * 2 + a) * h->wprof_stride : nullptr;
}
const float *spot_table_f(const emoo_handle *h, int s, int p, int a) {
    return h->wspot[s][p] ? h->wproff + (size_t)((3 * s + p) * 2 + a) * h->wprof_stride : nullptr;
}

int edge_plane(const Geom &g, bool isB, int comp, int dim, bool right) {
    if (!right) return 1;
    bool along = comp == dim;
    if (!isB) return along ? g.n[dim] : g.n[dim] + 1;
    return along ? g.n[dim] + 1 : g.n[dim];
}

// LightBC::applyBCs, src/grid/lightBC.cpp:165-200: six whole-plane writes per
// external side, E through the E storage, B through the current B role.
int light_planes(emoo_handle *h, int s, PlaneSet *ps, bool slots) {
    LightState *L = light_of(h);
    static const int EPOL[3][3] = {{1, 2, 0}, {2, 0, 1}, {0, 1, 2}};
    static const int BPOL[3][3] = {{2, 1, 0}, {0, 2, 1}, {1, 0, 2}};
    int dim = s / 2;
    bool right = (s % 2) == 1;
    int sign = right ? 1 : -1;
    double E1[3], B1[3];
    for (int i = 0; i < 3; i++) {
        E1[i] = h->info.E0[i];
        B1[i] = h->info.B0[i];
    }
    double dx = h->g.d[dim];
    double bphase = (dx + sign * h->dtp) / 2;
    int n = 0;
    for (int i = 0; i < 3; i++) {
        int eid = EPOL[dim][i], bid = BPOL[dim][i];
        double es = 0.0, bs = 0.0;  // spot parts
        if (L && L->p[s][eid].nw > 0 && eid != dim) {
            double ev = light_sum(h, L->p[s][eid], h->t, 0.0, &es);
            E1[eid] += ev;
            int bsign = sign * (int)pow(-1, i + 1);
            double bsp;
            double bv = bsign * light_sum(h, L->p[s][eid], h->t, bphase, &bsp);
            B1[bid] += bv;
            bs = bsign * bsp;
        }
        // the B component paired with E component eid sits at the same
        // transverse offsets, so both take side s / component eid's factors
        const int sp = eid != dim ? eid : -1;
        const double *t1 = sp >= 0 ? spot_table(h, s, sp, 0) : nullptr;
        const double *t2 = sp >= 0 ? spot_table(h, s, sp, 1) : nullptr;
        const float *t1f = sp >= 0 ? spot_table_f(h, s, sp, 0) : nullptr;
        const float *t2f = sp >= 0 ? spot_table_f(h, s, sp, 1) : nullptr;
        const int ie = edge_plane(h->g, false, eid, dim, right), ib = edge_plane(h->g, true, bid, dim, right);
        if (slots) {
            ps[n++] = PlaneSet{h->slot[EMOO_EX + eid], dim, ie, E1[eid], es, t1, t2, t1f, t2f};
            double *bp = h->bswap ? h->slot[EMOO_BX_TM1 + bid] : h->slot[EMOO_BX + bid];
            ps[n++] = PlaneSet{bp, dim, ib, B1[bid], bs, t1, t2, t1f, t2f};
        } else {
            // mixed form: slot index in f, resolved by the mixed plane-set launcher
            ps[n++] = PlaneSet{(double *)(intptr_t)(EMOO_EX + eid), dim, ie, E1[eid], es, t1, t2, t1f, t2f};
            ps[n++] = PlaneSet{(double *)(intptr_t)(EMOO_BX + bid), dim, ib, B1[bid], bs, t1, t2, t1f, t2f};
        }
    }
    return n;
}

// The pulses of each external side and polarisation (LightBC's constructor,
// src/grid/lightBC.cpp:10-142).
LightState build_light(const emoo_input_info &info) {
    LightState L;
    memset(&L, 0, sizeof(L));
    for (int s = 0; s < 6; s++) {
        int side = (s % 2 == 0) ? -(s / 2 + 1) : (s / 2 + 1);
        for (int w = 0; w < info.nwaves && w < EMOO_NWAVE; w++) {
            if (info.inSide[w] != side) continue;
            int pid = info.inPolE[w] - 1;
            if (pid < 0 || pid > 2) continue;
            Pulses &P = L.p[s][pid];
            P.amp[P.nw] = info.peakamps[w];
            P.omg[P.nw] = info.omegas[w];
            P.pha[P.nw] = info.phases[w];
            P.del[P.nw] = info.delays[w];
            P.iw[P.nw] = info.invWidths[w];
            P.wid[P.nw] = w;
            P.nw++;
        }
    }
    return L;
}

// d/d(amplitude), d/d(phase in degrees) and, for a sine-series envelope,
// d/d(coef[k]) of wave w's term amp cos(omega (t + dt) + phase pi / 180)
// env(t), times scale; appended to the op's spot list when the wave has a
// spot, to its uniform list otherwise.
void pulse_derivs(const emoo_handle *h, int w, double t, double dt, double scale, AdBcOp &op) {
    const emoo_input_info &in = h->info;
    const emoo_wave_shape *sh = shape_of(h, w);
    const bool series = sh && sh->ncoef > 0;
    const double arg = in.omegas[w] * (t + dt) + in.phases[w] * PI_D / 180.0;
    const double env = series ? sine_envelope(*sh, t) : exp(-pow((t - in.delays[w]) * in.invWidths[w], 2));
    const bool spot = sh && sh->waist > 0;
    std::vector<int> &K = spot ? op.ks : op.ku;
    std::vector<double> &C = spot ? op.cs : op.cu;
    K.push_back(2 * w);
    C.push_back(scale * cos(arg) * env);
    K.push_back(2 * w + 1);
    C.push_back(-scale * in.peakamps[w] * sin(arg) * (PI_D / 180.0) * env);
    if (series && t >= sh->t_start && t <= sh->t_start + sh->window) {
        const double a = (t - sh->t_start) / sh->window;
        for (int k = 1; k <= sh->ncoef; k++) {
            K.push_back(2 * in.nwaves + EMOO_NCOEF * w + k - 1);
            C.push_back(scale * in.peakamps[w] * cos(arg) * sin(k * PI_D * a));
        }
    }
}

}  // namespace

int emoo::light_planes_public(emoo_handle *h, int s, PlaneSet *ps) { return light_planes(h, s, ps, false); }
int emoo::light_planes_slots(emoo_handle *h, int s, PlaneSet *ps) { return light_planes(h, s, ps, true); }

namespace {
int do_sort(emoo_handle *h);  // below
}

// Sorts the store by cell (dropping removed particles); perm_out (device,
// the store's size before the call) receives perm[i] = the index before the
// sort of the i-th particle after it.
int emoo::sort_with_permutation(emoo_handle *h, uint32_t *perm_out) {
    const int64_t n = h->np;
    EMOO_TRY(do_sort(h));
    if (n) EMOO_CUDA(cudaMemcpyAsync(perm_out, h->perm[0], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->stream));
    return EMOO_OK;
}

namespace {
int execute_bc(emoo_handle *h, int send_id);  // below
}

int emoo::ad_execute_bc(emoo_handle *h, int send_id) { return execute_bc(h, send_id); }

// executeBC(-1) on the FP64 slots as a list of operations, at the handle's
// current time and B roles, in the order execute_bc_slots applies them; each
// plane carries its value's derivatives with respect to the wave parameters.
int emoo::ad_bc_ops(emoo_handle *h, std::vector<AdBcOp> &ops) {
    static const int EPOL[3][3] = {{1, 2, 0}, {2, 0, 1}, {0, 1, 2}};  // as light_planes
    ops.clear();
    const emoo_input_info &in = h->info;
    int mask = 0;
    for (int d = 0; d < 3; d++) {
        if (h->bc.fbc[2 * d] == FBC_PERIODIC) {
            mask |= 1 << d;
            continue;
        }
        if (mask) {
            AdBcOp g{};
            g.kind = 0;
            g.mask = mask;
            ops.push_back(g);
            mask = 0;
        }
        for (int r = 0; r < 2; r++) {
            const int s = 2 * d + r;
            if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
            PlaneSet ps[6];
            const int n = light_planes(h, s, ps, true);
            const int side = (s % 2 == 0) ? -(s / 2 + 1) : (s / 2 + 1);
            const int sign = r ? 1 : -1;
            const double bphase = (h->g.d[d] + sign * h->dtp) / 2;
            for (int i = 0; i < n; i++) {
                AdBcOp op{};
                op.kind = 1;
                op.slot = -1;
                for (int k = 0; k < EMOO_NFIELDS; k++)
                    if (h->slot[k] == ps[i].f) op.slot = k;
                if (op.slot < 0) return EMOO_ERR_STATE;
                op.dim = ps[i].dim;
                op.idx = ps[i].idx;
                op.value = ps[i].v;
                op.vs = ps[i].vs;
                op.t1 = ps[i].t1;
                op.t2 = ps[i].t2;
                const int c = i / 2;
                const int eid = EPOL[d][c];
                if (eid != d) {
                    for (int w = 0; w < in.nwaves && w < EMOO_NWAVE; w++) {
                        if (in.inSide[w] != side || in.inPolE[w] - 1 != eid) continue;
                        if (i % 2 == 0) pulse_derivs(h, w, h->t, 0.0, 1.0, op);
                        else pulse_derivs(h, w, h->t, bphase, sign * (int)pow(-1, c + 1), op);
                    }
                }
                ops.push_back(op);
            }
        }
    }
    if (mask) {
        AdBcOp g{};
        g.kind = 0;
        g.mask = mask;
        ops.push_back(g);
    }
    return EMOO_OK;
}

namespace {

int bc_kind_particle(const char *s) {
    if (strcmp(s, "periodic") == 0) return PBC_PERIODIC;
    if (strcmp(s, "reflecting") == 0) return PBC_REFLECTING;
    if (strcmp(s, "absorbing") == 0) return PBC_ABSORBING;
    return -1;
}

int bc_kind_field(const char *s) {
    if (strcmp(s, "periodic") == 0) return FBC_PERIODIC;
    if (strcmp(s, "external") == 0) return FBC_EXTERNAL;
    return -1;
}

int set_device(emoo_handle *h) {
    EMOO_CUDA(cudaSetDevice(h->dev));
    return EMOO_OK;
}

template <typename T>
int dalloc(T *&p, size_t n) {
    p = nullptr;
    if (n == 0) n = 1;
    EMOO_CUDA(cudaMalloc(&p, n * sizeof(T)));
    return EMOO_OK;
}

template <typename T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

void free_particles(emoo_handle *h) {
    dfree(h->x); dfree(h->y); dfree(h->z); dfree(h->vx); dfree(h->vy); dfree(h->vz); dfree(h->gam);
    dfree(h->ids); dfree(h->fcache);
    dfree(h->cell); dfree(h->ox); dfree(h->oy); dfree(h->oz); dfree(h->ux); dfree(h->uy); dfree(h->uz);
    dfree(h->key[0]); dfree(h->key[1]); dfree(h->perm[0]); dfree(h->perm[1]);
    dfree(h->g0);
    if (h->pay) cudaFree(h->pay);
    h->pay = nullptr;
    if (h->pay4) cudaFree(h->pay4);
    h->pay4 = nullptr;
}

// Particle storage for `cap` particles; existing content is preserved.
int reserve(emoo_handle *h, int64_t cap) {
    if (cap <= h->cap) return EMOO_OK;
    if (cap >= (int64_t)UINT32_MAX - 2) return EMOO_ERR_OOM;
    int64_t np = h->np;
    auto grow = [&](auto *&p, bool want) -> int {
        using T = std::remove_reference_t<decltype(*p)>;
        if (!want) return EMOO_OK;
        T *q = nullptr;
        EMOO_TRY(dalloc(q, (size_t)cap));
        if (p && np) EMOO_CUDA(cudaMemcpyAsync(q, p, sizeof(T) * (size_t)np, cudaMemcpyDeviceToDevice, h->stream));
        if (p) cudaFree(p);
        p = q;
        return EMOO_OK;
    };
    bool f64 = h->precision == EMOO_FP64;
    EMOO_TRY(grow(h->x, f64)); EMOO_TRY(grow(h->y, f64)); EMOO_TRY(grow(h->z, f64));
    EMOO_TRY(grow(h->vx, f64)); EMOO_TRY(grow(h->vy, f64)); EMOO_TRY(grow(h->vz, f64));
    EMOO_TRY(grow(h->gam, f64));
    EMOO_TRY(grow(h->cell, !f64)); EMOO_TRY(grow(h->ox, !f64)); EMOO_TRY(grow(h->oy, !f64)); EMOO_TRY(grow(h->oz, !f64));
    EMOO_TRY(grow(h->ux, !f64)); EMOO_TRY(grow(h->uy, !f64)); EMOO_TRY(grow(h->uz, !f64));
    EMOO_TRY(grow(h->ids, h->opts.track_ids != 0));
    EMOO_TRY(grow(h->g0, h->g0 != nullptr));
    dfree(h->fcache);
    dfree(h->key[0]); dfree(h->key[1]); dfree(h->perm[0]); dfree(h->perm[1]);
    EMOO_TRY(dalloc(h->key[0], (size_t)cap)); EMOO_TRY(dalloc(h->key[1], (size_t)cap));
    EMOO_TRY(dalloc(h->perm[0], (size_t)cap)); EMOO_TRY(dalloc(h->perm[1], (size_t)cap));
    if (h->pay) cudaFree(h->pay);
    h->pay = nullptr;
    if (h->pay4) cudaFree(h->pay4);
    h->pay4 = nullptr;
    // scratch of one array per element size: cap 8-byte elements (also the
    // staging area of the loaders, 7 doubles per particle in chunks) and cap
    // 4-byte elements; the sort swaps each array with the buffer of its size
    h->pay_bytes = sizeof(double) * (size_t)cap;
    EMOO_CUDA(cudaMalloc(&h->pay, h->pay_bytes));
    EMOO_CUDA(cudaMalloc(&h->pay4, sizeof(float) * (size_t)cap));
    h->cap = cap;
    return EMOO_OK;
}

}  // namespace

int emoo::reserve_store(emoo_handle *h, int64_t cap) { return reserve(h, cap); }

namespace {

// Opens a gap of n particles at the end of species s's segment and returns
// its start index.
int make_room(emoo_handle *h, int s, int64_t n, int64_t *at) {
    if (h->np + n > h->cap) EMOO_TRY(reserve(h, std::max(h->np + n, h->cap + h->cap / 2)));
    int64_t pos = h->off[s + 1];
    int64_t tail = h->np - pos;
    if (tail > 0) {
        auto shift = [&](auto *p) -> int {
            using T = std::remove_reference_t<decltype(*p)>;
            if (!p) return EMOO_OK;
            T *tmp = (T *)h->pay;
            EMOO_CUDA(cudaMemcpyAsync(tmp, p + pos, sizeof(T) * (size_t)tail, cudaMemcpyDeviceToDevice, h->stream));
            EMOO_CUDA(cudaMemcpyAsync(p + pos + n, tmp, sizeof(T) * (size_t)tail, cudaMemcpyDeviceToDevice, h->stream));
            return EMOO_OK;
        };
        EMOO_TRY(shift(h->x)); EMOO_TRY(shift(h->y)); EMOO_TRY(shift(h->z));
        EMOO_TRY(shift(h->vx)); EMOO_TRY(shift(h->vy)); EMOO_TRY(shift(h->vz)); EMOO_TRY(shift(h->gam));
        EMOO_TRY(shift(h->cell)); EMOO_TRY(shift(h->ox)); EMOO_TRY(shift(h->oy)); EMOO_TRY(shift(h->oz));
        EMOO_TRY(shift(h->ux)); EMOO_TRY(shift(h->uy)); EMOO_TRY(shift(h->uz)); EMOO_TRY(shift(h->ids));
        EMOO_TRY(shift(h->g0));
    }
    for (int q = s + 1; q <= h->nspec; q++) h->off[q] += n;
    h->count[s] += n;
    h->np += n;
    *at = pos;
    return EMOO_OK;
}

__attribute__((unused)) int sync(emoo_handle *h) {
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int key_bits(emoo_handle *h) {
    uint64_t maxkey = (uint64_t)h->nspec * (uint64_t)h->g.ncell + 2;
    int b = 1;
    while ((1ull << b) <= maxkey) b++;
    return b;
}

int do_sort(emoo_handle *h) {
    if (h->np == 0) return EMOO_OK;
    if (h->precision == EMOO_FP64) EMOO_TRY(sort_keys_f64(h));
    else EMOO_TRY(mixed_sort_keys(h));
    bool f64 = h->precision == EMOO_FP64;
    EMOO_TRY(radix_sort_perm(h, h->np, f64 ? key_bits(h) : mixed_key_bits(h)));
    EMOO_TRY(gather_payload(h, h->np, !f64));
    int64_t cnt[EMOO_NSPEC];
    EMOO_TRY(count_species(h, h->np, f64 ? h->g.ncell : h->g.npts, cnt));
    int64_t off = 0;
    for (int s = 0; s < h->nspec; s++) {
        h->off[s] = off;
        h->count[s] = cnt[s];
        off += cnt[s];
    }
    h->off[h->nspec] = off;
    h->np = off;
    h->dead_pending = 0;
    dfree(h->fcache);
    return EMOO_OK;
}

// Drops the particles absorbing walls removed since the last sort, keeping
// each species' order: a stable sort by (species, removed) keys.
int compact(emoo_handle *h) {
    if (!h->dead_pending || h->np == 0) {
        h->dead_pending = 0;
        return EMOO_OK;
    }
    if (h->precision == EMOO_FP64) EMOO_TRY(compact_keys_f64(h));
    else EMOO_TRY(mixed_compact_keys(h));
    int bits = 1;
    while ((1 << bits) <= h->nspec) bits++;
    EMOO_TRY(radix_sort_perm(h, h->np, bits));
    EMOO_TRY(gather_payload(h, h->np));
    int64_t cnt[EMOO_NSPEC];
    EMOO_TRY(count_species(h, h->np, 1, cnt));
    int64_t off = 0;
    for (int s = 0; s < h->nspec; s++) {
        h->off[s] = off;
        h->count[s] = cnt[s];
        off += cnt[s];
    }
    h->off[h->nspec] = off;
    h->np = off;
    h->dead_pending = 0;
    dfree(h->fcache);
    return EMOO_OK;
}

bool has_absorbing(const emoo_handle *h) {
    for (int s = 0; s < 6; s++)
        if (h->bc.pbc[s] == PBC_ABSORBING) return true;
    return false;
}

int execute_bc(emoo_handle *h, int send_id);

int deposit_all(emoo_handle *h, int with_rho) {
    if (h->precision != EMOO_FP64) return mixed_deposit(h, with_rho);
    EMOO_TRY(deposit_f64(h, with_rho));
    return EMOO_OK;
}

int execute_bc_slots(emoo_handle *h, int send_id);

int poisson_init(emoo_handle *h, int iters[4]) {
    if (!h->poisson) return EMOO_ERR_STATE;
    // src/poisson/poisson.cpp:98-156: tolerances from the Dirichlet values
    const emoo_input_info &in = h->info;
    double vmax = in.bound_phi[0], vmin = in.bound_phi[0];
    for (int i = 0; i < 6; i++) {
        vmax = std::max(vmax, in.bound_phi[i]);
        vmin = std::min(vmin, in.bound_phi[i]);
    }
    double conv_phi = vmax - vmin;
    vmax = vmin = in.bound_Ax[0];
    for (int i = 0; i < 6; i++) {
        double a[3] = {in.bound_Ax[i], in.bound_Ay[i], in.bound_Az[i]};
        for (double v : a) {
            vmax = std::max(vmax, v);
            vmin = std::min(vmin, v);
        }
    }
    double conv_A = vmax - vmin;
    double mult = -4 * PI_D;
    double tol = std::max(conv_phi * CONV_RATIO, CONV_CRIT);
    int it[4] = {0, 0, 0, 0}, cv, ok = 1;
    if (h->poisson_solver == EMOO_POISSON_MULTIGRID) {
        // the same four solves, phiToE after the first and AToB after the last
        for (int q = 0; q < 4; q++) {
            EMOO_TRY(multigrid_f64(h, q == 0 ? EMOO_PHI1 : EMOO_AX1 + (q - 1), q == 0 ? EMOO_PHI2 : EMOO_AX2 + (q - 1),
                                   q == 0 ? EMOO_RHO : EMOO_JX + (q - 1), mult, &it[q], &cv));
            ok &= cv;
            if (q == 0) EMOO_TRY(phi_to_e_f64(h));
        }
        EMOO_TRY(a_to_b_f64(h));
        EMOO_TRY(execute_bc_slots(h, EMOO_SEND_EB));
        if (h->precision != EMOO_FP64) EMOO_TRY(mixed_fields_from_slots(h));
        if (iters)
            for (int q = 0; q < 4; q++) iters[q] = it[q];
        return ok ? EMOO_OK : EMOO_ERR_NOT_CONVERGED;
    }
    EMOO_TRY(jacobi_f64(h, EMOO_PHI1, EMOO_PHI2, EMOO_RHO, tol, mult, &it[0], &cv));
    ok &= it[0] < ITER_MAX;
    EMOO_TRY(phi_to_e_f64(h));
    tol = std::max(conv_A * CONV_RATIO, CONV_CRIT);
    for (int q = 0; q < 3; q++) {
        EMOO_TRY(jacobi_f64(h, EMOO_AX1 + q, EMOO_AX2 + q, EMOO_JX + q, tol, mult, &it[1 + q], &cv));
        ok &= it[1 + q] < ITER_MAX;
    }
    EMOO_TRY(a_to_b_f64(h));
    EMOO_TRY(execute_bc_slots(h, EMOO_SEND_EB));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_fields_from_slots(h));
    if (iters)
        for (int q = 0; q < 4; q++) iters[q] = it[q];
    return ok ? EMOO_OK : EMOO_ERR_NOT_CONVERGED;
}

// Grid::InitializeFields, src/grid/grid.cpp:554-574
int const_init(emoo_handle *h) {
    const emoo_input_info &in = h->info;
    bool cst = in.restart == 0 && strcmp(in.fields_init, "constant") == 0;
    int64_t n = h->g.npts;
    if (h->precision != EMOO_FP64) {
        if (!cst) {  // constJ(0,0,0), constRho(0)
            for (int c = 0; c < 4; c++) {
                EMOO_TRY(fill_f64(h, h->slot[EMOO_JX + c], n, 0.0, h->stream));
                EMOO_TRY(mixed_set_field(h, EMOO_JX + c, h->slot[EMOO_JX + c]));
            }
        }
        return mixed_const_fields(h);
    }
    if (!cst) {
        for (int q = 0; q < 3; q++) EMOO_TRY(fill_f64(h, h->slot[EMOO_JX + q], n, 0.0, h->stream));
        EMOO_TRY(fill_f64(h, h->slot[EMOO_RHO], n, 0.0, h->stream));
    }
    for (int q = 0; q < 3; q++) {
        EMOO_TRY(fill_f64(h, h->slot[EMOO_EX + q], n, in.E0[q], h->stream));
        // constB sets both the B and B_tm1 members (src/grid/grid.cpp:523-530)
        EMOO_TRY(fill_f64(h, h->slot[EMOO_BX + q], n, in.B0[q], h->stream));
        EMOO_TRY(fill_f64(h, h->slot[EMOO_BX_TM1 + q], n, in.B0[q], h->stream));
    }
    return EMOO_OK;
}

// Grid::executeBC(sendID), src/grid/grid.cpp:577-585: dimensions in order,
// left then right; periodic ghost copies of consecutive periodic dimensions
// are independent and issued as one launch.
int execute_bc(emoo_handle *h, int send_id) {
    if (h->precision != EMOO_FP64) {
        if (send_id == EMOO_SEND_EB) return mixed_ghost_fill(h);
        if (send_id == EMOO_SEND_JRHO) return mixed_fold_public(h);
        // single fields (Poisson potentials) live on the FP64 slots
    }
    return execute_bc_slots(h, send_id);
}

// executeBC on the FP64 grid slots.
int execute_bc_slots(emoo_handle *h, int send_id) {
    if (h->policy == EMOO_POLICY_CORRECTED && send_id == EMOO_SEND_JRHO) return fold_full_f64(h, FOLD_ALL);
    if (h->policy == EMOO_POLICY_CORRECTED && send_id == EMOO_SEND_EB) return ghost_full_f64(h);
    if (send_id == EMOO_SEND_JRHO) {
        for (int d = 0; d < 3; d++)
            if (h->bc.fbc[2 * d] == FBC_PERIODIC) EMOO_TRY(fold_f64(h, d));
        return EMOO_OK;
    }
    if (send_id < EMOO_SEND_JRHO || send_id >= EMOO_NFIELDS) return EMOO_ERR_ARG;
    // fields the ghost copy touches: through the field pointer table (fixed slots)
    int ids_eb[6] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ};
    const int *ids = send_id == EMOO_SEND_EB ? ids_eb : &send_id;
    int nids = send_id == EMOO_SEND_EB ? 6 : 1;
    int mask = 0;
    for (int d = 0; d < 3; d++) {
        if (h->bc.fbc[2 * d] == FBC_PERIODIC) {
            mask |= 1 << d;
            continue;
        }
        if (mask) {
            EMOO_TRY(ghost_fill_f64(h, ids, nids, mask));
            mask = 0;
        }
        for (int r = 0; r < 2; r++) {
            int s = 2 * d + r;
            if (h->bc.fbc[s] != FBC_EXTERNAL) continue;
            if (send_id == EMOO_SEND_EB) {
                PlaneSet ps[6];
                int n = light_planes(h, s, ps, true);
                EMOO_TRY(plane_set_f64(h, ps, n));
            } else if (h->poisson && send_id > 0) {
                int id = send_id;
                int fid = (id == EMOO_PHI1 || id == EMOO_PHI2) ? 0 : (id == EMOO_AX1 || id == EMOO_AX2) ? 1
                          : (id == EMOO_AY1 || id == EMOO_AY2) ? 2 : (id == EMOO_AZ1 || id == EMOO_AZ2) ? 3 : -1;
                if (fid < 0) return EMOO_ERR_ARG;  // the reference asserts here (poissonBC.cpp:226)
                double v = fid == 0 ? h->info.bound_phi[s] : fid == 1 ? h->info.bound_Ax[s]
                                    : fid == 2 ? h->info.bound_Ay[s] : h->info.bound_Az[s];
                PlaneSet p{h->slot[id], d, r == 0 ? 1 : h->g.n[d] + 1, v};
                EMOO_TRY(plane_set_f64(h, &p, 1));
            }
        }
    }
    if (mask) EMOO_TRY(ghost_fill_f64(h, ids, nids, mask));
    return EMOO_OK;
}

// The history row from the particle moments and field energies.
void history_from(const emoo_handle *h, const double m4[4], const double e6[6], double out8[8]) {
    double B_en = e6[3] + e6[4] + e6[5];
    double E_en = e6[0] + e6[1] + e6[2];
    out8[0] = h->t;
    out8[1] = m4[1];
    out8[2] = m4[2];
    out8[3] = m4[3];
    out8[4] = m4[0];
    out8[5] = B_en;
    out8[6] = E_en;
    out8[7] = B_en + E_en + m4[0];
}

int history_row(emoo_handle *h, double out8[8]) {
    double m4[4], e6[6];
    if (h->precision == EMOO_FP64) {
        EMOO_TRY(particle_moments_f64(h, m4));
        EMOO_TRY(field_energy_f64(h, e6));
    } else {
        EMOO_TRY(mixed_moments(h, m4));
        EMOO_TRY(mixed_field_energy(h, e6));
    }
    history_from(h, m4, e6, out8);
    return EMOO_OK;
}

int reset_counters(emoo_handle *h) {
    EMOO_CUDA(cudaMemsetAsync(h->ctr, 0, sizeof(DevCounters), h->stream));
    return EMOO_OK;
}

int read_counters(emoo_handle *h, int64_t *counts6, bool accumulate) {
    DevCounters c;
    EMOO_CUDA(cudaMemcpyAsync(&c, h->ctr, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    if (counts6)
        for (int s = 0; s < 6; s++) counts6[s] = (accumulate ? counts6[s] : 0) + (int64_t)c.cross[s];
    if (c.err & ERR_FIXED_OVERFLOW) return EMOO_ERR_FIXED_OVERFLOW;
    if (c.err & ERR_BOUNDS) return EMOO_ERR_BOUNDS;
    return EMOO_OK;
}

// Every entry point: the handle's device current, and the device particle
// store refreshed from host-resident arrays if a streamed step left it stale.
#define HANDLE_CHECK(h)                      \
    do {                                     \
        if (!(h)) return EMOO_ERR_ARG;       \
        EMOO_TRY(set_device(h));             \
        EMOO_TRY(host_store_sync(h));        \
    } while (0)

// Entry points that change the particle store: not while the particles are
// host-resident (emoo_detach_particles first).
#define STORE_WRITE_CHECK(h)                               \
    do {                                                   \
        if ((h)->host_mode) return EMOO_ERR_STATE;         \
    } while (0)

}  // namespace

namespace emoo {

// The attached arrays into the device store (the loader's conversion).
static int host_upload(emoo_handle *h) {
    for (int s = 0; s < h->nspec; s++) {
        const emoo_handle::Attached &a = h->attached[s];
        if (h->count[s] > 0)
            EMOO_TRY(mixed_from_f64(h, h->off[s], h->count[s], a.p[0], a.p[1], a.p[2], a.p[3], a.p[4], a.p[5],
                                    a.p[6]));
    }
    h->store_stale = 0;
    if (h->opts.deposit_rho) h->rho_stale = 1;  // rho follows the store
    return EMOO_OK;
}

// The device store into the attached arrays (the readback's conversion).
static int host_download(emoo_handle *h) {
    for (int s = 0; s < h->nspec; s++) {
        const emoo_handle::Attached &a = h->attached[s];
        if (h->count[s] > 0)
            EMOO_TRY(mixed_to_f64(h, h->off[s], h->count[s], a.p[0], a.p[1], a.p[2], a.p[3], a.p[4], a.p[5],
                                  a.p[6]));
    }
    return EMOO_OK;
}

int host_store_sync(emoo_handle *h) {
    if (!h->host_mode || !h->store_stale) return EMOO_OK;
    return host_upload(h);
}

}  // namespace emoo

extern "C" {

int emoo_default_opts(emoo_opts *o) {
    if (!o) return EMOO_ERR_ARG;
    memset(o, 0, sizeof(*o));
    o->precision = EMOO_FP64;
    o->device = 0;
    o->dt = 0.0;
    o->capacity = 0;
    o->track_ids = 1;
    o->deposit_rho = 1;
    o->history_every = 10;
    o->rho_background = 0.0;
    o->rho_background_xmin = -HUGE_VAL;
    o->poisson_solver = EMOO_POISSON_JACOBI;
    o->poisson_rtol = 1e-10;
    return EMOO_OK;
}

const char *emoo_strerror(int s) {
    switch (s) {
        case EMOO_OK: return "ok";
        case EMOO_ERR_ARG: return "bad argument";
        case EMOO_ERR_OOM: return "out of memory or capacity";
        case EMOO_ERR_NOT_CONVERGED: return "Poisson solve did not converge (Jacobi iteration cap or multigrid cycle cap)";
        case EMOO_ERR_FIXED_OVERFLOW: return "fixed-point accumulator saturated";
        case EMOO_ERR_BOUNDS: return "device bounds check failed";
        case EMOO_ERR_CUDA: return "CUDA runtime error";
        case EMOO_ERR_INPUT: return "input error";
        case EMOO_ERR_STATE: return "invalid call for the handle state";
        case EMOO_ERR_UNSUPPORTED: return "unsupported option combination";
        default: return "unknown status";
    }
}

int emoo_create(const emoo_input_info *info, const emoo_opts *opts, emoo_handle **out) {
    if (!info || !out) return EMOO_ERR_ARG;
    *out = nullptr;
    emoo_opts o;
    if (opts) o = *opts;
    else emoo_default_opts(&o);
    if (o.precision != EMOO_FP64 && o.precision != EMOO_MIXED) return EMOO_ERR_ARG;
    if (!std::isfinite(o.rho_background) || std::isnan(o.rho_background_xmin)) return EMOO_ERR_ARG;
    if (info->nspecies < 0 || info->nspecies > EMOO_NSPEC) return EMOO_ERR_ARG;
    for (int d = 0; d < 3; d++)
        if (info->nCell[d] < 1 || !(info->Lxyz[d] > 0)) return EMOO_ERR_ARG;
    int pbc[6], fbc[6];
    for (int s = 0; s < 6; s++) {
        pbc[s] = bc_kind_particle(info->parts_bound[s]);
        fbc[s] = bc_kind_field(info->fields_bound[s]);
        if (pbc[s] < 0 || fbc[s] < 0) return EMOO_ERR_INPUT;  // the reference throws "Unable to find ... boundary"
    }
    for (int d = 0; d < 3; d++)
        if ((fbc[2 * d] == FBC_PERIODIC) != (fbc[2 * d + 1] == FBC_PERIODIC)) return EMOO_ERR_INPUT;
    emoo_handle *h = new (std::nothrow) emoo_handle();
    if (!h) return EMOO_ERR_OOM;
    h->info = *info;
    h->opts = o;
    h->dev = o.device;
    h->precision = o.precision;
    if (h->opts.history_every <= 0) h->opts.history_every = 10;
    int rc = set_device(h);
    if (rc) {
        delete h;
        return rc;
    }
    make_geom(*info, h->g);
    for (int s = 0; s < 6; s++) {
        h->bc.pbc[s] = pbc[s];
        h->bc.fbc[s] = fbc[s];
    }
    for (int d = 0; d < 3; d++) {
        // Domain::xyz0_ = x0 + L * 0 (src/domain/domain.cpp:96-99); BC limits
        // xMin_ and xMin_ + L (bc_p_periodic.cpp:79-80)
        h->bc.xmin[d] = info->xyz0[d] + info->Lxyz[d] * 0;
        h->bc.xmax[d] = h->bc.xmin[d] + info->Lxyz[d];
    }
    h->poisson = info->restart == 0 && strcmp(info->fields_init, "poisson") == 0;
    {
        int prc = EMOO_OK;
        if (o.policy != EMOO_POLICY_REFERENCE && o.policy != EMOO_POLICY_CORRECTED) prc = EMOO_ERR_ARG;
        if (o.policy == EMOO_POLICY_CORRECTED) {
            // every dimension periodic (particle and field sides) or walled
            // (particle sides reflecting or absorbing, field sides external)
            for (int d = 0; d < 3; d++) {
                const int pl = h->bc.pbc[2 * d], pr = h->bc.pbc[2 * d + 1];
                const int fl = h->bc.fbc[2 * d], fr = h->bc.fbc[2 * d + 1];
                const bool periodic = pl == PBC_PERIODIC && pr == PBC_PERIODIC && fl == FBC_PERIODIC &&
                                      fr == FBC_PERIODIC;
                const bool walled = pl != PBC_PERIODIC && pr != PBC_PERIODIC && fl == FBC_EXTERNAL &&
                                    fr == FBC_EXTERNAL;
                if (!periodic && !walled) prc = EMOO_ERR_UNSUPPORTED;
            }
            h->policy = o.policy;
            h->g.vshift = 1;
        }
        if (o.poisson_solver != EMOO_POISSON_JACOBI && o.poisson_solver != EMOO_POISSON_MULTIGRID) prc = EMOO_ERR_ARG;
        if (o.poisson_solver == EMOO_POISSON_MULTIGRID) {
            for (int d = 0; d < 3; d++) {
                int a = h->bc.fbc[2 * d], b = h->bc.fbc[2 * d + 1];
                if (a != b || (a != FBC_PERIODIC && a != FBC_EXTERNAL)) prc = EMOO_ERR_UNSUPPORTED;
            }
            h->poisson_solver = o.poisson_solver;
            h->poisson_rtol = o.poisson_rtol > 0 ? o.poisson_rtol : 1e-10;
        }
        if (prc != EMOO_OK) {
            emoo_destroy(h);
            return prc;
        }
    }
    // first physical x index (grid point x0 + (i - 1) dx) the background covers
    h->rho_bg_first = h->g.n[0] + 1;
    for (int i = 1; i <= h->g.n[0]; i++)
        if (info->xyz0[0] + (i - 1) * h->g.d[0] >= o.rho_background_xmin) {
            h->rho_bg_first = i;
            break;
        }
    h->nspec = info->nspecies;
    // the sort keys (species * cells + cell, and the removed-particle key
    // above them) are 32-bit words
    if ((h->precision == EMOO_FP64 ? key_bits(h) : mixed_key_bits(h)) > 32) {
        emoo_destroy(h);
        return EMOO_ERR_UNSUPPORTED;
    }
    double mindx = std::min(std::min(h->g.d[0], h->g.d[1]), h->g.d[2]);
    h->dt = o.dt > 0 ? o.dt : (mindx / 1) / 100.0;  // src/main.cpp:213-214
    h->t = info->t0;
    h->dtp = h->dt;
    // LightBC registry
    light_registry().push_back({h, build_light(*info)});
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        emoo_destroy(h);
        return cuda_status(e);
    }
    rc = EMOO_OK;
    if (h->precision == EMOO_FP64 || true) {
        // FP64 slots: the whole grid for the FP64 form; for the mixed form they
        // hold the FP64 initialisation (Poisson) and serve get/set_field.
        for (int f = 0; f < EMOO_NFIELDS && rc == EMOO_OK; f++) {
            rc = dalloc(h->slot[f], (size_t)h->g.npts);
            if (rc == EMOO_OK) {
                cudaError_t me = cudaMemsetAsync(h->slot[f], 0, sizeof(double) * (size_t)h->g.npts, h->stream);
                if (me != cudaSuccess) rc = cuda_status(me);
            }
        }
    }
    if (rc == EMOO_OK) rc = dalloc(h->ctr, 1);
    if (rc == EMOO_OK) rc = reset_counters(h);
    if (rc == EMOO_OK && h->precision == EMOO_MIXED) rc = mixed_alloc(h);
    int64_t cap = o.capacity > 0 ? o.capacity : info->nparticles_tot;
    if (rc == EMOO_OK && cap > 0) rc = reserve(h, cap);
    if (rc == EMOO_OK) {
        cudaError_t se = cudaStreamSynchronize(h->stream);
        if (se != cudaSuccess) rc = cuda_status(se);
    }
    if (rc != EMOO_OK) {
        emoo_destroy(h);
        return rc;
    }
    *out = h;
    return EMOO_OK;
}

int emoo_destroy(emoo_handle *h) {
    if (!h) return EMOO_ERR_ARG;
    cudaSetDevice(h->dev);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (int f = 0; f < EMOO_NFIELDS; f++) dfree(h->slot[f]);
    free_particles(h);
    if (h->mf) mixed_free(h);
    dfree(h->hist);
    dfree(h->scan_tmp);
    dfree(h->d_spec_count);
    dfree(h->ctr);
    dfree(h->red);
    dfree(h->wprof);
    dfree(h->wproff);
    if (h->jacobi_state) cudaFree(h->jacobi_state);
    multigrid_free(h);
    if (h->mhost) cudaFree(h->mhost);
    for (int i = 0; i < 2; i++)
        if (h->prof_ev[i]) cudaEventDestroy(h->prof_ev[i]);
    for (cudaEvent_t e : h->prof_pending) cudaEventDestroy(e);
    for (cudaEvent_t e : h->prof_pool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    auto &r = light_registry();
    for (size_t i = 0; i < r.size(); i++)
        if (r[i].first == h) {
            r.erase(r.begin() + (long)i);
            break;
        }
    delete h;
    return EMOO_OK;
}

namespace {
// emoo_step leaves rho pending (the loop never reads it); this deposits it -
// at the particles' current positions, folded, with the background - which
// is what the last step's deposit and fold would have left. Called wherever
// rho is read and before anything moves the particles.
int materialize_rho(emoo_handle *h) {
    if (!h->rho_stale) return EMOO_OK;
    h->rho_stale = 0;
    if (h->precision != EMOO_FP64) return mixed_materialize_rho(h);
    EMOO_TRY(deposit_rho_f64(h));
    if (h->policy == EMOO_POLICY_CORRECTED) return fold_full_f64(h, FOLD_RHO);
    for (int d = 0; d < 3; d++)
        if (h->bc.fbc[2 * d] == FBC_PERIODIC) EMOO_TRY(fold_f64(h, d, FOLD_RHO));
    return EMOO_OK;
}
}  // namespace

int emoo_load_particles(emoo_handle *h, int species, int64_t n, const double *x, const double *y, const double *z,
                        const double *vx, const double *vy, const double *vz, const double *gamma,
                        const int64_t *ids) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(compact(h));
    if (species < 0 || species >= h->nspec || n < 0) return EMOO_ERR_ARG;
    if (n == 0) return EMOO_OK;
    if (!x || !y || !z || !vx || !vy || !vz) return EMOO_ERR_ARG;
    int64_t first_id = h->np;
    int64_t at;
    EMOO_TRY(make_room(h, species, n, &at));
    if (h->precision == EMOO_FP64) {
        size_t b = sizeof(double) * (size_t)n;
        EMOO_CUDA(cudaMemcpyAsync(h->x + at, x, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->y + at, y, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->z + at, z, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vx + at, vx, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vy + at, vy, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vz + at, vz, b, cudaMemcpyHostToDevice, h->stream));
        if (gamma) EMOO_CUDA(cudaMemcpyAsync(h->gam + at, gamma, b, cudaMemcpyHostToDevice, h->stream));
        else EMOO_CUDA(cudaMemsetAsync(h->gam + at, 0, b, h->stream));
    } else {
        EMOO_TRY(mixed_from_f64(h, at, n, x, y, z, vx, vy, vz, gamma));
    }
    if (h->ids) {
        std::vector<int64_t> tmp;
        const int64_t *src = ids;
        if (!src) {
            tmp.resize((size_t)n);
            for (int64_t i = 0; i < n; i++) tmp[(size_t)i] = first_id + i;
            src = tmp.data();
        }
        EMOO_CUDA(cudaMemcpyAsync(h->ids + at, src, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    dfree(h->fcache);
    return EMOO_OK;
}

int emoo_load_generated(emoo_handle *h, const emoo_gen_params *g, int64_t n) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(compact(h));
    if (!g || g->species < 0 || g->species >= h->nspec || n < 0) return EMOO_ERR_ARG;
    if (n == 0) return EMOO_OK;
    int64_t first_id = h->np;
    int64_t at;
    EMOO_TRY(make_room(h, g->species, n, &at));
    if (h->precision == EMOO_FP64) {
        EMOO_TRY(generate_device(h, g, 0, n, at));
    } else {
        // staged in chunks through the payload scratch (7 doubles per particle)
        int64_t chunk = (int64_t)(h->pay_bytes / (7 * sizeof(double)));
        if (chunk < 1) return EMOO_ERR_OOM;
        for (int64_t b = 0; b < n; b += chunk) {
            int64_t m = std::min(chunk, n - b);
            EMOO_TRY(generate_device(h, g, b, m, 0));
            double *s = (double *)h->pay;
            EMOO_TRY(mixed_from_f64(h, at + b, -m, s, s + m, s + 2 * m, s + 3 * m, s + 4 * m, s + 5 * m, s + 6 * m));
        }
    }
    if (h->ids) {
        std::vector<int64_t> tmp((size_t)n);
        for (int64_t i = 0; i < n; i++) tmp[(size_t)i] = first_id + i;
        EMOO_CUDA(cudaMemcpyAsync(h->ids + at, tmp.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice,
                                  h->stream));
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    dfree(h->fcache);
    return EMOO_OK;
}

int emoo_num_particles(emoo_handle *h, int species, int64_t *n) {
    if (h && h->host_mode && n && species < h->nspec) {  // counts do not change while attached
        *n = species < 0 ? h->np : h->count[species];
        return EMOO_OK;
    }
    HANDLE_CHECK(h);
    if (!n) return EMOO_ERR_ARG;
    if (species >= h->nspec) return EMOO_ERR_ARG;
    EMOO_TRY(compact(h));
    *n = species < 0 ? h->np : h->count[species];
    return EMOO_OK;
}

int emoo_get_particles(emoo_handle *h, int species, int64_t cap, double *x, double *y, double *z, double *vx,
                       double *vy, double *vz, double *gamma, int64_t *ids, int64_t *n) {
    if (h && h->host_mode && !ids) {  // the attached arrays are the state: copied as they are
        if (species < 0 || species >= h->nspec || !n) return EMOO_ERR_ARG;
        const int64_t cnt = h->count[species];
        *n = cnt;
        if (cap < cnt || !x || !y || !z || !vx || !vy || !vz) return EMOO_ERR_ARG;
        const emoo_handle::Attached &a = h->attached[species];
        double *out[7] = {x, y, z, vx, vy, vz, gamma};
        for (int q = 0; q < 7; q++)
            if (out[q] && a.p[q] && out[q] != a.p[q]) memcpy(out[q], a.p[q], sizeof(double) * (size_t)cnt);
        if (gamma && !a.p[6]) memset(gamma, 0, sizeof(double) * (size_t)cnt);
        return EMOO_OK;
    }
    HANDLE_CHECK(h);
    if (species < 0 || species >= h->nspec || !n) return EMOO_ERR_ARG;
    EMOO_TRY(compact(h));
    int64_t cnt = h->count[species];
    *n = cnt;
    if (cap < cnt) return EMOO_ERR_ARG;
    if (!x || !y || !z || !vx || !vy || !vz) return EMOO_ERR_ARG;
    int64_t at = h->off[species];
    if (h->precision == EMOO_FP64) {
        size_t b = sizeof(double) * (size_t)cnt;
        EMOO_CUDA(cudaMemcpyAsync(x, h->x + at, b, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(y, h->y + at, b, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(z, h->z + at, b, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(vx, h->vx + at, b, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(vy, h->vy + at, b, cudaMemcpyDeviceToHost, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(vz, h->vz + at, b, cudaMemcpyDeviceToHost, h->stream));
        if (gamma) EMOO_CUDA(cudaMemcpyAsync(gamma, h->gam + at, b, cudaMemcpyDeviceToHost, h->stream));
    } else {
        EMOO_TRY(mixed_to_f64(h, at, cnt, x, y, z, vx, vy, vz, gamma));
    }
    if (ids) {
        if (!h->ids) return EMOO_ERR_STATE;
        EMOO_CUDA(cudaMemcpyAsync(ids, h->ids + at, sizeof(int64_t) * (size_t)cnt, cudaMemcpyDeviceToHost, h->stream));
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_get_particle_fields(emoo_handle *h, int species, int64_t cap, double *e1, double *e2, double *e3, double *b1,
                             double *b2, double *b3, int64_t *n) {
    HANDLE_CHECK(h);
    if (species < 0 || species >= h->nspec || !n) return EMOO_ERR_ARG;
    EMOO_TRY(compact(h));  // a compaction drops the cache: it no longer matches the store
    if (!h->fcache) return EMOO_ERR_STATE;
    int64_t cnt = h->count[species];
    *n = cnt;
    if (cap < cnt) return EMOO_ERR_ARG;
    double *outs[6] = {e1, e2, e3, b1, b2, b3};
    int64_t at = h->off[species];
    for (int q = 0; q < 6; q++) {
        if (!outs[q]) return EMOO_ERR_ARG;
        EMOO_CUDA(cudaMemcpyAsync(outs[q], h->fcache + (size_t)q * h->cap + at, sizeof(double) * (size_t)cnt,
                                  cudaMemcpyDeviceToHost, h->stream));
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_get_field(emoo_handle *h, int id, double *out) {
    HANDLE_CHECK(h);
    if (id < 0 || id >= EMOO_NFIELDS || !out) return EMOO_ERR_ARG;
    if (id == EMOO_RHO) EMOO_TRY(materialize_rho(h));
    size_t b = sizeof(double) * (size_t)h->g.npts;
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_get_field(h, id, h->slot[id]));
    EMOO_CUDA(cudaMemcpyAsync(out, h->slot[id], b, cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_set_field(emoo_handle *h, int id, const double *in) {
    HANDLE_CHECK(h);
    if (id < 0 || id >= EMOO_NFIELDS || !in) return EMOO_ERR_ARG;
    size_t b = sizeof(double) * (size_t)h->g.npts;
    EMOO_CUDA(cudaMemcpyAsync(h->slot[id], in, b, cudaMemcpyHostToDevice, h->stream));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_set_field(h, id, h->slot[id]));
    if (id == EMOO_RHO) h->rho_stale = 0;
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_cell_id(emoo_handle *h, double x, double y, double z, int *cid) {
    if (!h || !cid) return EMOO_ERR_ARG;
    const Geom &g = h->g;
    int ix = (int)((x - g.x0[0]) * g.id[0]) + 1;
    int iy = (int)((y - g.x0[1]) * g.id[1]) + 1;
    int iz = (int)((z - g.x0[2]) * g.id[2]) + 1;
    *cid = g.cny * ix + g.cnz * iy + iz;
    return EMOO_OK;
}

int emoo_init_fields(emoo_handle *h, int iters[4]) {
    HANDLE_CHECK(h);
    // time_phys and dt_phys are still zero during the reference's field
    // initialisation (src/main.cpp:174 runs before :212-214)
    h->t = 0.0;
    h->dtp = 0.0;
    int rc = EMOO_OK;
    if (h->poisson) {
        h->rho_stale = 0;
        rc = deposit_all(h, 1);
        if (rc == EMOO_OK) rc = execute_bc(h, EMOO_SEND_JRHO);
        // the mixed form solves in FP64 on the grid slots
        if (rc == EMOO_OK && h->precision != EMOO_FP64) rc = mixed_deposit_to_f64(h);
        if (rc == EMOO_OK) rc = poisson_init(h, iters);
    } else {
        rc = const_init(h);
    }
    h->t = h->info.t0;
    h->dtp = h->dt;
    if (rc != EMOO_OK && rc != EMOO_ERR_NOT_CONVERGED) return rc;
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    h->fields_initialised = 1;
    return rc;
}

int emoo_poisson_init(emoo_handle *h, int iters[4]) {
    HANDLE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    double t = h->t, dtp = h->dtp;
    h->t = 0.0;
    h->dtp = 0.0;
    int rc = EMOO_OK;
    if (h->precision != EMOO_FP64) rc = mixed_deposit_to_f64(h);
    if (rc == EMOO_OK) rc = poisson_init(h, iters);
    h->t = t;
    h->dtp = dtp;
    cudaStreamSynchronize(h->stream);
    return rc;
}

int emoo_sort(emoo_handle *h) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(do_sort(h));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return read_err(h);
}

int emoo_interpolate(emoo_handle *h) {
    HANDLE_CHECK(h);
    EMOO_TRY(compact(h));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_interpolate(h));
    else EMOO_TRY(interpolate_f64(h));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return read_err(h);
}

int emoo_push(emoo_handle *h) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_push_cached(h));
    else EMOO_TRY(push_cached_f64(h, h->dtp));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_apply_particle_bc(emoo_handle *h, int64_t counts6[6]) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(reset_counters(h));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_particle_bc(h));
    else EMOO_TRY(particle_bc_f64(h));
    int rc = read_counters(h, counts6, false);
    const bool absorbing = has_absorbing(h);
    // clearGhosts: removed particles leave the store (compaction by the sort)
    if (rc == EMOO_OK && absorbing) rc = do_sort(h);
    return rc;
}

int emoo_deposit(emoo_handle *h, int with_rho) {
    HANDLE_CHECK(h);
    EMOO_TRY(deposit_all(h, with_rho));
    if (with_rho) h->rho_stale = 0;  // else rho stays as the last deposit left it (pending or not)
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return read_err(h);
}

int emoo_execute_bc(emoo_handle *h, int send_id) {
    HANDLE_CHECK(h);
    if (send_id == EMOO_SEND_JRHO || send_id == EMOO_RHO) EMOO_TRY(materialize_rho(h));
    EMOO_TRY(execute_bc(h, send_id));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_evolve_fields(emoo_handle *h, int electrostatic) {
    HANDLE_CHECK(h);
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_yee_public(h, h->dtp, electrostatic));
    else if (electrostatic) EMOO_TRY(yee_es_f64(h, h->dtp));
    else EMOO_TRY(yee_f64(h, h->dtp));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_set_waves(emoo_handle *h, int nwaves, const double *amp, const double *phase_deg) {
    HANDLE_CHECK(h);
    if (nwaves != h->info.nwaves || nwaves < 0 || nwaves > EMOO_NWAVE || (nwaves && (!amp || !phase_deg)))
        return EMOO_ERR_ARG;
    for (int w = 0; w < nwaves; w++)  // all checked before any is applied
        if (!std::isfinite(amp[w]) || !std::isfinite(phase_deg[w])) return EMOO_ERR_ARG;
    LightState *L = light_of(h);
    if (!L) return EMOO_ERR_STATE;
    for (int w = 0; w < nwaves; w++) {
        h->info.peakamps[w] = amp[w];
        h->info.phases[w] = phase_deg[w];
    }
    *L = build_light(h->info);
    return EMOO_OK;
}

namespace {
// Side index (0..5: x-left, x-right, y-left, ...) of an input wave side
// (-1 x left, +1 x right, -2 y left, ...), or -1.
int side_index(int side) {
    if (side == 0 || side < -3 || side > 3) return -1;
    return 2 * (std::abs(side) - 1) + (side > 0 ? 1 : 0);
}

// Recomputes the spot factor tables from the handle's wave shapes; returns
// EMOO_ERR_ARG when two spotted waves of one side and polarisation differ in
// waist or centre.
int build_spots(emoo_handle *h) {
    const emoo_input_info &in = h->info;
    int spot_w[6][3];
    for (auto &r : spot_w)
        for (int &v : r) v = -1;
    for (int w = 0; w < in.nwaves && w < EMOO_NWAVE; w++) {
        const emoo_wave_shape *sh = shape_of(h, w);
        if (!sh || !(sh->waist > 0)) continue;
        const int s = side_index(in.inSide[w]), p = in.inPolE[w] - 1;
        if (s < 0 || p < 0 || p > 2) continue;
        const int o = spot_w[s][p];
        if (o >= 0) {
            const emoo_wave_shape &a = h->wshape[o];
            if (a.waist != sh->waist || a.center[0] != sh->center[0] || a.center[1] != sh->center[1])
                return EMOO_ERR_ARG;
        } else {
            spot_w[s][p] = w;
        }
    }
    const Geom &g = h->g;
    const int stride = std::max(std::max(g.tot[0], g.tot[1]), g.tot[2]);
    std::vector<double> tab((size_t)36 * stride, 0.0);
    std::vector<float> tabf((size_t)36 * stride, 0.0f);
    bool any = false;
    for (int s = 0; s < 6; s++) {
        const int d = s / 2, o[2] = {(d == 0) ? 1 : 0, (d == 2) ? 1 : 2};
        for (int p = 0; p < 3; p++) {
            const int w = spot_w[s][p];
            if (w < 0) continue;
            any = true;
            const emoo_wave_shape &sh = h->wshape[w];
            for (int a = 0; a < 2; a++) {
                const int ax = o[a];
                const double hh = ax == p ? 0.5 : 0.0;
                const double x0 = in.xyz0[ax], dd = g.d[ax];
                const size_t base = (size_t)((3 * s + p) * 2 + a) * stride;
                for (int j = 0; j < g.tot[ax]; j++) {
                    const double pos = x0 + (j - 1 + hh) * dd;
                    const double r = (pos - sh.center[a]) / sh.waist;
                    tab[base + j] = exp(-(r * r));
                    tabf[base + j] = (float)tab[base + j];
                }
            }
        }
    }
    if (any && !h->wprof) {
        EMOO_TRY(dalloc(h->wprof, tab.size()));
        EMOO_TRY(dalloc(h->wproff, tabf.size()));
    }
    if (any) {
        EMOO_CUDA(cudaMemcpyAsync(h->wprof, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->wproff, tabf.data(), sizeof(float) * tabf.size(), cudaMemcpyHostToDevice,
                                  h->stream));
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
    }
    h->wprof_stride = stride;
    for (int s = 0; s < 6; s++)
        for (int p = 0; p < 3; p++) h->wspot[s][p] = spot_w[s][p] >= 0;
    return EMOO_OK;
}
}  // namespace

int emoo_set_wave_shape(emoo_handle *h, int wave, const emoo_wave_shape *shape) {
    HANDLE_CHECK(h);
    if (wave < 0 || wave >= h->info.nwaves || wave >= EMOO_NWAVE) return EMOO_ERR_ARG;
    if (shape) {
        const emoo_wave_shape &sh = *shape;
        if (!std::isfinite(sh.waist) || sh.waist < 0 || !std::isfinite(sh.center[0]) || !std::isfinite(sh.center[1]))
            return EMOO_ERR_ARG;
        if (sh.ncoef < 0 || sh.ncoef > EMOO_NCOEF) return EMOO_ERR_ARG;
        if (sh.ncoef > 0 && !(std::isfinite(sh.t_start) && std::isfinite(sh.window) && sh.window > 0))
            return EMOO_ERR_ARG;
        for (int k = 0; k < sh.ncoef; k++)
            if (!std::isfinite(sh.coef[k])) return EMOO_ERR_ARG;
    }
    const emoo_wave_shape old = h->wshape[wave];
    const int old_on = h->wshaped[wave];
    if (shape) {
        h->wshape[wave] = *shape;
        for (int k = shape->ncoef; k < EMOO_NCOEF; k++) h->wshape[wave].coef[k] = 0.0;
        h->wshaped[wave] = 1;
    } else {
        h->wshape[wave] = emoo_wave_shape{};
        h->wshaped[wave] = 0;
    }
    const int rc = build_spots(h);
    if (rc != EMOO_OK) {
        h->wshape[wave] = old;
        h->wshaped[wave] = old_on;
        build_spots(h);
    }
    return rc;
}

int emoo_ad_nparams(const emoo_handle *h) {
    if (!h) return EMOO_ERR_ARG;
    bool series = false;
    for (int w = 0; w < h->info.nwaves && w < EMOO_NWAVE; w++) series |= h->wshaped[w] && h->wshape[w].ncoef > 0;
    return 2 * h->info.nwaves + (series ? EMOO_NCOEF * h->info.nwaves : 0);
}

int emoo_step(emoo_handle *h, int nsteps, int64_t counts6[6]) {
    if (!h) return EMOO_ERR_ARG;
    EMOO_TRY(set_device(h));  // host-resident particles: the store is refreshed below only where needed
    if (nsteps < 0) return EMOO_ERR_ARG;
    EMOO_TRY(reset_counters(h));
    // with deposit_rho the step deposits J only and leaves rho pending
    // (materialize_rho); otherwise rho is left as it is and folded each step,
    // as the reference does when it deposits J alone
    const bool lazy_rho = h->opts.deposit_rho != 0;
    const int fold_what = lazy_rho ? FOLD_J : FOLD_ALL;
    for (int it = 0; it < nsteps; it++) {
        int64_t ti = h->step_index;
        if (h->host_mode) {
            // host-resident particles: stream them through the fused kernel, in
            // both directions at once over the host link; a step that sorts,
            // writes a history row or makes the first push (or has particle
            // removal) runs on the device store between an upload and a readback
            const bool sort_now = h->info.nstep_sort > 0 && ti % h->info.nstep_sort == 0;
            const bool hist_now = ti >= h->next_hist;
            const bool streamed = h->precision == EMOO_MIXED && !sort_now &&
                                  !(h->info.relativity != 0 && h->first_push) && !has_absorbing(h);
            if (streamed) {
                // a history row: field energies before the step, particle moments
                // from the pre-push state the kernel also leaves in the device store
                double e6[6];
                if (hist_now) EMOO_TRY(mixed_field_energy(h, e6));
                EMOO_TRY(mixed_step_host(h, h->dtp, fold_what, hist_now ? 1 : 0));
                if (hist_now) {
                    double m4[4], row[8];
                    EMOO_TRY(mixed_moments(h, m4));
                    history_from(h, m4, e6, row);
                    h->hist_rows.insert(h->hist_rows.end(), row, row + 8);
                    h->next_hist += h->opts.history_every;
                }
                h->store_stale = 1;
                h->t += h->dtp;
                h->step_index++;
                if (lazy_rho) h->rho_stale = 1;
                continue;
            }
            EMOO_TRY(host_store_sync(h));
        }
        if (h->info.nstep_sort > 0 && ti % h->info.nstep_sort == 0) EMOO_TRY(do_sort(h));
        if (ti >= h->next_hist) {
            double row[8];
            EMOO_TRY(history_row(h, row));
            h->hist_rows.insert(h->hist_rows.end(), row, row + 8);
            h->next_hist += h->opts.history_every;
        }
        if (h->precision == EMOO_FP64) {
            EMOO_TRY(fused_step_f64(h, h->dtp, 0));
            if (h->policy == EMOO_POLICY_CORRECTED) EMOO_TRY(fold_full_f64(h, fold_what));
            else
                for (int d = 0; d < 3; d++)
                    if (h->bc.fbc[2 * d] == FBC_PERIODIC) EMOO_TRY(fold_f64(h, d, fold_what));
            if (h->info.electrostatic == 1) EMOO_TRY(yee_es_f64(h, h->dtp));
            else EMOO_TRY(yee_f64(h, h->dtp));
            EMOO_TRY(execute_bc(h, EMOO_SEND_EB));
        } else {
            EMOO_TRY(mixed_step(h, h->dtp, 0, fold_what));
        }
        h->t += h->dtp;
        h->step_index++;
        if (lazy_rho) h->rho_stale = 1;
        if (h->host_mode) EMOO_TRY(host_download(h));
    }
    int64_t c6[6];
    const int rc = read_counters(h, c6, false);
    for (int s = 0; s < 6; s++)
        if (h->bc.pbc[s] == PBC_ABSORBING && c6[s] > 0) h->dead_pending = 1;
    if (counts6)
        for (int s = 0; s < 6; s++) counts6[s] = c6[s];
    return rc;
}

int emoo_history(emoo_handle *h, double out8[8]) {
    HANDLE_CHECK(h);
    if (!out8) return EMOO_ERR_ARG;
    return history_row(h, out8);
}

int emoo_history_rows(emoo_handle *h, int cap, double *rows, int *n) {
    if (!h || !n || (rows && cap < 0)) return EMOO_ERR_ARG;
    int have = (int)(h->hist_rows.size() / 8);
    *n = have;
    if (rows) {
        int m = std::min(cap, have);
        memcpy(rows, h->hist_rows.data(), sizeof(double) * 8 * (size_t)m);
    }
    return EMOO_OK;
}

int emoo_gauss_residual(emoo_handle *h, double out2[2]) {
    HANDLE_CHECK(h);
    if (!out2) return EMOO_ERR_ARG;
    EMOO_TRY(materialize_rho(h));
    if (h->precision != EMOO_FP64) EMOO_TRY(mixed_fields_to_slots(h));
    return gauss_residual_f64(h, out2);
}

int emoo_time(emoo_handle *h, double *t, double *dt) {
    if (!h) return EMOO_ERR_ARG;
    if (t) *t = h->t;
    if (dt) *dt = h->dt;
    return EMOO_OK;
}

int emoo_perturb(emoo_handle *h, uint64_t seed, double rel) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    if (h->precision != EMOO_FP64) return EMOO_ERR_UNSUPPORTED;
    if (!(rel >= 0.0 && rel < 1.0)) return EMOO_ERR_ARG;
    EMOO_TRY(perturb_f64(h, seed, rel));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

int emoo_check(emoo_handle *h) {
    HANDLE_CHECK(h);
    return read_err(h);
}

int emoo_attach_particles(emoo_handle *h, int species, int64_t n, double *x, double *y, double *z, double *vx,
                          double *vy, double *vz, double *gamma) {
    HANDLE_CHECK(h);
    // the mixed form, and no particle removal (the arrays keep their length)
    if (h->precision != EMOO_MIXED || has_absorbing(h)) return EMOO_ERR_UNSUPPORTED;
    if (species < 0 || species >= h->nspec) return EMOO_ERR_ARG;
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(compact(h));
    if (n != h->count[species]) return EMOO_ERR_ARG;
    double *p[7] = {x, y, z, vx, vy, vz, gamma};
    const bool rel = h->info.relativity != 0;
    for (int q = 0; q < 7 && n > 0; q++) {  // an empty species needs no arrays
        if (!p[q] && (q < 6 || rel)) return EMOO_ERR_ARG;
        if (p[q] && !mixed_device_accessible(h, p[q])) return EMOO_ERR_UNSUPPORTED;
    }
    emoo_handle::Attached &a = h->attached[species];
    a.n = n;
    for (int q = 0; q < 7; q++) a.p[q] = p[q];
    bool all = true;
    for (int s = 0; s < h->nspec; s++) all = all && h->attached[s].n == h->count[s];
    if (all) {
        MHost m = {};
        m.g = h->g;
        m.rel = rel ? 1 : 0;
        for (int s = 0; s < h->nspec; s++) {
            const emoo_handle::Attached &b = h->attached[s];
            m.x[s] = b.p[0], m.y[s] = b.p[1], m.z[s] = b.p[2];
            m.vx[s] = b.p[3], m.vy[s] = b.p[4], m.vz[s] = b.p[5], m.gam[s] = b.p[6];
        }
        if (!h->mhost) EMOO_CUDA(cudaMalloc(&h->mhost, sizeof(MHost)));
        EMOO_CUDA(cudaMemcpyAsync(h->mhost, &m, sizeof(MHost), cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaStreamSynchronize(h->stream));
        h->host_mode = 1;
        h->store_stale = 1;  // the arrays are the particle state from now on
    }
    return EMOO_OK;
}

int emoo_detach_particles(emoo_handle *h) {
    HANDLE_CHECK(h);  // refreshes the store from the arrays
    for (int s = 0; s < EMOO_NSPEC; s++) h->attached[s] = emoo_handle::Attached();
    h->host_mode = 0;
    h->store_stale = 0;
    return EMOO_OK;
}

int emoo_set_particles(emoo_handle *h, int species, int64_t n, const double *x, const double *y, const double *z,
                       const double *vx, const double *vy, const double *vz, const double *gamma) {
    HANDLE_CHECK(h);
    STORE_WRITE_CHECK(h);
    EMOO_TRY(materialize_rho(h));
    EMOO_TRY(compact(h));
    if (species < 0 || species >= h->nspec || n != h->count[species]) return EMOO_ERR_ARG;
    if (n == 0) return EMOO_OK;
    if (!x || !y || !z || !vx || !vy || !vz) return EMOO_ERR_ARG;
    int64_t at = h->off[species];
    if (h->precision == EMOO_FP64) {
        size_t b = sizeof(double) * (size_t)n;
        EMOO_CUDA(cudaMemcpyAsync(h->x + at, x, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->y + at, y, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->z + at, z, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vx + at, vx, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vy + at, vy, b, cudaMemcpyHostToDevice, h->stream));
        EMOO_CUDA(cudaMemcpyAsync(h->vz + at, vz, b, cudaMemcpyHostToDevice, h->stream));
        if (gamma) EMOO_CUDA(cudaMemcpyAsync(h->gam + at, gamma, b, cudaMemcpyHostToDevice, h->stream));
    } else {
        EMOO_TRY(mixed_from_f64(h, at, n, x, y, z, vx, vy, vz, gamma));
    }
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    dfree(h->fcache);
    return read_err(h);
}

int emoo_get_stream(emoo_handle *h, void **stream) {
    if (!h || !stream) return EMOO_ERR_ARG;
    *stream = (void *)h->stream;
    return EMOO_OK;
}

int emoo_set_profiling(emoo_handle *h, int on) {
    HANDLE_CHECK(h);
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (cudaEvent_t e : h->prof_pending) h->prof_pool.push_back(e);
    h->prof_pending.clear();
    h->prof_ms = 0.0;
    h->prof_count = 0;
    if (on) {
        for (int i = 0; i < 2; i++)
            if (!h->prof_ev[i]) EMOO_CUDA(cudaEventCreate(&h->prof_ev[i]));
    }
    h->prof_on = on ? 1 : 0;
    return EMOO_OK;
}

int emoo_get_stats(emoo_handle *h, emoo_stats *s) {
    HANDLE_CHECK(h);
    if (!s) return EMOO_ERR_ARG;
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i + 1 < h->prof_pending.size(); i += 2) {
        float ms = 0.0f;
        EMOO_CUDA(cudaEventElapsedTime(&ms, h->prof_pending[i], h->prof_pending[i + 1]));
        h->prof_ms += ms;
        h->prof_count++;
        h->prof_pool.push_back(h->prof_pending[i]);
        h->prof_pool.push_back(h->prof_pending[i + 1]);
    }
    h->prof_pending.clear();
    s->launches = h->launches;
    s->timed_launches = h->prof_count;
    s->timed_ms = h->prof_ms;
    s->ad_cell_mismatch = h->ad_cell_mismatch;
    return EMOO_OK;
}

}  // extern "C"
