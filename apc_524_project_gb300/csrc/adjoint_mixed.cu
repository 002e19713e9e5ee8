// adjoint_mixed.cu - the differentiated run of the mixed-precision form (no
// reference counterpart): forward and adjoint in FP32, gradients with
// respect to the wave parameters accumulated in FP64.
//
// The differentiated step is the mixed loop's step with J only (the push of
// k_fused_m, the J fold, the FP32 Yee update, executeBC(-1) with LightBC),
// under either policy: the corrected one's reverse adds the adjoints of the
// charge-conserving current (particles_mixed.cu), the whole-range folds and
// copies, the mirror folds and the planes set between the Yee halves.
// State is checkpointed every `checkpoint_every` steps as mixed snapshots
// (28 bytes per particle, 36 bytes per grid point: a quarter of the FP64
// form's, so sqrt(N) checkpointing of long horizons fits in HBM); each
// segment is recomputed forward, keeping the state before each of its
// steps, then reversed. Per step in reverse: the plane and ghost-copy
// adjoints of executeBC(-1), the transposed Yee stencils, the fold adjoint
// (adjoint_fields.cuh, float), then the particle kernel of particles_mixed.cu
// (deposit adjoint as a gather of the J adjoint, boundary, push and gather
// adjoints, the last a scatter of FP32 atomics).
//
// Before the first push the relativistic mixed state holds the loaded
// velocity; the run first stores u = gamma v (the first push's own input), so
// every step of the run is the same function. The store is sorted by cell at
// the start of every segment (the deposit's run sums and the gather's
// locality depend on it); a sort is a permutation, whose adjoint maps the
// particle adjoints back through it. The velocity gradient is d objective /
// d v with gamma held, gamma d objective / d u, returned in the store's order
// before the run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "adjoint_fields.cuh"
#include "dev_common.cuh"
#include "emoo_internal.h"

namespace emoo {

namespace {

using FOutF = adf::FOutT<float>;
using JPtrsF = adf::JPtrsT<float>;
using Slots6F = adf::Slots6T<float>;

constexpr int NSLOT = EMOO_BZ_TM1 + 1;

int pblocks_m(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 64)); }

dim3 grid_all_m(const Geom &g, dim3 blk) {
    return dim3((g.tot[2] + blk.x - 1) / blk.x, (g.tot[1] + blk.y - 1) / blk.y, g.tot[0]);
}

FOutF field_out_f(float *const *slots, int bswap) {
    FOutF F;
    for (int c = 0; c < 3; c++) {
        F.E[c] = slots[EMOO_EX + c];
        F.B[c] = bswap ? slots[EMOO_BX_TM1 + c] : slots[EMOO_BX + c];
        F.T[c] = bswap ? slots[EMOO_BX + c] : slots[EMOO_BX_TM1 + c];
    }
    return F;
}

struct SlabM {
    int lo, hi;  // grid point x index range [lo, hi)
};

// 0.5 V sum(E^2 + B^2) over the slab from the FP32 fields, FP64 sums.
__global__ void k_objective_field_m(Geom g, SlabM sl, FOutF F, double *out) {
    const int64_t ny = g.n[1], nz = g.n[2];
    const int64_t m = (int64_t)(sl.hi - sl.lo) * ny * nz;
    double a = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % nz) + 1;
        const int j = (int)((t / nz) % ny) + 1;
        const int i = (int)(t / (nz * ny)) + sl.lo;
        const int64_t p = gidx(g, i, j, k);
        for (int c = 0; c < 3; c++) {
            const double e = F.E[c][p], b = F.B[c][p];
            a += e * e + b * b;
        }
    }
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, 0.5 * g.vol * a);
}

// Seeds the field adjoints with V (E, B) on the slab.
__global__ void k_objective_field_seed_m(Geom g, SlabM sl, FOutF F, FOutF A) {
    const int64_t ny = g.n[1], nz = g.n[2];
    const int64_t m = (int64_t)(sl.hi - sl.lo) * ny * nz;
    const float v = (float)g.vol;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % nz) + 1;
        const int j = (int)((t / nz) % ny) + 1;
        const int i = (int)(t / (nz * ny)) + sl.lo;
        const int64_t p = gidx(g, i, j, k);
        for (int c = 0; c < 3; c++) {
            A.E[c][p] += v * F.E[c][p];
            A.B[c][p] += v * F.B[c][p];
        }
    }
}

// ---- snapshots of the mixed state -------------------------------------------

struct MSnap {
    char *buf = nullptr;
    int bswap = 0;
    double t = 0.0;
    int64_t step = 0;
    int64_t np = 0;  // the store's size and species segments at the snapshot
    int64_t off[EMOO_NSPEC + 1] = {};
    int64_t count[EMOO_NSPEC] = {};
};

struct AdRunM {
    emoo_handle *h = nullptr;
    int64_t cap = 0, npts = 0;  // particle capacity of the buffers (the store's size at the start)
    std::vector<void *> owned;

    void *alloc(size_t bytes) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
        owned.push_back(p);
        return p;
    }
    ~AdRunM() {
        for (void *p : owned) cudaFree(p);
    }
    // layout (capacity cap): cell int32[cap] | ox oy oz ux uy uz float[cap] | E xyz, B slots (B, B_tm1
    // storage) float[npts]
    size_t snap_bytes() const { return (size_t)cap * 28 + (size_t)npts * 36; }
    float *pf(const MSnap &s, int k) const { return (float *)(s.buf + (size_t)cap * 4) + (size_t)k * cap; }
    float *ff(const MSnap &s, int k) const { return (float *)(s.buf + (size_t)cap * 28) + (size_t)k * npts; }
    int save(MSnap &s) {
        if (!s.buf) s.buf = (char *)alloc(snap_bytes());
        if (!s.buf) return EMOO_ERR_OOM;
        cudaStream_t st = h->stream;
        const int64_t np = h->np;
        if (np) {
            EMOO_CUDA(cudaMemcpyAsync(s.buf, h->cell, sizeof(int32_t) * np, cudaMemcpyDeviceToDevice, st));
            const float *P[6] = {h->ox, h->oy, h->oz, h->ux, h->uy, h->uz};
            for (int k = 0; k < 6; k++)
                EMOO_CUDA(cudaMemcpyAsync(pf(s, k), P[k], sizeof(float) * np, cudaMemcpyDeviceToDevice, st));
        }
        float *E[3], *Bs[6];
        mixed_field_arrays(h, E, Bs);
        for (int k = 0; k < 9; k++) {
            const float *src = k < 3 ? E[k] : Bs[k - 3];
            EMOO_CUDA(cudaMemcpyAsync(ff(s, k), src, sizeof(float) * npts, cudaMemcpyDeviceToDevice, st));
        }
        s.bswap = h->bswap;
        s.t = h->t;
        s.step = h->step_index;
        s.np = np;
        for (int k = 0; k <= EMOO_NSPEC; k++) s.off[k] = h->off[k];
        for (int k = 0; k < EMOO_NSPEC; k++) s.count[k] = h->count[k];
        return EMOO_OK;
    }
    int restore(const MSnap &s) {
        cudaStream_t st = h->stream;
        const int64_t np = s.np;
        if (np) {
            EMOO_CUDA(cudaMemcpyAsync(h->cell, s.buf, sizeof(int32_t) * np, cudaMemcpyDeviceToDevice, st));
            float *P[6] = {h->ox, h->oy, h->oz, h->ux, h->uy, h->uz};
            for (int k = 0; k < 6; k++)
                EMOO_CUDA(cudaMemcpyAsync(P[k], pf(s, k), sizeof(float) * np, cudaMemcpyDeviceToDevice, st));
        }
        float *E[3], *Bs[6];
        mixed_field_arrays(h, E, Bs);
        for (int k = 0; k < 9; k++) {
            float *dst = k < 3 ? E[k] : Bs[k - 3];
            EMOO_CUDA(cudaMemcpyAsync(dst, ff(s, k), sizeof(float) * npts, cudaMemcpyDeviceToDevice, st));
        }
        h->bswap = s.bswap;
        h->t = s.t;
        h->step_index = s.step;
        h->np = np;
        for (int k = 0; k <= EMOO_NSPEC; k++) h->off[k] = s.off[k];
        for (int k = 0; k < EMOO_NSPEC; k++) h->count[k] = s.count[k];
        return EMOO_OK;
    }
    MSnapView view(const MSnap &s) const {
        MSnapView v;
        v.cell = (const int32_t *)s.buf;
        for (int a = 0; a < 3; a++) {
            v.o[a] = pf(s, a);
            v.u[a] = pf(s, 3 + a);
            v.E[a] = ff(s, a);
            v.B[a] = ff(s, s.bswap ? 6 + a : 3 + a);
            v.T[a] = ff(s, s.bswap ? 3 + a : 6 + a);
        }
        return v;
    }
};

// The adjoint of a sort: the particle adjoints after it (order of the sorted
// store, n_after entries) go back to the order before it: dst[perm[i]] =
// src[i]; particles the sort dropped (removed earlier) keep 0.
struct Lam6 {
    float *p[6];
};
__global__ void k_unsort_adjoint(Lam6 src, Lam6 dst, const uint32_t *perm, int64_t n_after) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_after) return;
    const uint32_t j = perm[i];
#pragma unroll
    for (int k = 0; k < 6; k++) dst.p[k][j] = src.p[k][i];
}

MSnapView handle_view(emoo_handle *h) {
    MSnapView v;
    v.cell = h->cell;
    const float *o[3] = {h->ox, h->oy, h->oz}, *u[3] = {h->ux, h->uy, h->uz};
    float *E[3], *Bs[6];
    mixed_field_arrays(h, E, Bs);
    for (int a = 0; a < 3; a++) {
        v.o[a] = o[a];
        v.u[a] = u[a];
        v.E[a] = E[a];
        v.B[a] = h->bswap ? Bs[3 + a] : Bs[a];
        v.T[a] = h->bswap ? Bs[a] : Bs[3 + a];
    }
    return v;
}

int primal_step_m(emoo_handle *h) {
    EMOO_TRY(mixed_step(h, h->dtp, 0, FOLD_J));
    h->t += h->dtp;
    h->step_index++;
    return EMOO_OK;
}

struct ObjM {
    int kind;
    SlabM sl;
    int species;
    double xlo, xhi;
};

int objective_m(emoo_handle *h, const ObjM &os, double *dev, double *out) {
    EMOO_CUDA(cudaMemsetAsync(dev, 0, sizeof(double), h->stream));
    if (os.kind == EMOO_AD_OBJ_FIELD) {
        float *sl[NSLOT] = {}, *E[3], *Bs[6];
        mixed_field_arrays(h, E, Bs);
        for (int c = 0; c < 3; c++) {
            sl[EMOO_EX + c] = E[c];
            sl[EMOO_BX + c] = Bs[c];
            sl[EMOO_BX_TM1 + c] = Bs[3 + c];
        }
        h->launches++;
        k_objective_field_m<<<pblocks_m((int64_t)(os.sl.hi - os.sl.lo) * h->g.n[1] * h->g.n[2]), 256, 0, h->stream>>>(
            h->g, os.sl, field_out_f(sl, h->bswap), dev);
        EMOO_CUDA(cudaGetLastError());
    } else {
        EMOO_TRY(mixed_ad_kinetic(h, handle_view(h), os.species, os.xlo, os.xhi, dev, nullptr));
    }
    EMOO_CUDA(cudaMemcpyAsync(out, dev, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return EMOO_OK;
}

struct LedgerM {
    std::vector<AdBcOp> ops;
    double *sums = nullptr;
    size_t cap = 0;
};

// Adjoints of plane sets, last first, each recorded in the ledger.
int planes_adj_m(emoo_handle *h, const std::vector<AdBcOp> &ops, float *const *lslot, LedgerM &pl) {
    for (auto it = ops.rbegin(); it != ops.rend(); ++it) {
        const AdBcOp &op = *it;
        if (op.kind != 1) continue;
        if (pl.ops.size() >= pl.cap) return EMOO_ERR_STATE;
        double *sums = pl.sums + 2 * adf::PLANE_BLOCKS * pl.ops.size();
        pl.ops.push_back(op);
        h->launches++;
        adf::k_plane_adj<float><<<adf::PLANE_BLOCKS, 256, 0, h->stream>>>(h->g, lslot[op.slot], op.dim, op.idx, op.t1,
                                                                          op.t2, sums);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// Adjoint of the corrected policy's whole-range periodic copies (fold = 0) or
// folds (fold = 1) of the float adjoint slots `ids`, with the mirror folds of
// J at reflecting walls (fold = 1): dimensions and sides reversed.
int periodic_full_adj_m(emoo_handle *h, float *const *lslot, const int *ids, int nids, int fold) {
    const Geom &g = h->g;
    adf::Slots9T<float> fl{};
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
                adf::k_mirror_fold_adj<float><<<grd, blk, 0, h->stream>>>(g, fl, d, r);
            }
            continue;
        }
        dim3 grd((g.tot[o2] + 31) / 32, (g.tot[o1] + 7) / 8, nids);
        h->launches++;
        adf::k_periodic_full_adj<float><<<grd, blk, 0, h->stream>>>(g, fl, d, fold);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// The field part of one corrected step in reverse (forward: J fold, E half,
// E images, planes, B half, E/B/B_tm1 images, planes), the FP64 form's
// sequence on the float adjoint slots; leaves the current adjoint in the J
// slots for the particle kernel.
int adj_fields_corrected_m(emoo_handle *h, const MSnap &S, const std::vector<AdBcOp> &ops, float *const *lslot,
                           LedgerM &pl) {
    static const int ids_e[3] = {EMOO_EX, EMOO_EY, EMOO_EZ};
    static const int ids9[9] = {EMOO_EX, EMOO_EY, EMOO_EZ, EMOO_BX, EMOO_BY, EMOO_BZ,
                                EMOO_BX_TM1, EMOO_BY_TM1, EMOO_BZ_TM1};
    static const int ids_j[3] = {EMOO_JX, EMOO_JY, EMOO_JZ};
    const Geom &g = h->g;
    const FOutF A = field_out_f(lslot, S.bswap ^ 1);
    JPtrsF LJ{{lslot[EMOO_JX], lslot[EMOO_JY], lslot[EMOO_JZ]}};
    dim3 blk(32, 8);
    const adf::YeeCoef<float> yc = adf::yee_coef<float>(g, h->dtp);
    EMOO_TRY(planes_adj_m(h, ops, lslot, pl));
    EMOO_TRY(periodic_full_adj_m(h, lslot, ids9, 9, 0));
    h->launches += 2;
    adf::k_yee_b_adj<float><<<grid_all_m(g, blk), blk, 0, h->stream>>>(g, yc, A);
    // the B half overwrote the B role's physical points
    adf::Slots9T<float> lb{{A.B[0], A.B[1], A.B[2]}};
    adf::k_clear_phys<float><<<dim3((g.n[2] + 31) / 32, (g.n[1] + 7) / 8, g.n[0]), blk, 0, h->stream>>>(g, lb);
    EMOO_TRY(planes_adj_m(h, ops, lslot, pl));
    EMOO_TRY(periodic_full_adj_m(h, lslot, ids_e, 3, 0));
    h->launches++;
    adf::k_yee_e_adj<float><<<grid_all_m(g, blk), blk, 0, h->stream>>>(g, yc, A, LJ);
    EMOO_TRY(periodic_full_adj_m(h, lslot, ids_j, 3, 1));
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

// adjoint of one step, given the state before it (S) and the cell array of
// the state after it
int adj_step_m(emoo_handle *h, AdRunM &R, const MSnap &S, const int32_t *cell_after, float *const lo[3],
               float *const lu[3], float *const *lslot, LedgerM &pl, unsigned long long *mismatch) {
    const Geom &g = h->g;
    const int b1 = S.bswap ^ 1;  // B roles after the step's Yee update
    std::vector<AdBcOp> ops;
    {
        const double t_save = h->t;
        const int b_save = h->bswap;
        h->t = S.t;
        h->bswap = b1;
        const int rc = ad_bc_ops(h, ops);
        h->t = t_save;
        h->bswap = b_save;
        EMOO_TRY(rc);
    }
    if (h->policy == EMOO_POLICY_CORRECTED) {
        EMOO_TRY(adj_fields_corrected_m(h, S, ops, lslot, pl));
        const FOutF LF = field_out_f(lslot, S.bswap);
        const float *lj[3] = {lslot[EMOO_JX], lslot[EMOO_JY], lslot[EMOO_JZ]};
        float *lE[3] = {LF.E[0], LF.E[1], LF.E[2]}, *lB[3] = {LF.B[0], LF.B[1], LF.B[2]},
              *lT[3] = {LF.T[0], LF.T[1], LF.T[2]};
        return mixed_ad_particles(h, R.view(S), cell_after, lo, lu, lj, lE, lB, lT, mismatch);
    }
    for (auto it = ops.rbegin(); it != ops.rend(); ++it) {
        const AdBcOp &op = *it;
        if (op.kind == 0) {
            Slots6F fl{{lslot[EMOO_EX], lslot[EMOO_EY], lslot[EMOO_EZ], lslot[EMOO_BX], lslot[EMOO_BY], lslot[EMOO_BZ]}};
            for (int d = 2; d >= 0; d--) {
                if (!((op.mask >> d) & 1)) continue;
                const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
                dim3 blk(32, 8);
                dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, 6);
                for (int side = 1; side >= 0; side--) {
                    h->launches++;
                    adf::k_ghost_adj<float><<<grd, blk, 0, h->stream>>>(g, fl, d, side);
                }
            }
        } else {
            if (pl.ops.size() >= pl.cap) return EMOO_ERR_STATE;
            double *sums = pl.sums + 2 * adf::PLANE_BLOCKS * pl.ops.size();
            pl.ops.push_back(op);
            h->launches++;
            adf::k_plane_adj<float><<<adf::PLANE_BLOCKS, 256, 0, h->stream>>>(g, lslot[op.slot], op.dim, op.idx, op.t1,
                                                                              op.t2, sums);
        }
    }
    EMOO_CUDA(cudaGetLastError());
    FOutF A = field_out_f(lslot, b1);
    JPtrsF LJ{{lslot[EMOO_JX], lslot[EMOO_JY], lslot[EMOO_JZ]}};
    dim3 blk(32, 8);
    h->launches += 2;
    const adf::YeeCoef<float> yc = adf::yee_coef<float>(g, h->dtp);
    adf::k_yee_b_adj<float><<<grid_all_m(g, blk), blk, 0, h->stream>>>(g, yc, A);
    adf::k_yee_e_adj<float><<<grid_all_m(g, blk), blk, 0, h->stream>>>(g, yc, A, LJ);
    for (int d = 2; d >= 0; d--) {
        if (h->bc.fbc[2 * d] != FBC_PERIODIC) continue;
        const int f0 = (d == 0) ? EMOO_JY : EMOO_JX;
        const int f1 = (d == 2) ? EMOO_JY : EMOO_JZ;
        const int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
        dim3 grd((g.n[o2] + 31) / 32, (g.n[o1] + 7) / 8, 2);
        h->launches++;
        adf::k_fold_adj<float><<<grd, blk, 0, h->stream>>>(g, d, lslot[f0], lslot[f1]);
    }
    EMOO_CUDA(cudaGetLastError());
    const FOutF LF = field_out_f(lslot, S.bswap);
    const float *lj[3] = {lslot[EMOO_JX], lslot[EMOO_JY], lslot[EMOO_JZ]};
    float *lE[3] = {LF.E[0], LF.E[1], LF.E[2]}, *lB[3] = {LF.B[0], LF.B[1], LF.B[2]},
          *lT[3] = {LF.T[0], LF.T[1], LF.T[2]};
    return mixed_ad_particles(h, R.view(S), cell_after, lo, lu, lj, lE, lB, lT, mismatch);
}

}  // namespace

int ad_run_mixed(emoo_handle *h, const emoo_ad_spec *spec, int mode, emoo_ad_result *out, double *grad_theta,
                 double *grad_v) {
    if (mode == EMOO_AD_TANGENT) return EMOO_ERR_UNSUPPORTED;
    if (h->opts.deposit_rho) h->rho_stale = 1;
    for (int s = 0; s < 6; s++)
        if (h->bc.pbc[s] == PBC_ABSORBING) h->dead_pending = 1;
    EMOO_TRY(mixed_ad_momentum_from_velocity(h));
    AdRunM R;
    R.h = h;
    const int64_t np0 = h->np;
    R.cap = std::max<int64_t>(np0, 1);
    R.npts = h->g.npts;
    ObjM os;
    os.kind = spec->objective;
    os.sl = SlabM{spec->slab_lo + 1, spec->slab_hi + 1};
    os.species = spec->species;
    os.xlo = h->info.xyz0[0] + spec->slab_lo * h->g.d[0];
    os.xhi = h->info.xyz0[0] + spec->slab_hi * h->g.d[0];
    const int ntheta = emoo_ad_nparams(h);
    double *dev = (double *)R.alloc(sizeof(double));
    unsigned long long *mism = (unsigned long long *)R.alloc(sizeof(unsigned long long));
    if (!dev || !mism) return EMOO_ERR_OOM;
    EMOO_CUDA(cudaMemsetAsync(mism, 0, sizeof(unsigned long long), h->stream));
    memset(out, 0, sizeof(*out));
    cudaEvent_t ev[4];
    for (auto &e : ev) EMOO_CUDA(cudaEventCreate(&e));
    struct EvFree {
        cudaEvent_t *e;
        ~EvFree() {
            for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]);
        }
    } evfree{ev};
    // The store is sorted by cell at the start of every segment of
    // checkpoint_every steps (the whole run is one segment without
    // checkpoints); sort s leaves perm[s] (perm[s][i]: the index before the
    // sort of particle i after it) and the store's size before it.
    const int N = spec->nsteps;
    const int K = spec->checkpoint_every >= 1 ? spec->checkpoint_every : std::max(N, 1);
    const int nseg = std::max((N + K - 1) / K, 1);
    std::vector<uint32_t *> perm(nseg, nullptr);
    std::vector<int64_t> np_before(nseg, 0);
    auto segment_start = [&](int sgi) -> int {
        if (!perm[sgi] && !(perm[sgi] = (uint32_t *)R.alloc(sizeof(uint32_t) * (size_t)R.cap))) return EMOO_ERR_OOM;
        np_before[sgi] = h->np;
        return sort_with_permutation(h, perm[sgi]);
    };

    if (mode == EMOO_AD_FORWARD) {
        EMOO_CUDA(cudaEventRecord(ev[0], h->stream));
        for (int n = 0; n < N; n++) {
            if (n % K == 0) EMOO_TRY(segment_start(n / K));
            EMOO_TRY(primal_step_m(h));
        }
        EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
        EMOO_TRY(objective_m(h, os, dev, &out->objective));
        float ms = 0;
        EMOO_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        out->forward_ms = ms;
        return read_err(h);
    }

    // ---- adjoint: forward with checkpoints (after each segment's sort)
    std::vector<MSnap> ck(nseg);
    EMOO_CUDA(cudaEventRecord(ev[0], h->stream));
    for (int n = 0; n < N; n++) {
        if (n % K == 0) {
            EMOO_TRY(segment_start(n / K));
            EMOO_TRY(R.save(ck[n / K]));
        }
        EMOO_TRY(primal_step_m(h));
    }
    if (N == 0) {
        EMOO_TRY(segment_start(0));
        EMOO_TRY(R.save(ck[0]));
    }
    EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
    EMOO_TRY(objective_m(h, os, dev, &out->objective));
    {
        float ms = 0;
        EMOO_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        out->forward_ms = ms;
    }
    MSnap fin;
    EMOO_TRY(R.save(fin));
    // adjoint state: offsets and momenta per particle (two sets, for the
    // sorts' adjoints), the 13 field slots
    float *lam[6], *lam2[6], *lslot[NSLOT];
    for (int a = 0; a < 6; a++) {
        lam[a] = (float *)R.alloc(sizeof(float) * (size_t)R.cap);
        lam2[a] = (float *)R.alloc(sizeof(float) * (size_t)R.cap);
        if (!lam[a] || !lam2[a]) return EMOO_ERR_OOM;
        EMOO_CUDA(cudaMemsetAsync(lam[a], 0, sizeof(float) * R.cap, h->stream));
    }
    for (int k = 0; k < NSLOT; k++) {
        if (!(lslot[k] = (float *)R.alloc(sizeof(float) * (size_t)R.npts))) return EMOO_ERR_OOM;
        EMOO_CUDA(cudaMemsetAsync(lslot[k], 0, sizeof(float) * R.npts, h->stream));
    }
    if (os.kind == EMOO_AD_OBJ_FIELD) {
        float *sl[NSLOT] = {}, *E[3], *Bs[6];
        mixed_field_arrays(h, E, Bs);
        for (int c = 0; c < 3; c++) {
            sl[EMOO_EX + c] = E[c];
            sl[EMOO_BX + c] = Bs[c];
            sl[EMOO_BX_TM1 + c] = Bs[3 + c];
        }
        h->launches++;
        k_objective_field_seed_m<<<pblocks_m((int64_t)(os.sl.hi - os.sl.lo) * h->g.n[1] * h->g.n[2]), 256, 0,
                                   h->stream>>>(h->g, os.sl, field_out_f(sl, h->bswap), field_out_f(lslot, h->bswap));
        EMOO_CUDA(cudaGetLastError());
    } else {
        float *lu[3] = {lam[3], lam[4], lam[5]};
        EMOO_TRY(mixed_ad_kinetic(h, handle_view(h), os.species, os.xlo, os.xhi, nullptr, lu));
    }
    LedgerM pl;
    {
        std::vector<AdBcOp> ops;
        EMOO_TRY(ad_bc_ops(h, ops));
        size_t per = 0;
        for (const AdBcOp &op : ops) per += op.kind == 1;
        pl.cap = per * (size_t)N * (h->policy == EMOO_POLICY_CORRECTED ? 2 : 1);  // corrected: set twice a step
        if (pl.cap && !(pl.sums = (double *)R.alloc(sizeof(double) * 2 * adf::PLANE_BLOCKS * pl.cap)))
            return EMOO_ERR_OOM;
        pl.ops.reserve(pl.cap);
    }
    std::vector<MSnap> tape(std::min(K, std::max(N, 1)));
    float rec_ms = 0, rev_ms = 0;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
        const int n0 = sgi * K, n1 = std::min(N, n0 + K);
        EMOO_CUDA(cudaEventRecord(ev[1], h->stream));
        EMOO_TRY(R.restore(ck[sgi]));
        for (int n = n0; n < n1; n++) {
            EMOO_TRY(R.save(tape[n - n0]));
            if (n + 1 < n1) EMOO_TRY(primal_step_m(h));
        }
        EMOO_CUDA(cudaEventRecord(ev[2], h->stream));
        for (int n = n1 - 1; n >= n0; n--) {
            // the recorded next state, in this segment's order (the next
            // checkpoint follows a sort, so the last step of a segment has none)
            const int32_t *after = n + 1 < n1 ? (const int32_t *)tape[n + 1 - n0].buf
                                              : (sgi + 1 == nseg ? (const int32_t *)fin.buf : nullptr);
            float *lo[3] = {lam[0], lam[1], lam[2]}, *lu[3] = {lam[3], lam[4], lam[5]};
            EMOO_TRY(adj_step_m(h, R, tape[n - n0], after, lo, lu, lslot, pl, mism));
        }
        // the adjoint of the segment's sort
        for (int a = 0; a < 6; a++)
            EMOO_CUDA(cudaMemsetAsync(lam2[a], 0, sizeof(float) * (size_t)np_before[sgi], h->stream));
        if (ck[sgi].np) {
            Lam6 src{{lam[0], lam[1], lam[2], lam[3], lam[4], lam[5]}};
            Lam6 dst{{lam2[0], lam2[1], lam2[2], lam2[3], lam2[4], lam2[5]}};
            h->launches++;
            k_unsort_adjoint<<<(unsigned)((ck[sgi].np + 255) / 256), 256, 0, h->stream>>>(src, dst, perm[sgi],
                                                                                            ck[sgi].np);
            EMOO_CUDA(cudaGetLastError());
        }
        for (int a = 0; a < 6; a++) std::swap(lam[a], lam2[a]);
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
    {
        unsigned long long m = 0;
        EMOO_CUDA(cudaMemcpy(&m, mism, sizeof(m), cudaMemcpyDeviceToHost));
        h->ad_cell_mismatch = (int64_t)m;
    }
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
    if (grad_v && np0) {
        // d objective / d v (gamma held) = gamma d objective / d u, gamma from
        // the run's start; the adjoints are in the store's order before the
        // run, the first checkpoint in the order after the first sort
        const int64_t n = ck[0].np;
        std::vector<uint32_t> p0(n);
        std::vector<float> u(n), l(np0);
        std::vector<double> g(np0, 1.0);
        const bool rel = h->info.relativity != 0;
        if (n) EMOO_CUDA(cudaMemcpy(p0.data(), perm[0], sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
        if (rel && n) {
            const MSnapView v0 = R.view(ck[0]);
            std::vector<double> g2(n, 0.0);
            for (int a = 0; a < 3; a++) {
                EMOO_CUDA(cudaMemcpy(u.data(), v0.u[a], sizeof(float) * n, cudaMemcpyDeviceToHost));
                for (int64_t i = 0; i < n; i++) g2[i] += (double)u[i] * (double)u[i];
            }
            for (int64_t i = 0; i < n; i++) g[p0[i]] = std::sqrt(1.0 + g2[i]);
        }
        for (int a = 0; a < 3; a++) {
            EMOO_CUDA(cudaMemcpy(l.data(), lam[3 + a], sizeof(float) * np0, cudaMemcpyDeviceToHost));
            for (int64_t q = 0; q < np0; q++) grad_v[a * np0 + q] = g[q] * l[q];
        }
    }
    EMOO_TRY(R.restore(fin));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    return read_err(h);
}

}  // namespace emoo
