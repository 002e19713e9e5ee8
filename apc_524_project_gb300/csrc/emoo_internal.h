// emoo_internal.h - handle layout and kernel launcher declarations shared by
// the host API (api.cpp) and the CUDA translation units.
#ifndef EMOO_INTERNAL_H
#define EMOO_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "emoo.h"

namespace emoo {

constexpr double UNIT_ACC = 0.58668774;       // src/globals.hpp:12
constexpr double UNIT_RHOJ = 4.80320427e-13;  // src/globals.hpp:16
constexpr double PI_D = 3.14159265358979323846;
constexpr int ITER_MAX = 10000;  // src/poisson/poisson.cpp:14
constexpr double CONV_CRIT = 1e-12;
constexpr double CONV_RATIO = 1e-9;

enum { PBC_PERIODIC = 0, PBC_REFLECTING = 1, PBC_ABSORBING = 2 };
enum { FBC_PERIODIC = 0, FBC_EXTERNAL = 1 };

// Device error word bits.
enum { ERR_BOUNDS = 1, ERR_FIXED_OVERFLOW = 2, ERR_NAN = 4 };

// Grid geometry in the reference layout: (n+3)^3 points per field, C order,
// physical points 1..n, ghost planes 0 and n+1, extra plane n+2
// (src/grid/grid.cpp:17-43).
struct Geom {
    int n[3];
    int tot[3];
    int64_t sx, sy;  // strides of i and j (k is contiguous)
    int64_t npts;
    int cny, cnz;    // strides of the reference cellID: (ny+2)(nz+2) * ix + (nz+2) * iy + iz
    int64_t ncell;   // (nx+2)(ny+2)(nz+2): cellID range
    double x0[3], L[3], d[3], id[3];
    int p2[3];  // d[i] is a power of two: x / d == x * id exactly
    double vol, ivol;
    int vol_p2;
    double area[3], iarea[3];  // area[i] = d[j] * d[k], j,k the other two axes in cyclic order
    int area_p2[3];
    // gather / deposit vertex of cell i: x0 + d (i - vshift); 0 the reference's
    // ghost-offset vertex, 1 the cell's own lower corner (corrected policy)
    int vshift = 0;
};

// Host-resident particles (emoo_attach_particles): the caller's FP64 arrays
// per species, and the geometry the fused kernel converts with. Lives in
// device memory; the kernel reads it through one pointer.
struct MHost {
    Geom g;
    int rel;
    double *x[EMOO_NSPEC], *y[EMOO_NSPEC], *z[EMOO_NSPEC];
    double *vx[EMOO_NSPEC], *vy[EMOO_NSPEC], *vz[EMOO_NSPEC], *gam[EMOO_NSPEC];
};

// Per-species constants, precomputed on the host in the reference's order of
// operations so the device arithmetic stays bit-identical to the reference.
struct SpeciesTab {
    int nspec;
    int64_t off[EMOO_NSPEC + 1];  // species s occupies [off[s], off[s+1])
    double q[EMOO_NSPEC], m[EMOO_NSPEC];
    double qp[EMOO_NSPEC];   // ((0.5 * dt * q) / m) * UNIT_ACC   (src/pusher/boris.cpp:34-35)
    double uq[EMOO_NSPEC];   // UNIT_RHOJ * q                      (src/particles/deposit.cpp:30)
    double cr[EMOO_NSPEC];   // (UNIT_RHOJ * (q / vol)) / vol      (src/particles/deposit.cpp:53)
    int deposit[EMOO_NSPEC]; // 0 for test-particle species
};

// Boundary kinds per side (x-, x+, y-, y+, z-, z+).
struct BCTab {
    int pbc[6];
    int fbc[6];
    double xmin[3], xmax[3];
};

struct DevCounters {
    unsigned long long cross[6];
    unsigned long long err;
    unsigned long long pad;
};

// One LightBC plane write (src/grid/lightBC.cpp:196-197). With a transverse
// profile (shaped waves with a spot) the value at transverse point (p, q) of
// the plane is v + vs t1[p] t2[q]; t1 / t2 (t1f / t2f for the FP32 grid) are
// the spot's per-axis factors, null for the reference's uniform plane.
struct PlaneSet {
    double *f = nullptr;
    int dim = 0, idx = 0;
    double v = 0.0;
    double vs = 0.0;
    const double *t1 = nullptr, *t2 = nullptr;
    const float *t1f = nullptr, *t2f = nullptr;
};

// One operation of executeBC(-1) on the FP64 slots, for the differentiated
// step: a periodic ghost copy of the E / B slots over the dims in `mask`, or
// a plane set of slot `slot` to value + vs t1[p] t2[q], with the derivatives
// of value (ku, cu) and of vs (ks, cs) with respect to the wave parameters
// (parameter 2 w: amplitude of wave w, 2 w + 1: its phase in degrees,
// 2 nwaves + EMOO_NCOEF w + k: its envelope coefficient k).
struct AdBcOp {
    int kind;  // 0 ghost copy, 1 plane set
    int mask;
    int slot, dim, idx;
    double value, vs;
    const double *t1, *t2;
    std::vector<int> ku, ks;
    std::vector<double> cu, cs;
};

struct FieldsF32;  // mixed-form grid storage (particles_mixed.cu)

}  // namespace emoo

struct emoo_handle {
    emoo_input_info info;
    emoo_opts opts;
    int dev = 0;
    cudaStream_t stream = nullptr;
    emoo::Geom g;
    emoo::BCTab bc;
    int poisson = 0;
    int precision = EMOO_FP64;

    // FP64 grid: storage slots indexed like the reference fieldPtr_.
    double *slot[EMOO_NFIELDS] = {};
    int bswap = 0;  // B / B_tm1 member roles exchanged (see evolveFields)

    // particles (species-major segments)
    int nspec = 0;
    int64_t cap = 0;
    int64_t np = 0;
    int64_t count[EMOO_NSPEC] = {};
    int64_t off[EMOO_NSPEC + 1] = {};
    // FP64 SoA
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr, *gam = nullptr;
    double *fcache = nullptr;  // 6 * cap interpolated fields (allocated on demand)
    int64_t *ids = nullptr;
    // mixed SoA
    int32_t *cell = nullptr;
    float *ox = nullptr, *oy = nullptr, *oz = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr;
    // relativistic mixed form until the first push: the loaded gamma (the
    // momentum slots hold the loaded velocity); freed by the first push
    float *g0 = nullptr;
    int first_push = 0;
    emoo::FieldsF32 *mf = nullptr;

    // sort scratch
    uint32_t *key[2] = {nullptr, nullptr};
    uint32_t *perm[2] = {nullptr, nullptr};
    uint32_t *hist = nullptr;
    uint32_t *scan_tmp = nullptr;
    size_t hist_cap = 0, scan_cap = 0;
    void *pay = nullptr;   // scratch of cap 8-byte elements (staging, and the sort's 8-byte payload swaps)
    size_t pay_bytes = 0;
    void *pay4 = nullptr;  // scratch of cap 4-byte elements (the sort's 4-byte payload swaps)
    int64_t *d_spec_count = nullptr;

    // reductions and counters
    emoo::DevCounters *ctr = nullptr;
    double *red = nullptr;  // reduction partials
    size_t red_cap = 0;
    void *jacobi_state = nullptr;
    int poisson_solver = 0;      // EMOO_POISSON_JACOBI / EMOO_POISSON_MULTIGRID
    double poisson_rtol = 1e-10; // multigrid stop, relative to the start residual
    void *mg = nullptr;          // multigrid levels (multigrid.cu), kept between solves
    // host-resident particles: the attached arrays are the state; the device
    // store is refreshed from them (store_stale) before anything reads it
    struct Attached {
        int64_t n = -1;  // -1: not attached
        double *p[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    } attached[EMOO_NSPEC];
    int host_mode = 0;
    int store_stale = 0;
    emoo::MHost *mhost = nullptr;  // device copy of the attached pointers

    double dt = 0.0;    // configured step
    double t = 0.0;     // time_phys
    double dtp = 0.0;   // dt_phys (zero during field initialisation, like the reference)
    int64_t step_index = 0;
    int64_t next_hist = 0;
    std::vector<double> hist_rows;
    int fields_initialised = 0;
    // shaped injected waves (emoo_set_wave_shape) and the transverse spot
    // factors of each external side and polarisation: for side s and E
    // component p, wprof + ((3 s + p) 2 + a) wprof_stride holds the factor
    // along the plane's first (a = 0) or second (a = 1) transverse axis
    emoo_wave_shape wshape[EMOO_NWAVE] = {};
    int wshaped[EMOO_NWAVE] = {};
    int wspot[6][3] = {};
    double *wprof = nullptr;
    float *wproff = nullptr;
    int wprof_stride = 0;
    // The loop never reads rho, so emoo_step deposits J only and leaves rho
    // pending: it is deposited (with fold and background) at the particles'
    // positions when something reads it or before the particles change.
    int rho_stale = 0;
    int rho_bg_first = 1;  // first physical x index the immobile background covers
    // Absorbing walls mark removed particles (FP64: x = NaN, mixed: cell < 0)
    // and the loop skips them; they leave the store at the next sort, or at
    // the next call that reads or changes the particle store (compaction).
    int dead_pending = 0;
    // last mixed-form adjoint run: particles whose recomputed cell after a
    // step disagreed with the recorded one (0 when the recomputation is the
    // primal's, as it is by construction)
    int64_t ad_cell_mismatch = 0;
    int policy = EMOO_POLICY_REFERENCE;

    // instrumentation: kernel launches issued, and CUDA-event timing of the
    // fused particle kernel (the dominant kernel of the step) when enabled
    int64_t launches = 0;
    int prof_on = 0;
    cudaEvent_t prof_ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> prof_pending;  // (start, stop) pairs not yet read
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms = 0.0;
    int64_t prof_count = 0;
};

namespace emoo {

// ---- geometry ----
void make_geom(const emoo_input_info &in, Geom &g);

// ---- FP64 field kernels (fields_f64.cu) ----
int yee_f64(emoo_handle *h, double dt);
int yee_es_f64(emoo_handle *h, double dt);
int ghost_fill_f64(emoo_handle *h, const int *ids, int nids, int dims_mask);
constexpr int FOLD_J = 1, FOLD_RHO = 2, FOLD_ALL = 3;
int fold_f64(emoo_handle *h, int dim, int what = FOLD_ALL);
// corrected policy: periodic folds (J and rho) and ghost copies (E, B, B_tm1)
// over the whole transverse range, dimension by dimension
int fold_full_f64(emoo_handle *h, int what);
int ghost_full_f64(emoo_handle *h);
int ghost_e_full_f64(emoo_handle *h);
// one half of yee_f64 with the current B roles and no boundary work: E (half
// 0) or B (half 1); and the corrected policy's periodic ghost copies alone
int yee_half_f64(emoo_handle *h, double dt, int half);
int periodic_copies_f64(emoo_handle *h, const int *ids, int nids);
int poisson_field_bc(emoo_handle *h, int id);
int multigrid_f64(emoo_handle *h, int id1, int id2, int rid, double mult, int *cycles, int *converged);
int mixed_step_host(emoo_handle *h, double dtp, int fold_what, int store_pre);
int mixed_moments(emoo_handle *h, double out4[4]);
int mixed_interpolate(emoo_handle *h);
int mixed_push_cached(emoo_handle *h);
int mixed_particle_bc(emoo_handle *h);
int mixed_field_energy(emoo_handle *h, double out6[6]);
bool mixed_device_accessible(const emoo_handle *h, const void *p);
// host-resident particles: refresh the device store from the attached arrays
// when a streamed step left it stale (every entry point that reads the store
// calls it); EMOO_ERR_STATE from entry points that would change the store
int host_store_sync(emoo_handle *h);
void multigrid_free(emoo_handle *h);
int plane_set_f64(emoo_handle *h, const PlaneSet *ps, int n);
int jacobi_f64(emoo_handle *h, int id1, int id2, int rid, double tol, double mult, int *iters, int *converged);
int phi_to_e_f64(emoo_handle *h);
int a_to_b_f64(emoo_handle *h);
int field_energy_f64(emoo_handle *h, double out6[6]);
int gauss_residual_f64(emoo_handle *h, double out2[2]);
int fill_f64(emoo_handle *h, double *p, int64_t n, double v, cudaStream_t s);
int rho_background_f64(emoo_handle *h, int with_rho);  // rho += opts.rho_background at the physical points

// ---- FP64 particle kernels (particles_f64.cu) ----
void species_tab(emoo_handle *h, double dtp, SpeciesTab &st);
int interpolate_f64(emoo_handle *h);
int push_cached_f64(emoo_handle *h, double dtp);
int particle_bc_f64(emoo_handle *h);
int perturb_f64(emoo_handle *h, uint64_t seed, double rel);
int deposit_f64(emoo_handle *h, int with_rho);
int fused_step_f64(emoo_handle *h, double dtp, int with_rho);
int deposit_rho_f64(emoo_handle *h);  // rho alone at the current positions, plus the background
int particle_moments_f64(emoo_handle *h, double out4[4]);
int sort_keys_f64(emoo_handle *h);
int compact_keys_f64(emoo_handle *h);  // species index, nspec for removed particles

// ---- sort (sort.cu) ----
int radix_sort_perm(emoo_handle *h, int64_t n, int key_bits);
// Permutes the particle store through perm[0]; cells_from_keys (mixed form,
// after mixed_sort_keys): the cells come from the sorted keys instead.
int gather_payload(emoo_handle *h, int64_t n, bool cells_from_keys = false);
int count_species(emoo_handle *h, int64_t n, int64_t stride, int64_t *counts_host);

// ---- loader (loader.cu) ----
int generate_device(emoo_handle *h, const emoo_gen_params *gp, int64_t first, int64_t n, int64_t dst);

// ---- mixed form (particles_mixed.cu) ----
int mixed_alloc(emoo_handle *h);
void mixed_free(emoo_handle *h);
int mixed_from_f64(emoo_handle *h, int64_t first, int64_t n, const double *x, const double *y, const double *z,
                   const double *vx, const double *vy, const double *vz, const double *gam);
int mixed_to_f64(emoo_handle *h, int64_t first, int64_t n, double *x, double *y, double *z, double *vx,
                 double *vy, double *vz, double *gam);
int mixed_step(emoo_handle *h, double dtp, int with_rho, int fold_what);
int mixed_materialize_rho(emoo_handle *h);
int mixed_sort_keys(emoo_handle *h);
int mixed_compact_keys(emoo_handle *h);

// ---- differentiation of the mixed step (particles_mixed.cu) ----
// A particle and field state of the mixed form (a snapshot, or the handle's
// own arrays): cell, offsets, momenta; E and the B / B_tm1 roles.
struct MSnapView {
    const int32_t *cell;
    const float *o[3], *u[3];
    const float *E[3], *B[3], *T[3];
};
void mixed_field_arrays(emoo_handle *h, float *E[3], float *Bslot[6]);
void mixed_point_arrays(emoo_handle *h, long long *J[4], double *q0);
int mixed_ad_momentum_from_velocity(emoo_handle *h);
int mixed_ad_particles(emoo_handle *h, const MSnapView &S, const int32_t *cell_after, float *const lo[3],
                       float *const lu[3], const float *const lj[3], float *const lE[3], float *const lB[3],
                       float *const lT[3], unsigned long long *mismatch);
int mixed_ad_kinetic(emoo_handle *h, const MSnapView &S, int species, double xlo, double xhi, double *dev_out,
                     float *const lu[3]);
// the mixed form's differentiated run (adjoint_mixed.cu), behind emoo_ad_run
int ad_run_mixed(emoo_handle *h, const emoo_ad_spec *spec, int mode, emoo_ad_result *out, double *grad_theta,
                 double *grad_v);
int mixed_get_field(emoo_handle *h, int id, double *out_dev);
int mixed_set_field(emoo_handle *h, int id, const double *in_dev);
int mixed_moments(emoo_handle *h, double out4[4]);
int mixed_field_energy(emoo_handle *h, double out6[6]);
int mixed_ghost_fill(emoo_handle *h);
int mixed_plane_sets(emoo_handle *h, const PlaneSet *ps, int n);
int mixed_deposit(emoo_handle *h, int with_rho);
int mixed_fold_public(emoo_handle *h);
int mixed_yee_public(emoo_handle *h, double dtp, int es);
int mixed_deposit_to_f64(emoo_handle *h);
int mixed_fields_from_slots(emoo_handle *h);
int mixed_fields_to_slots(emoo_handle *h);
int mixed_const_fields(emoo_handle *h);
int mixed_key_bits(emoo_handle *h);

// ---- helpers ----
int cuda_status(cudaError_t e);
int read_err(emoo_handle *h);
int prof_accumulate(emoo_handle *h);

// ---- differentiation support (api.cpp) ----
int ad_execute_bc(emoo_handle *h, int send_id);
int ad_bc_ops(emoo_handle *h, std::vector<AdBcOp> &ops);
int light_planes_public(emoo_handle *h, int s, PlaneSet *ps);
int light_planes_slots(emoo_handle *h, int s, PlaneSet *ps);  // the FP64 slots' planes
int sort_with_permutation(emoo_handle *h, uint32_t *perm_out);
int reserve_store(emoo_handle *h, int64_t cap);  // particle capacity, contents kept

}  // namespace emoo

#define EMOO_CUDA(call)                                        \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return emoo::cuda_status(e_);   \
    } while (0)

#define EMOO_TRY(call)              \
    do {                            \
        int rc_ = (call);           \
        if (rc_ != EMOO_OK) return rc_; \
    } while (0)

#endif
