/*
 * emoo.h - C ABI of the GB300 (sm_103a) EMOOPIC per-timestep PIC loop.
 *
 * One opaque handle owns one device-resident simulation domain on one GPU:
 * the Yee grid (reference layout: (n+3)^3 points per field, C order
 * [i][j][k], one ghost layer plus one extra plane, field IDs as in the
 * reference Grid) and a structure-of-arrays particle store sorted by cell.
 *
 * Every entry point returns an int status (EMOO_OK = 0, negative on error),
 * throws nothing across the ABI and is synchronous unless documented
 * otherwise. A handle is owned by one host thread; all of its work runs on
 * the handle's own CUDA stream.
 *
 * Each declaration cites the reference interface it replaces as
 * path:line inside the reference project (DenSto/APC_524_Project).
 */
#ifndef EMOO_H
#define EMOO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMOO_NDIM 3
#define EMOO_NCHAR 64
#define EMOO_NSPEC 32
#define EMOO_NWAVE 32

/* Status codes. */
#define EMOO_OK 0
#define EMOO_ERR_ARG (-1)            /* bad argument (null pointer, out-of-range id, size) */
#define EMOO_ERR_OOM (-2)            /* device or host allocation failed, or capacity exceeded */
#define EMOO_ERR_NOT_CONVERGED (-3)  /* Poisson solve reached its iteration (Jacobi) or cycle (multigrid) cap */
#define EMOO_ERR_FIXED_OVERFLOW (-4) /* fixed-point current/charge accumulator saturated */
#define EMOO_ERR_BOUNDS (-5)         /* a device-side bounds check recorded a bad index */
#define EMOO_ERR_CUDA (-6)           /* a CUDA runtime call failed */
#define EMOO_ERR_INPUT (-7)          /* input file missing, unparsable or inconsistent */
#define EMOO_ERR_STATE (-8)          /* call not valid in the handle's current state */
#define EMOO_ERR_UNSUPPORTED (-9)    /* option combination not implemented */

/* Precision forms. */
#define EMOO_FP64 0  /* FP64 positions, velocities, fields and current (reference parity form) */
#define EMOO_MIXED 1 /* int32 cell + FP32 offset, FP32 momentum and fields, int64 fixed-point current */

/* Field IDs, src/grid/grid.cpp:44-60 (Grid) and src/poisson/poisson.cpp:98-111 (Poisson_Solver). */
#define EMOO_EX 0
#define EMOO_EY 1
#define EMOO_EZ 2
#define EMOO_BX 3
#define EMOO_BY 4
#define EMOO_BZ 5
#define EMOO_JX 6
#define EMOO_JY 7
#define EMOO_JZ 8
#define EMOO_RHO 9
#define EMOO_BX_TM1 10
#define EMOO_BY_TM1 11
#define EMOO_BZ_TM1 12
#define EMOO_PHI1 13
#define EMOO_AX1 14
#define EMOO_AY1 15
#define EMOO_AZ1 16
#define EMOO_PHI2 17
#define EMOO_AX2 18
#define EMOO_AY2 19
#define EMOO_AZ2 20
#define EMOO_NFIELDS 21

/* Boundary-condition exchange selectors of Grid::executeBC(sendID),
 * src/grid/spookyGrid.cpp:8-16: -1 = E,B ghost fill; -2 = periodic fold of
 * J-perp and rho; >= 0 = one field. */
#define EMOO_SEND_EB (-1)
#define EMOO_SEND_JRHO (-2)

/*
 * Run configuration. Binary-identical to the reference's Input_Info_t
 * (src/IO/input.hpp:15-126): same members, same order, same array bounds
 * (long is 64-bit on the LP64 targets this library supports), so the
 * reference parser's output can be handed over unchanged.
 */
typedef struct emoo_input_info {
    int nCell[EMOO_NDIM];
    int nProc[EMOO_NDIM];
    int nt;
    int restart;
    int debug;
    int relativity;
    int electrostatic;
    int nspecies;
    int nstep_fields;
    int nstep_parts;
    int nstep_restart;
    int nstep_sort;
    int which_fields;
    int output_pCount;
    int nwaves;
    int inSide[EMOO_NWAVE];
    int inPolE[EMOO_NWAVE];
    int isTestParticle[EMOO_NSPEC];
    int64_t nparticles_tot;
    int64_t nparticles_domain;
    double t0;
    double dens_phys;
    double super_ratio;
    double mass_ratio[EMOO_NSPEC];
    double charge_ratio[EMOO_NSPEC];
    double dens_frac[EMOO_NSPEC];
    double temp[EMOO_NSPEC];
    double peakamps[EMOO_NWAVE];
    double omegas[EMOO_NWAVE];
    double phases[EMOO_NWAVE];
    double invWidths[EMOO_NWAVE];
    double delays[EMOO_NWAVE];
    double E0[EMOO_NDIM];
    double B0[EMOO_NDIM];
    double bound_phi[2 * EMOO_NDIM];
    double bound_Ax[2 * EMOO_NDIM];
    double bound_Ay[2 * EMOO_NDIM];
    double bound_Az[2 * EMOO_NDIM];
    double xyz0[EMOO_NDIM];
    double Lxyz[EMOO_NDIM];
    char distname[EMOO_NCHAR];
    char parts_init[EMOO_NCHAR];
    char fields_init[EMOO_NCHAR];
    char parts_bound[2 * EMOO_NDIM][EMOO_NCHAR];
    char fields_bound[2 * EMOO_NDIM][EMOO_NCHAR];
} emoo_input_info;

/* Options the reference fixes in code. */
typedef struct emoo_opts {
    int precision;         /* EMOO_FP64 or EMOO_MIXED */
    int device;            /* CUDA device ordinal */
    double dt;             /* time step; <= 0 selects the reference's mindx/100 (src/main.cpp:213-214) */
    int64_t capacity;      /* particle capacity to reserve; 0 = nparticles_tot of the input */
    int track_ids;         /* 1 = carry a 64-bit particle id through sorts (needed to read back by id) */
    int deposit_rho;       /* 1 = deposit rho every step as the reference does (src/main.cpp:245) */
    int history_every;     /* history cadence in steps; the reference hard-codes 10 (src/IO/output.cpp:46) */
    double rho_background; /* uniform immobile background charge density added to rho, reference units */
    double rho_background_xmin; /* the background covers the physical points with x >= this
                                   (emoo_default_opts: -HUGE_VAL, every point) */
    int policy;            /* EMOO_POLICY_REFERENCE (default) or EMOO_POLICY_CORRECTED */
    int poisson_solver;    /* EMOO_POISSON_JACOBI (default) or EMOO_POISSON_MULTIGRID */
    double poisson_rtol;   /* multigrid stop: max |residual| <= rtol max |right side| (default 1e-10) */
} emoo_opts;

/* Field-start solvers for "poisson" initialisation. JACOBI is
 * Poisson_Solver::run_poisson_solver_ (src/poisson/poisson.cpp:172-287) with
 * its stop test and 10000-iteration cap, bit-compatible with the reference.
 * MULTIGRID (no reference counterpart) solves the same discrete equations -
 * the Jacobi iteration's fixed point: the 7-point Laplacian of phi (A) equals
 * -4 pi rho (J) at every unknown point, periodic dimensions wrapping and
 * external ones holding the PoissonBC planes 1 and n + 1 - by FP64 V-cycles
 * until max |residual| <= poisson_rtol max |right side|, in tens of cycles
 * where the Jacobi needs thousands of sweeps or never meets its test (on a
 * periodic grid with an even side the Jacobi iteration's odd-even mode does
 * not decay). With every dimension periodic the right side's mean is removed
 * and the potential's mean is set to zero, invisible to phiToE / AToB. The
 * iteration counts emoo_init_fields reports are then V-cycles. Both
 * dimensions' sides must be periodic, or both external, for MULTIGRID
 * (EMOO_ERR_UNSUPPORTED at emoo_create otherwise). */
#define EMOO_POISSON_JACOBI 0
#define EMOO_POISSON_MULTIGRID 1

/* Physics policies. REFERENCE reproduces the reference's arithmetic with its
 * quirks (ghost-offset gather / deposit vertex, the Jx index of Grid::addJ,
 * src/grid/oGrid.cpp:101, ghost copies and folds over the physical
 * transverse range only, current from the velocity at the new position).
 * CORRECTED (no reference counterpart; both forms; each dimension periodic,
 * or walled with reflecting or absorbing particle sides and external field
 * sides, EMOO_ERR_UNSUPPORTED otherwise): the cell's own lower corner as
 * vertex, the fixed Jx index, Villasenor and Buneman's charge-conserving
 * current along each particle's path (so rho(t + dt) - rho(t) + dt div J = 0
 * and the Gauss-law residual stays at its initial value; the current beyond
 * a reflecting wall folded back as its mirror image, a removed particle's
 * path continued past an absorbing wall), periodic copies and folds of every
 * component over the whole range, and E's boundary values (periodic images,
 * LightBC planes) set between the two halves of the Yee update as well as
 * after them (time-centred at the wrap and at the planes). */
#define EMOO_POLICY_REFERENCE 0
#define EMOO_POLICY_CORRECTED 1

/* Seeded sampler of one species (no reference counterpart: replaces the
 * sequential ran2 loader of src/particles/particle_handler.cpp:47-84 with
 * independent per-particle streams, identical on host and device). */
typedef struct emoo_gen_params {
    uint64_t seed;
    int species;
    int relativistic_gamma; /* 1: gamma = sqrt(1 - v^2), the reference loader's convention (particle_handler.cpp:77) */
    double x0[3], L[3];     /* sampling box */
    double vth[3];          /* thermal speed per axis */
    double vdrift[3];       /* drift velocity */
    double dens_amp;        /* delta n / n of a cos(2 pi k (x - x0) / Lx) modulation along x (0 = uniform) */
    double dens_k;          /* mode number k of that modulation */
} emoo_gen_params;

typedef struct emoo_handle emoo_handle;

/* Fills *o with the defaults (FP64, device 0, reference dt, rho every step, history every 10). */
int emoo_default_opts(emoo_opts *o);

/* Reads an input file in the reference's libconfig format into *out (zeroed
 * first). Replaces Input::readinfo, src/IO/readinfo.cpp:18-733: same setting
 * paths, defaults and required settings. Returns EMOO_ERR_INPUT with a
 * message (emoo_input_message) where the reference prints an error and
 * returns EXIT_FAILURE, and also where it would terminate on an uncaught
 * exception (missing relativity / electrostatic / output_pCount). Host only. */
int emoo_read_input(const char *path, emoo_input_info *out);

/* emoo_read_input on a string holding the file's text. */
int emoo_parse_input(const char *text, emoo_input_info *out);

/* Message of the last failed emoo_read_input / emoo_parse_input on this thread. */
const char *emoo_input_message(void);

/* Input::ProcessInfo, src/IO/check.cpp:12-147, for one domain: super-particle
 * scaling of mass, charge and temperature, density-fraction normalisation,
 * boundary consistency; EMOO_ERR_INPUT where the reference counts an error. */
int emoo_process_info(emoo_input_info *info);

/* Human-readable text of a status code. Never null. */
const char *emoo_strerror(int status);

/* Builds the device domain: Domain + Grid/Poisson_Solver + field and particle
 * boundaries + Particle_Handler with the pusher named by info->relativity.
 * Replaces src/main.cpp:115-150 (Domain, setPusher, Part_BC_Factory,
 * Grid/Poisson_Solver, Field_BC_Factory). All fields start at zero. */
int emoo_create(const emoo_input_info *info, const emoo_opts *opts, emoo_handle **out);

/* Frees everything the handle owns. Replaces src/main.cpp:307-316. */
int emoo_destroy(emoo_handle *h);

/* Copies n particles of species `species` from caller-owned host SoA arrays.
 * gamma may be null (then 0, like new_particle, src/particles/particle.cpp:4-21);
 * ids may be null (then consecutive from the current count). Replaces the
 * particle construction of Particle_Handler::Load,
 * src/particles/particle_handler.cpp:53-84. */
int emoo_load_particles(emoo_handle *h, int species, int64_t n, const double *x, const double *y,
                        const double *z, const double *vx, const double *vy, const double *vz,
                        const double *gamma, const int64_t *ids);

/* Host-side sampler: fills particles [first, first+n) of the stream described
 * by g into caller-owned arrays (gamma may be null). Pure host code. */
int emoo_generate_host(const emoo_gen_params *g, int64_t first, int64_t n, double *x, double *y, double *z,
                       double *vx, double *vy, double *vz, double *gamma);

/* Device-side sampler: appends particles [0, n) of the stream g to species
 * g->species directly in device memory; bit-identical to emoo_generate_host. */
int emoo_load_generated(emoo_handle *h, const emoo_gen_params *g, int64_t n);

/* Number of live particles of a species (all species when species < 0). */
int emoo_num_particles(emoo_handle *h, int species, int64_t *n);

/* Copies the particles of a species back to host arrays of capacity cap, in
 * device order; *n receives the count. gamma / ids may be null. */
int emoo_get_particles(emoo_handle *h, int species, int64_t cap, double *x, double *y, double *z,
                       double *vx, double *vy, double *vz, double *gamma, int64_t *ids, int64_t *n);

/* Copies the per-particle interpolated fields cached by emoo_interpolate
 * (the reference's Particle::field, src/particles/particle.hpp:4-7). */
int emoo_get_particle_fields(emoo_handle *h, int species, int64_t cap, double *e1, double *e2, double *e3,
                             double *b1, double *b2, double *b3, int64_t *n);

/* Whole-array field access in the reference layout: (n+3)^3 doubles, C order
 * [i][j][k]. Replaces Grid::getFieldPtr, src/grid/grid.hpp:68. */
int emoo_get_field(emoo_handle *h, int field_id, double *out);
int emoo_set_field(emoo_handle *h, int field_id, const double *in);

/* Reference getCellID for a position (ghost offset included),
 * src/grid/oGrid.cpp:208-227. Host-side, no device work. */
int emoo_cell_id(emoo_handle *h, double x, double y, double z, int *cell_id);

/* Field initialisation of src/main.cpp:159-179: for "poisson" deposit rho/J,
 * fold (-2), then the four Jacobi solves + phiToE + AToB + E/B ghost fill
 * (src/poisson/poisson.cpp:143-170); for "constant" E0/B0
 * (src/grid/grid.cpp:554-574). Then the per-particle interpolation.
 * iters (may be null) receives the four Jacobi iteration counts. */
int emoo_init_fields(emoo_handle *h, int iters[4]);

/* Poisson_Solver::InitializeFields alone, on whatever rho/J the grid holds,
 * src/poisson/poisson.cpp:143-170. Returns EMOO_ERR_NOT_CONVERGED (after
 * finishing exactly like the reference) when a solve hit ITER_MAX. */
int emoo_poisson_init(emoo_handle *h, int iters[4]);

/* Stable counting sort of each species by cell (ascending (ix,iy,iz)).
 * Replaces Particle_Handler::SortParticles, src/particles/particle_handler.cpp:180-183
 * (the reference uses an unstable std::sort, descending). */
int emoo_sort(emoo_handle *h);

/* Gathers E and (B + B_tm1)/2 at every particle into the per-particle field
 * cache. Replaces Particle_Handler::InterpolateEB,
 * src/particles/particle_handler.cpp:138-173. */
int emoo_interpolate(emoo_handle *h);

/* Pushes every particle with its cached field (Boris or relativistic Boris).
 * Replaces Particle_Handler::Push, src/particles/particle_handler.cpp:124-128. */
int emoo_push(emoo_handle *h);

/* Applies the six particle boundaries in the reference order (x-, x+, y-, y+,
 * z-, z+); counts6 (may be null) receives the crossings per side.
 * Replaces executeParticleBoundaryConditions + clearGhosts,
 * src/particles/particle_handler.cpp:287-295 and :271-284. */
int emoo_apply_particle_bc(emoo_handle *h, int64_t counts6[6]);

/* Zeroes J (and rho) and deposits every non-test particle.
 * Replaces Particle_Handler::depositRhoJ, src/particles/particle_handler.cpp:185-239. */
int emoo_deposit(emoo_handle *h, int with_rho);

/* Grid::executeBC(sendID), src/grid/grid.cpp:577-585. */
int emoo_execute_bc(emoo_handle *h, int send_id);

/* Grid::evolveFields / evolveFieldsES, src/grid/oGrid.cpp:15-81. */
int emoo_evolve_fields(emoo_handle *h, int electrostatic);

/* The fused time loop: nsteps passes of src/main.cpp:221-287 (sort every
 * nstep_sort, history every history_every, gather+push+BC+deposit in one
 * kernel, fold, Yee update, ghost fill). Crossing counts accumulate into
 * counts6 (may be null). With host-resident particles (emoo_attach_particles)
 * each step reads and writes the attached arrays. */
int emoo_step(emoo_handle *h, int nsteps, int64_t counts6[6]);

/* The history row of src/IO/output.cpp:52-123 for the current state:
 * {t, sum m vx, sum m vy, sum m vz, particle KE, B energy, E energy, total}. */
int emoo_history(emoo_handle *h, double out8[8]);

/* Rows recorded by emoo_step (every history_every steps, before the push,
 * like the reference). Copies up to cap rows of 8 doubles; *n = rows held.
 * EMOO_ERR_ARG: n null, or rows given with a negative cap. */
int emoo_history_rows(emoo_handle *h, int cap, double *rows, int *n);

/* Gauss-law residual of the current state: max and L2 norm over physical
 * vertices of (div E - 4 pi rho) (no reference counterpart). */
int emoo_gauss_residual(emoo_handle *h, double out2[2]);

/* Current simulation time and step size. */
int emoo_time(emoo_handle *h, double *t, double *dt);

/* Sensitivity probe (no reference counterpart; FP64 form only): multiplies
 * every live particle's velocity components and every point of E, B and
 * B_tm1 by (1 + rel u), and moves each position component by rel d u (kept
 * only inside the box), u uniform in [-1, 1) and independent per particle or
 * point and component, drawn from seed. With rel = 2^-24 applied after every
 * step, an ensemble of FP64 runs measures how far FP32 rounding alone moves
 * the loop's result: the bar the mixed form's error is stated against. */
int emoo_perturb(emoo_handle *h, uint64_t seed, double rel);

/* Device-side error word (bounds checks, fixed-point saturation) since the
 * last call; cleared by reading. */
int emoo_check(emoo_handle *h);

/* Host-resident particles (mixed form; no reference counterpart). Makes the
 * caller's FP64 arrays of one species (n = its current count, in the order
 * emoo_get_particles returns; gamma required for the relativistic pusher)
 * the particle state: once every species is attached, emoo_step streams
 * them through the GPU, reading and writing the arrays in place within one
 * kernel, so the host link carries both directions at once. The result
 * equals, bit for bit, emoo_set_particles + emoo_step(1) +
 * emoo_get_particles per step on the same arrays; a step that sorts or makes
 * the first push runs that way (a history row is taken from the state the
 * streamed kernel also leaves in the device store). The arrays must stay
 * valid and addressable by the GPU (pinned, or any host memory where the
 * device reads pageable memory); EMOO_ERR_UNSUPPORTED otherwise, for the FP64
 * form, or with absorbing particle boundaries (the arrays keep their
 * length). While attached, entry points that change the particle store
 * (load, set, sort, push, particle BCs, restart read, emoo_ad_run) return
 * EMOO_ERR_STATE; those that read it see the arrays' state; and
 * emoo_get_particles copies the arrays. emoo_detach_particles ends it, with
 * the device store holding the arrays' state. */
int emoo_attach_particles(emoo_handle *h, int species, int64_t n, double *x, double *y, double *z, double *vx,
                          double *vy, double *vz, double *gamma);
int emoo_detach_particles(emoo_handle *h);

/* Overwrites the state of the n particles of a species (n must equal its
 * current count) from caller-owned host SoA arrays, in device order (the
 * order emoo_get_particles returns). For callers that keep the particle
 * vector in host memory between steps, as the reference's Particle_Handler
 * does (src/particles/particle_handler.hpp:53). gamma may be null. */
int emoo_set_particles(emoo_handle *h, int species, int64_t n, const double *x, const double *y, const double *z,
                       const double *vx, const double *vy, const double *vz, const double *gamma);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events after the handle's. */
int emoo_get_stream(emoo_handle *h, void **stream);

/* Instrumentation counters. */
typedef struct emoo_stats {
    int64_t launches;       /* kernels launched by the handle so far */
    int64_t timed_launches; /* launches of the fused particle kernel timed since profiling was enabled */
    double timed_ms;        /* their summed CUDA-event durations */
    int64_t ad_cell_mismatch; /* last mixed-form adjoint run: particles whose recomputed cell disagreed (0) */
} emoo_stats;

/* Enables (1) or disables (0) CUDA-event timing of every fused particle
 * kernel launch; enabling resets the timed counters. */
int emoo_set_profiling(emoo_handle *h, int on);

/* Reads the counters (waits for the handle's stream). */
int emoo_get_stats(emoo_handle *h, emoo_stats *s);

/* Largest n emoo_sort_permutation_noalloc accepts. */
#define EMOO_NOALLOC_SORT_MAX 1048576

/* Stable sort permutation of n 32-bit keys that allocates no memory. It has
 * no counterpart in the reference: it is the scratch-free form of the
 * counting sort behind emoo_sort, for callers that cannot call cudaMalloc -
 * hosts that give all device memory to their own pool allocator and refuse
 * other allocations, and loops that cannot take the device-wide
 * synchronisation cudaMalloc and cudaFree may cause.
 *
 * keys (device, n values, only the low key_bits bits used, 1 <= key_bits <=
 * 32) is read; perm (device, n values) receives the permutation: perm[i] is
 * the index in keys of the i-th smallest key, equal keys in input order. The
 * work is queued on `stream` (a cudaStream_t, null for the default stream)
 * and the call returns without waiting for it.
 *
 * Scratch is one fixed 12.25 MiB device array in the library, held by every GPU
 * that loads the library until the process exits; n above
 * EMOO_NOALLOC_SORT_MAX is rejected with EMOO_ERR_ARG. The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) with the
 * device current; make that first call before any stream capture. The
 * address is kept for the life of the process: it belongs to the device's
 * primary context, so a cudaDeviceReset (or anything else that destroys that
 * context) makes it stale, and this entry point must not be called on that
 * device afterwards. All calls
 * share the array and it keeps the last call's contents, so calls whose GPU
 * work overlaps race: order them (one stream, or events). */
int emoo_sort_permutation_noalloc(const uint32_t *keys, int64_t n, int key_bits, uint32_t *perm, void *stream);

/* ---- differentiation of the FP64 time loop ------------------------------
 * No reference counterpart. The differentiated step is the loop's step
 * without sorting and charge density (gather, push, particle boundaries,
 * current deposit, J fold, Yee update, executeBC(-1) with LightBC). Its
 * parameters are the particles' velocities at the start of the run and the
 * amplitude and phase (degrees) of every injected wave, theta = (amp_0,
 * phase_0, amp_1, phase_1, ...); the objective is the field energy
 * 0.5 V sum(E^2 + B^2) over the grid points of the cells with x index in
 * [slab_lo, slab_hi) after the run's last step (B: the current B role).
 * When a wave has a sine-series envelope (emoo_set_wave_shape), theta goes
 * on with the envelope coefficients, EMOO_NCOEF per wave: theta[2 nwaves +
 * EMOO_NCOEF w + k] = coef[k] of wave w (emoo_ad_nparams gives the length).
 * The objective is either the field energy above, or (EMOO_AD_OBJ_KINETIC)
 * the kinetic energy sum m (gamma - 1) (relativistic; 0.5 m v^2 otherwise,
 * m the species' mass_ratio) of the particles of one species (or all) whose
 * x lies in [xyz0 + slab_lo dx, xyz0 + slab_hi dx) after the last step.
 * The cell a particle is in and whether a boundary fires are held fixed (the
 * step is differentiated between such events), and so is whether a particle
 * is inside the kinetic objective's range. FP64 handles only, not the
 * electrostatic update. */
#define EMOO_AD_FORWARD 0 /* objective only */
#define EMOO_AD_TANGENT 1 /* objective and its derivative along (dtheta, dv) */
#define EMOO_AD_ADJOINT 2 /* objective and its gradient */

#define EMOO_AD_OBJ_FIELD 0   /* field energy over the slab's grid points */
#define EMOO_AD_OBJ_KINETIC 1 /* kinetic energy of the particles in the slab */

typedef struct emoo_ad_spec {
    int nsteps;           /* steps of the run, from the handle's current state */
    int checkpoint_every; /* adjoint: state kept every this many steps, segments recomputed (>= 1) */
    int slab_lo, slab_hi; /* objective slab, cell x indices [slab_lo, slab_hi) */
    int objective;        /* EMOO_AD_OBJ_FIELD or EMOO_AD_OBJ_KINETIC */
    int species;          /* EMOO_AD_OBJ_KINETIC: the species counted, -1 for all */
} emoo_ad_spec;

/* Length of theta for emoo_ad_run: 2 nwaves, plus EMOO_NCOEF nwaves when a
 * wave has a sine-series envelope. */
int emoo_ad_nparams(const emoo_handle *h);

typedef struct emoo_ad_result {
    double objective;
    double tangent;      /* EMOO_AD_TANGENT: d objective along (dtheta, dv) */
    double forward_ms;   /* device time of the run's steps */
    double recompute_ms; /* EMOO_AD_ADJOINT: re-running the segments from their checkpoints */
    double reverse_ms;   /* EMOO_AD_ADJOINT: the adjoint steps */
} emoo_ad_result;

/* Sets the amplitude and phase (degrees) of the handle's nwaves injected
 * waves (nwaves must equal the input's wave count); LightBC uses them from
 * the next boundary update. */
int emoo_set_waves(emoo_handle *h, int nwaves, const double *amp, const double *phase_deg);

/* ---- shaped injected waves ------------------------------------------------
 * No reference counterpart: LightBC (src/grid/lightBC.cpp:165-200) writes one
 * value over a whole plane, with the Gaussian envelope of
 * src/utils/evaluateGaussianPulse.cpp:7-30. A shape gives injected wave
 * `wave` (input order) a transverse Gaussian spot, an envelope made of a
 * sine series, or both; its term of the LightBC sum becomes
 *
 *   amp cos(omega (t + dt) + phase pi / 180) env(t) S(a, b)
 *   env(t)  = sum_{k=1..ncoef} coef[k-1] sin(k pi (t - t_start) / window)
 *             for t_start <= t <= t_start + window, 0 elsewhere
 *             (ncoef = 0: the reference's exp(-((t - delay) invWidth)^2))
 *   S(a, b) = exp(-((a - center[0]) / waist)^2) exp(-((b - center[1]) / waist)^2)
 *             (waist = 0: S = 1, the reference's plane wave)
 *
 * a and b are the positions of a point of the written plane along the two
 * axes other than the side's, in axis order: xyz0 + (j - 1 + h) d for grid
 * index j, with h = 1/2 along the wave's E polarisation and 0 across it
 * (where that E component, and the B component LightBC pairs with it, sit).
 * The envelope is evaluated at t, the carrier at t + dt, as the reference's
 * Gaussian. Waves of one side and polarisation whose shapes have spots must
 * share the waist and centre. shape NULL restores the plain wave. */
#define EMOO_NCOEF 16

typedef struct emoo_wave_shape {
    double waist;          /* transverse 1/e field radius (length units); 0: plane wave */
    double center[2];      /* spot centre on the two transverse axes, in axis order */
    double t_start, window;  /* envelope window [t_start, t_start + window] (time units) */
    int ncoef;             /* sine-series coefficients used, 0..EMOO_NCOEF */
    double coef[EMOO_NCOEF];
} emoo_wave_shape;

int emoo_set_wave_shape(emoo_handle *h, int wave, const emoo_wave_shape *shape);

/* ---- output files ----------------------------------------------------------
 * Field time series, replacing Hdf5IO (src/IO/hdf5io.cpp:6-72, 108-141,
 * 169-350). The reference writes per field a 4-D dataset of the physical
 * points, dims [nx][ny][nz][time], chunked one snapshot per chunk, with the
 * point coordinates as attributes x, y, z, and a /time dataset. HDF5 is not
 * available to this library, so the same data go to raw little-endian files
 * in directory `dir` (created if missing): time.f64 (one double per
 * snapshot), per field <name>.f64 (the snapshots in order, each the physical
 * points as doubles in C order [i][j][k]: the reference dataset's chunks in
 * file order) and <name>.xyz (x[nx], y[ny], z[nz], written at the first
 * snapshot: xyz0 + offset + d (i - 1), the offset d/2 along an E or J
 * component's own axis and across a B component's two others, Grid::getGridPhys
 * src/grid/grid.cpp:415-466). The first call on a directory without
 * time.f64 starts the series; later calls append. which: the reference's
 * fields_to_write (src/IO/hdf5io.hpp:14-20): 0 rho, 1 E, 2 J, 3 B, 4 all;
 * names Ex Ey Ez Bx By Bz Jx Jy Jz rho; B is (B + B_tm1) / 2 (Grid::AvgB,
 * src/grid/grid.cpp:495-506). */
#define EMOO_FIELDS_RHO 0
#define EMOO_FIELDS_E 1
#define EMOO_FIELDS_J 2
#define EMOO_FIELDS_B 3
#define EMOO_FIELDS_ALL 4
int emoo_write_fields(emoo_handle *h, const char *dir, int which);

/* Restart files (the reference parses nstep_restart, src/IO/readinfo.cpp:706-711,
 * and writes none): the whole state the loop continues from - time and step,
 * B roles, the fields the loop reads and writes, the particle store in the
 * handle's precision (with ids when tracked), the history rows - in one file.
 * emoo_read_restart restores it into a handle created from the same input and
 * options (same grid, species and precision; EMOO_ERR_STATE otherwise); wave
 * shapes and other emoo_set_* settings are configuration and are set again by
 * the caller. Continuing from a restart reproduces the uninterrupted run. */
int emoo_write_restart(emoo_handle *h, const char *path);

/* emoo_read_restart checks the whole file before it changes the handle: the
 * header must be well formed (emoo_restart_info) and must match the handle's
 * grid, species, precision, id tracking and pusher (EMOO_ERR_STATE
 * otherwise); the handle is then untouched. Only an I/O error while the
 * arrays are read leaves it changed, with an empty particle store and its
 * fields to be set again (EMOO_ERR_INPUT). */
int emoo_read_restart(emoo_handle *h, const char *path);

/* What a restart file holds, from its header. */
typedef struct emoo_restart_desc {
    int precision; /* EMOO_FP64 or EMOO_MIXED */
    int n[3];      /* physical cells per dimension */
    int nspec;
    int has_ids;
    int64_t np;
    int64_t count[EMOO_NSPEC];
    double t;
    int64_t step_index;
    int64_t nhist_rows;
} emoo_restart_desc;

/* Reads and checks the header of a restart file without a handle (host only):
 * magic and version, precision, grid sizes, 0/1 flags, non-negative species
 * counts (zero past nspec) summing to np, the optional arrays as the writer
 * stores them, and a file length equal to what the header implies.
 * EMOO_ERR_INPUT when any of these fails. */
int emoo_restart_info(const char *path, emoo_restart_desc *out);

/* Runs spec->nsteps steps from the handle's current state and leaves it at
 * the final state. dtheta (emoo_ad_nparams) and dv (3 np host doubles: vx of
 * every particle, then vy, then vz, in storage order) give the tangent
 * direction (either may be NULL: zero); grad_theta (emoo_ad_nparams) and
 * grad_v (3 np, same layout) receive the adjoint gradient (either may be
 * NULL). Both policies, both precisions (mixed-precision handles: objective
 * and adjoint, no tangent). Electrostatic runs are not differentiated
 * (EMOO_ERR_UNSUPPORTED). */
int emoo_ad_run(emoo_handle *h, const emoo_ad_spec *spec, int mode, const double *dtheta, const double *dv,
                emoo_ad_result *out, double *grad_theta, double *grad_v);

#ifdef __cplusplus
}
#endif

#endif /* EMOO_H */
