// Test-side harness around the compiled reference serial build.
//
// This file is test infrastructure: it links against the reference's own
// objects (built in place by oracle/ref/Makefile) and exposes a flat C ABI so
// the golden-vector generator can drive the reference classes with seeded,
// identical inputs. It never ships with the product.
//
// The step order replicates the reference driver loop, src/main.cpp:221-287:
//   sort (every nstep_sort) -> history (every 10) -> Push -> particle BCs
//   (6 sides in order) -> clearGhosts -> depositRhoJ -> executeBC(-2)
//   -> evolveFields / evolveFieldsES -> executeBC(-1) -> InterpolateEB
//   -> time_phys += dt.
// Initialisation replicates src/main.cpp:155-179 (deposit + fold + Poisson
// solve, or constant fields) with time_phys = dt_phys = 0 during the field
// initialisation, exactly as the reference driver leaves them there.
#define MAIN_CPP
#include "globals.hpp"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <unistd.h>
#include "IO/input.hpp"
#include "IO/output.hpp"
#include "domain/domain.hpp"
#include "grid/grid.hpp"
#include "poisson/poisson.hpp"
#include "particles/particle.hpp"
#include "particles/particle_handler.hpp"
#include "particles/particle_utils.hpp"
#include "particles/interpolate.hpp"
#include "pusher/boris.hpp"
#include "pusher/relativisticBoris.hpp"
#include "boundaries/particle_bc_factory.hpp"
#include "boundaries/field_bc_factory.hpp"

namespace {

struct RefCtx {
    Input_Info_t info;
    Domain *domain = nullptr;
    Grid *grid = nullptr;
    bool poisson = false;
    Particle_Handler *ph = nullptr;
    Pusher *pusher = nullptr;
    BC_Particle **pbc = nullptr;
    Particle_Compare *cmp = nullptr;
    OutputBoxQuantities *box = nullptr;
    std::string boxfile;
    long boxsize = 0;
    double dt = 0.0, t0 = 0.0;
    int nfields = 16;
    long npoints = 0;
};

long file_size(const std::string &f) {
    FILE *fp = fopen(f.c_str(), "r");
    if (!fp) return 0;
    fseek(fp, 0, SEEK_END);
    long s = ftell(fp);
    fclose(fp);
    return s;
}

// Parses the last line of a history file written by OutputBoxQuantities.
int read_last_history(const std::string &f, double *out8) {
    FILE *fp = fopen(f.c_str(), "r");
    if (!fp) return -1;
    char line[1024], last[1024];
    last[0] = 0;
    while (fgets(line, sizeof line, fp)) {
        if (line[0] != '[') strcpy(last, line);
    }
    fclose(fp);
    int n = sscanf(last, "%lf %lf %lf %lf %lf %lf %lf %lf", &out8[0], &out8[1], &out8[2],
                   &out8[3], &out8[4], &out8[5], &out8[6], &out8[7]);
    return n == 8 ? 0 : -2;
}

}  // namespace

extern "C" {

int refh_sizeof_input_info(void) { return (int)sizeof(Input_Info_t); }

// Creates the reference objects from a filled Input_Info_t (same struct the
// reference parser fills, src/IO/input.hpp:15-126). All field slots are zeroed
// after construction (the reference allocates them uninitialised).
void *refh_create(const Input_Info_t *in, double dt, double t0, const char *tmpdir) {
    rank_MPI = 0;
    size_MPI = 1;
    debug = 0;
    time_phys = 0.0;
    dt_phys = 0.0;
    RefCtx *c = new RefCtx();
    c->info = *in;
    c->info.nProc[0] = c->info.nProc[1] = c->info.nProc[2] = 1;
    c->dt = dt;
    c->t0 = t0;
    c->domain = new Domain(&c->info);
    if (c->info.relativity == 0)
        c->pusher = new Boris();
    else
        c->pusher = new Relativistic_Boris();
    c->ph = new Particle_Handler();
    c->ph->setPusher(c->pusher);
    c->pbc = Part_BC_Factory::getInstance().constructConditions(c->domain, &c->info);
    c->ph->setParticleBoundaries(c->pbc);
    c->poisson = (c->info.restart == 0 && strcmp(c->info.fields_init, "poisson") == 0);
    if (c->poisson) {
        c->grid = new Poisson_Solver(c->domain, &c->info);
        c->nfields = 21;
    } else {
        c->grid = new Grid(c->domain->getnxyz(), 1, c->domain->getxyz0(), c->domain->getLxyz());
        c->nfields = 16;
    }
    Field_BC_Factory::getInstance().Construct(c->domain, c->grid, &c->info);
    int tot[3];
    c->grid->getnxyzTot(tot);
    c->npoints = (long)tot[0] * tot[1] * tot[2];
    double ****fp = c->grid->getFieldPtr();
    for (int id = 0; id < c->nfields; id++) memset(&fp[id][0][0][0], 0, sizeof(double) * c->npoints);
    c->cmp = new Particle_Compare(c->grid);
    char name[512];
    snprintf(name, sizeof name, "%s/refh_history_%d_%p.dat", tmpdir ? tmpdir : "/tmp", (int)getpid(),
             (void *)c);
    c->boxfile = name;
    unlink(name);
    c->box = new OutputBoxQuantities(c->boxfile.c_str(), c->grid, c->ph, &c->info);
    return c;
}

void refh_destroy(void *h) {
    RefCtx *c = (RefCtx *)h;
    unlink(c->boxfile.c_str());
    // OutputBoxQuantities declares a destructor it never defines
    // (src/IO/output.hpp:14); the reference driver never deletes it either.
    delete c->cmp;
    c->grid->freeBoundaries();
    delete c->grid;
    delete[] c->pbc;
    delete c->ph;
    delete c->pusher;
    delete c->domain;
    delete c;
}

long refh_npoints(void *h) { return ((RefCtx *)h)->npoints; }

// Appends particles (species index `type`) with charge, mass and test flag
// taken from the species tables of the Input_Info_t.
int refh_add_particles(void *h, long n, const double *x, const double *y, const double *z,
                       const double *vx, const double *vy, const double *vz, const double *gamma,
                       const int *type, const long *id) {
    RefCtx *c = (RefCtx *)h;
    std::vector<Particle> *parts = c->ph->getParticleVector();
    for (long i = 0; i < n; i++) {
        Particle p = new_particle();
        int s = type[i];
        p.type = s;
        p.q = c->info.charge_ratio[s];
        p.m = c->info.mass_ratio[s];
        p.isTestParticle = c->info.isTestParticle[s];
        p.x[0] = x[i];
        p.x[1] = y[i];
        p.x[2] = z[i];
        p.v[0] = vx[i];
        p.v[1] = vy[i];
        p.v[2] = vz[i];
        p.gamma = gamma ? gamma[i] : 0.0;
        p.my_id = id ? id[i] : i;
        p.initRank = 0;
        parts->push_back(p);
    }
    c->ph->incrementNParticles((int)n);
    return 0;
}

long refh_num_particles(void *h) { return (long)((RefCtx *)h)->ph->getParticleVector()->size(); }

int refh_get_particles(void *h, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                       double *gamma, int *type, long *id) {
    RefCtx *c = (RefCtx *)h;
    std::vector<Particle> &v = *c->ph->getParticleVector();
    for (size_t i = 0; i < v.size(); i++) {
        x[i] = v[i].x[0];
        y[i] = v[i].x[1];
        z[i] = v[i].x[2];
        vx[i] = v[i].v[0];
        vy[i] = v[i].v[1];
        vz[i] = v[i].v[2];
        gamma[i] = v[i].gamma;
        type[i] = v[i].type;
        id[i] = v[i].my_id;
    }
    return 0;
}

int refh_get_particle_fields(void *h, double *e1, double *e2, double *e3, double *b1, double *b2,
                             double *b3) {
    RefCtx *c = (RefCtx *)h;
    std::vector<Particle> &v = *c->ph->getParticleVector();
    for (size_t i = 0; i < v.size(); i++) {
        e1[i] = v[i].field.e1;
        e2[i] = v[i].field.e2;
        e3[i] = v[i].field.e3;
        b1[i] = v[i].field.b1;
        b2[i] = v[i].field.b2;
        b3[i] = v[i].field.b3;
    }
    return 0;
}

int refh_get_field(void *h, int id, double *out) {
    RefCtx *c = (RefCtx *)h;
    if (id < 0 || id >= c->nfields) return -1;
    memcpy(out, &c->grid->getFieldPtr()[id][0][0][0], sizeof(double) * c->npoints);
    return 0;
}

int refh_set_field(void *h, int id, const double *in) {
    RefCtx *c = (RefCtx *)h;
    if (id < 0 || id >= c->nfields) return -1;
    memcpy(&c->grid->getFieldPtr()[id][0][0][0], in, sizeof(double) * c->npoints);
    return 0;
}

int refh_cell_id(void *h, double x, double y, double z) { return ((RefCtx *)h)->grid->getCellID(x, y, z); }

// src/main.cpp:159-179 (time_phys and dt_phys are still zero at this point
// of the reference driver), then time_phys = t0 and dt_phys = dt.
int refh_init_fields(void *h) {
    RefCtx *c = (RefCtx *)h;
    time_phys = 0.0;
    dt_phys = 0.0;
    if (c->poisson) {
        c->ph->depositRhoJ(c->grid, true, c->domain, &c->info);
        c->grid->executeBC(-2);
    }
    c->grid->InitializeFields(&c->info);
    c->ph->InterpolateEB(c->grid);
    time_phys = c->t0;
    dt_phys = c->dt;
    return 0;
}

// Field initialisation alone (no deposit), for tests that inject rho / J.
int refh_initialize_fields_only(void *h) {
    RefCtx *c = (RefCtx *)h;
    time_phys = 0.0;
    dt_phys = 0.0;
    c->grid->InitializeFields(&c->info);
    time_phys = c->t0;
    dt_phys = c->dt;
    return 0;
}

void refh_set_time(void *h, double t, double dt) {
    (void)h;
    time_phys = t;
    dt_phys = dt;
}

int refh_sort(void *h) {
    RefCtx *c = (RefCtx *)h;
    c->ph->SortParticles(*c->cmp);
    return 0;
}

int refh_push(void *h) {
    RefCtx *c = (RefCtx *)h;
    c->ph->Push(c->dt);
    return 0;
}

// Particle boundaries, src/particles/particle_handler.cpp:287-295, with the
// per-side crossing count measured around each side's pass: the number of
// ghost copies a periodic side appends, or the number of live particles a
// reflecting side folds back.
int refh_particle_bc(void *h, long *counts6) {
    RefCtx *c = (RefCtx *)h;
    std::vector<Particle> *parts = c->ph->getParticleVector();
    double *x0 = c->domain->getxyz0();
    double *L = c->domain->getLxyz();
    for (int s = 0; s < 6; s++) {
        int d = s / 2;
        bool right = (s % 2) == 1;
        size_t before = parts->size();
        long nref = 0;
        bool reflecting = strcmp(c->info.parts_bound[s], "reflecting") == 0;
        if (reflecting) {
            double xmin = x0[d], xmax = x0[d] + L[d];
            for (size_t i = 0; i < parts->size(); i++) {
                const Particle &p = (*parts)[i];
                if (p.isGhost) continue;
                if (right && p.x[d] > xmax) nref++;
                if (!right && p.x[d] < xmin) nref++;
            }
        }
        int inc = c->pbc[s]->computeParticleBCs(parts);
        c->ph->incrementNParticles(inc);
        counts6[s] = reflecting ? nref : (long)(parts->size() - before);
    }
    return 0;
}

int refh_clear_ghosts(void *h) {
    ((RefCtx *)h)->ph->clearGhosts();
    return 0;
}

int refh_deposit(void *h, int with_rho) {
    RefCtx *c = (RefCtx *)h;
    c->ph->depositRhoJ(c->grid, with_rho != 0, c->domain, &c->info);
    return 0;
}

int refh_execute_bc(void *h, int send_id) {
    ((RefCtx *)h)->grid->executeBC(send_id);
    return 0;
}

int refh_evolve(void *h, int electrostatic) {
    RefCtx *c = (RefCtx *)h;
    if (electrostatic)
        c->grid->evolveFieldsES(c->dt);
    else
        c->grid->evolveFields(c->dt);
    return 0;
}

int refh_interpolate(void *h) {
    RefCtx *c = (RefCtx *)h;
    c->ph->InterpolateEB(c->grid);
    return 0;
}

// One pass of the driver loop body. hist8 receives the history row when the
// reference writes one this step (hist_written = 1).
int refh_step(void *h, int ti, long *counts6, double *hist8, int *hist_written) {
    RefCtx *c = (RefCtx *)h;
    if (c->info.nstep_sort > 0 && ti % c->info.nstep_sort == 0) c->ph->SortParticles(*c->cmp);
    c->box->output(time_phys, ti);
    long sz = file_size(c->boxfile);
    *hist_written = 0;
    if (sz != c->boxsize) {
        c->boxsize = sz;
        if (read_last_history(c->boxfile, hist8) == 0) *hist_written = 1;
    }
    c->ph->Push(dt_phys);
    refh_particle_bc(h, counts6);
    c->ph->clearGhosts();
    c->ph->depositRhoJ(c->grid, true, c->domain, &c->info);
    c->grid->executeBC(-2);
    if (c->info.electrostatic == 1)
        c->grid->evolveFieldsES(dt_phys);
    else
        c->grid->evolveFields(dt_phys);
    c->grid->executeBC(-1);
    c->ph->InterpolateEB(c->grid);
    time_phys += dt_phys;
    return 0;
}

double refh_time(void) { return time_phys; }

// Runs a bare pusher (src/pusher/boris.cpp:12-111 or
// src/pusher/relativisticBoris.cpp:28-143) on a single particle.
// state = {x, y, z, vx, vy, vz, gamma, q, m}; field = {e1, e2, e3, b1, b2, b3}.
int refh_pusher_steps(int relativistic, double *state, const double *field, double dt, long nsteps) {
    Pusher *pu = relativistic ? (Pusher *)new Relativistic_Boris() : (Pusher *)new Boris();
    Particle p = new_particle();
    for (int i = 0; i < 3; i++) {
        p.x[i] = state[i];
        p.v[i] = state[3 + i];
    }
    p.gamma = state[6];
    p.q = state[7];
    p.m = state[8];
    Field_part f;
    f.e1 = field[0];
    f.e2 = field[1];
    f.e3 = field[2];
    f.b1 = field[3];
    f.b2 = field[4];
    f.b3 = field[5];
    for (long s = 0; s < nsteps; s++) pu->Step(&p, &f, dt);
    for (int i = 0; i < 3; i++) {
        state[i] = p.x[i];
        state[3 + i] = p.v[i];
    }
    state[6] = p.gamma;
    delete pu;
    return 0;
}

// One history row (src/IO/output.cpp:52-123) for the current state.
int refh_history(void *h, double t, double *out8) {
    RefCtx *c = (RefCtx *)h;
    std::string f = c->boxfile + ".once";
    unlink(f.c_str());
    OutputBoxQuantities *b = new OutputBoxQuantities(f.c_str(), c->grid, c->ph, &c->info);
    b->output(t, 0);
    (void)b;  // not deletable, see refh_destroy
    int rc = read_last_history(f, out8);
    unlink(f.c_str());
    return rc;
}

}  // extern "C"
