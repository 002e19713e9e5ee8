// emoopic.hpp - the reference's C++ class API for the per-timestep loop, as
// thin header-only wrappers over the C ABI in emoo.h.
//
// A driver written against the reference classes (src/main.cpp) keeps its
// structure: Input -> Domain -> Particle_Handler + pusher -> particle BCs ->
// Grid / Poisson_Solver -> field BCs -> Load -> deposit -> InitializeFields
// -> time loop. All state lives in one device handle owned by the Grid (the
// reference's Grid, Particle_Handler and BC objects all address it); the
// particle and field arrays stay on the GPU and are copied to the host only
// through the explicit accessors below.
//
// Error behaviour: every wrapper throws emoopic::Error (a std::runtime_error
// carrying the emoo status) where the reference would print and exit, abort
// on an assert, or throw its "Unable to find ... boundary" runtime_error.
#ifndef EMOOPIC_HPP
#define EMOOPIC_HPP

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "emoo.h"

typedef emoo_input_info Input_Info_t;

namespace emoopic {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &what)
        : std::runtime_error(what + ": " + emoo_strerror(s)), status(s) {}
};

inline void check(int s, const char *what) {
    if (s != EMOO_OK) throw Error(s, what);
}

// Reference units (src/globals.hpp:6-30).
constexpr double UNIT_VTH = 0.002232;

// Process-wide options of the handle the Grid creates (precision, device,
// time step). The reference fixes dt = mindx/100 in its driver.
struct Options {
    emoo_opts o;
    Options() { emoo_default_opts(&o); }
    static Options &get() {
        static Options opt;
        return opt;
    }
};

}  // namespace emoopic

// ---------------------------------------------------------------- Input
// Input::readinfo / ProcessInfo / getinfo, src/IO/input.hpp:130-144.
class Input {
   public:
    Input() { memset(&info_, 0, sizeof(info_)); }
    int readinfo(const char *inputname) {
        int rc = emoo_read_input(inputname, &info_);
        if (rc != EMOO_OK) fprintf(stderr, "%s\n", emoo_input_message());
        return rc == EMOO_OK ? 0 : 1;  // EXIT_FAILURE like the reference
    }
    int ProcessInfo() { return emoo_process_info(&info_) == EMOO_OK ? 0 : 1; }
    Input_Info_t *getinfo() { return &info_; }

   private:
    Input_Info_t info_;
};

// ---------------------------------------------------------------- Domain
// One device-resident domain (the reference's Domain, src/domain/domain.hpp:12-60,
// collapsed to a single rank).
class Domain {
   public:
    explicit Domain(Input_Info_t *info) : info_(info) {
        for (int i = 0; i < 3; i++) {
            nxyz_[i] = info->nCell[i];
            xyz0_[i] = info->xyz0[i] + info->Lxyz[i] * 0;
            Lxyz_[i] = info->Lxyz[i];
        }
        info->nparticles_domain = info->nparticles_tot;
    }
    int *getnxyz() { return nxyz_; }
    double *getxyz0() { return xyz0_; }
    double *getLxyz() { return Lxyz_; }
    double getmindx() {
        double m = Lxyz_[0] / nxyz_[0];
        for (int i = 1; i < 3; i++) m = fmin(m, Lxyz_[i] / nxyz_[i]);
        return m;
    }
    Input_Info_t *info() { return info_; }

   private:
    Input_Info_t *info_;
    int nxyz_[3];
    double xyz0_[3], Lxyz_[3];
};

// ---------------------------------------------------------------- pushers
// Pusher / Boris / Relativistic_Boris (src/pusher/pusher.hpp:6-10): on the GPU
// the pusher is a property of the handle; the classes select it.
class Pusher {
   public:
    virtual ~Pusher() {}
    virtual int relativistic() const = 0;
};
class Boris : public Pusher {
   public:
    int relativistic() const override { return 0; }
};
class Relativistic_Boris : public Pusher {
   public:
    int relativistic() const override { return 1; }
};

// ---------------------------------------------------------------- boundaries
// The reference's string registries (Part_BC_Factory,
// src/boundaries/particle_bc_factory.hpp:20-110; Field_BC_Factory,
// src/boundaries/field_bc_factory.hpp:20-87): a boundary type is declared
// under a name with a factory function (declare, or a static
// RegisterParticleBoundary / RegisterFieldBoundary object), and the names in
// input.txt are looked up there, "Unable to find particle boundary <name>"
// (or field) when absent. The built-in names are registered by the
// factories themselves: "periodic", "reflecting", "absorbing" (particles)
// and "periodic", "external" (fields).
//
// The GPU applies the boundaries inside its kernels, so a boundary object
// only says which device boundary it is (kind()); a type declared under a new
// name - a subclass of BC_P_Reflecting, say - runs as the kind it returns.
// Before the device handle is created, the input's side names are replaced
// by the kinds their objects return.
class Domain;
class Grid;

class BC_Particle {
   public:
    BC_Particle(Domain *, int dim_Index, short isRight, const std::string &t)
        : type(t), dim_Index_(dim_Index), isRight_(isRight) {}
    virtual ~BC_Particle() {}
    virtual const char *kind() const = 0;  // "periodic", "reflecting" or "absorbing"
    std::string type;

   protected:
    int dim_Index_;
    short isRight_;
};
class BC_P_Periodic : public BC_Particle {
   public:
    using BC_Particle::BC_Particle;
    const char *kind() const override { return "periodic"; }
};
class BC_P_Reflecting : public BC_Particle {
   public:
    using BC_Particle::BC_Particle;
    const char *kind() const override { return "reflecting"; }
};
class BC_P_Absorbing : public BC_Particle {  // no reference counterpart: particles leaving are removed
   public:
    using BC_Particle::BC_Particle;
    const char *kind() const override { return "absorbing"; }
};

class BC_Field {
   public:
    BC_Field(int side, Domain *, Grid *, Input_Info_t *) : side_(side) {}
    virtual ~BC_Field() {}
    virtual const char *kind() const = 0;  // "periodic" or "external"

   protected:
    int side_;  // -1 / +1 along dimension dim, as the reference numbers sides (1-based |side|)
};
class BC_F_Periodic : public BC_Field {
   public:
    using BC_Field::BC_Field;
    const char *kind() const override { return "periodic"; }
};
class BC_F_External : public BC_Field {
   public:
    using BC_Field::BC_Field;
    const char *kind() const override { return "external"; }
};

template <typename T>
BC_Particle *makeBCParticle(Domain *domain, int dim_Index, short isRight, std::string type) {
    return new T(domain, dim_Index, isRight, type);
}
template <typename T>
BC_Field *makeBCField(int side, Domain *domain, Grid *grids, Input_Info_t *info) {
    return new T(side, domain, grids, info);
}

namespace emoopic {
// writes a device kind over an input side name
inline void set_name(char *dst, const char *kind) {
    strncpy(dst, kind, EMOO_NCHAR - 1);
    dst[EMOO_NCHAR - 1] = 0;
}
}  // namespace emoopic

class Part_BC_Factory {
   public:
    typedef BC_Particle *(*Factory)(Domain *domain, int dim_Index, short isRight, std::string type);
    static Part_BC_Factory &getInstance() {
        static Part_BC_Factory f;
        return f;
    }
    // the first declaration of a name stands, as the reference's map insert
    void declare(const std::string &type, Factory factory) { registry_.insert(std::make_pair(type, factory)); }
    Factory lookup(const std::string &type) const {
        auto i = registry_.find(type);
        if (i == registry_.end()) throw std::runtime_error("Unable to find particle boundary " + type);
        return i->second;
    }
    std::vector<const std::string *> types() const {
        std::vector<const std::string *> t;
        for (const auto &kv : registry_) t.push_back(&kv.first);
        return t;
    }
    // one object per side (x-, x+, y-, y+, z-, z+); the input's names become
    // the objects' device kinds. The caller deletes the objects and the array.
    BC_Particle **constructConditions(Domain *domain, Input_Info_t *info) {
        BC_Particle **ret = new BC_Particle *[6]();
        try {
            for (int i = 0; i < 6; i++) {
                ret[i] = lookup(info->parts_bound[i])(domain, i / 2, (short)(i % 2), info->parts_bound[i]);
                emoopic::set_name(info->parts_bound[i], ret[i]->kind());
            }
        } catch (...) {
            for (int i = 0; i < 6; i++) delete ret[i];
            delete[] ret;
            throw;
        }
        return ret;
    }

   private:
    Part_BC_Factory() {
        declare("periodic", makeBCParticle<BC_P_Periodic>);
        declare("reflecting", makeBCParticle<BC_P_Reflecting>);
        declare("absorbing", makeBCParticle<BC_P_Absorbing>);
    }
    std::map<std::string, Factory> registry_;
};

struct RegisterParticleBoundary {
    RegisterParticleBoundary(const std::string &type, Part_BC_Factory::Factory factory) {
        Part_BC_Factory::getInstance().declare(type, factory);
    }
};

class Field_BC_Factory {
   public:
    typedef BC_Field *(*Factory)(int side, Domain *domain, Grid *grids, Input_Info_t *info);
    static Field_BC_Factory &getInstance() {
        static Field_BC_Factory f;
        return f;
    }
    void declare(const std::string &type, Factory factory) { registry_.insert(std::make_pair(type, factory)); }
    Factory lookup(const std::string &type) const {
        auto i = registry_.find(type);
        if (i == registry_.end()) throw std::runtime_error("Unable to find field boundary " + type);
        return i->second;
    }
    std::vector<const std::string *> types() const {
        std::vector<const std::string *> t;
        for (const auto &kv : registry_) t.push_back(&kv.first);
        return t;
    }
    // The input's field side names become their objects' device kinds (the
    // Grid does this before it creates the device handle).
    void resolve(Domain *domain, Input_Info_t *info) {
        for (int i = 0; i < 6; i++) {
            const int side = (i % 2 ? 1 : -1) * (i / 2 + 1);
            BC_Field *b = lookup(info->fields_bound[i])(side, domain, nullptr, info);
            emoopic::set_name(info->fields_bound[i], b->kind());
            delete b;
        }
    }
    // The reference wires one object per side to the grid here; on the GPU
    // the handle holds the sides, so this checks that every name resolves.
    void Construct(Domain *domain, Grid *, Input_Info_t *info) {
        Input_Info_t tmp = *info;
        resolve(domain, &tmp);
    }

   private:
    Field_BC_Factory() {
        declare("periodic", makeBCField<BC_F_Periodic>);
        declare("external", makeBCField<BC_F_External>);
    }
    std::map<std::string, Factory> registry_;
};

struct RegisterFieldBoundary {
    RegisterFieldBoundary(const std::string &type, Field_BC_Factory::Factory factory) {
        Field_BC_Factory::getInstance().declare(type, factory);
    }
};

// ---------------------------------------------------------------- Grid
// Grid (src/grid/grid.hpp:22-232): field IDs, Yee update and boundary
// exchange. Owns the device handle.
class Grid {
   public:
    Grid(Domain *domain, Input_Info_t *info) : info_(*info) {
        Field_BC_Factory::getInstance().resolve(domain, &info_);
        emoo_opts o = emoopic::Options::get().o;
        if (o.dt <= 0) o.dt = domain->getmindx() / 100.0;  // src/main.cpp:213-214
        if (o.capacity <= 0) o.capacity = info->nparticles_tot;
        emoopic::check(emoo_create(&info_, &o, &h_), "emoo_create");
    }
    virtual ~Grid() {
        if (h_) emoo_destroy(h_);
    }
    Grid(const Grid &) = delete;
    Grid &operator=(const Grid &) = delete;

    // The device handle advances by its own step (emoo_opts.dt); a dt other
    // than that step is refused rather than silently replaced.
    int evolveFields(double dt) {
        check_dt(dt, "evolveFields");
        return emoo_evolve_fields(h_, 0);
    }
    int evolveFieldsES(double dt) {
        check_dt(dt, "evolveFieldsES");
        return emoo_evolve_fields(h_, 1);
    }
    void check_dt(double dt, const char *what) {
        double hdt = 0.0;
        emoo_time(h_, nullptr, &hdt);
        if (dt != hdt) throw emoopic::Error(EMOO_ERR_ARG, std::string(what) + ": dt differs from the handle's step");
    }
    void executeBC(int sendID) { emoopic::check(emoo_execute_bc(h_, sendID), "executeBC"); }
    virtual void InitializeFields(Input_Info_t *) {
        int it[4];
        emoopic::check(emoo_init_fields(h_, it), "InitializeFields");
    }
    int getCellID(double x, double y, double z) {
        int c;
        emoopic::check(emoo_cell_id(h_, x, y, z, &c), "getCellID");
        return c;
    }
    double getStepSize(int dim) { return info_.Lxyz[dim] / info_.nCell[dim]; }
    int getnxyzTot(int *n) {
        for (int i = 0; i < 3; i++) n[i] = info_.nCell[i] + 3;
        return 0;
    }
    // getFieldPtr() in the reference hands out the host arrays; here a field
    // is copied out / in as one (n+3)^3 C-order array.
    std::vector<double> getField(int fieldID) {
        int n[3];
        getnxyzTot(n);
        std::vector<double> v((size_t)n[0] * n[1] * n[2]);
        emoopic::check(emoo_get_field(h_, fieldID, v.data()), "getField");
        return v;
    }
    void setField(int fieldID, const std::vector<double> &v) {
        emoopic::check(emoo_set_field(h_, fieldID, v.data()), "setField");
    }
    emoo_handle *handle() { return h_; }

   protected:
    Input_Info_t info_;
    emoo_handle *h_ = nullptr;
};

// Poisson_Solver (src/poisson/poisson.hpp:8-80): the Jacobi start.
class Poisson_Solver : public Grid {
   public:
    Poisson_Solver(Domain *domain, Input_Info_t *info) : Grid(domain, info) {}
    void InitializeFields(Input_Info_t *) override {
        int it[4];
        int rc = emoo_poisson_init(h_, it);
        if (rc == EMOO_ERR_NOT_CONVERGED)
            printf("WARNING: Poisson FAILED to converge (%d/%d/%d/%d iterations)\n", it[0], it[1], it[2], it[3]);
        else
            emoopic::check(rc, "Poisson_Solver::InitializeFields");
    }
};

class Particle_Compare {
   public:
    explicit Particle_Compare(Grid *) {}
};

// ---------------------------------------------------------------- particles
// Particle_Handler (src/particles/particle_handler.hpp:21-60).
class Particle_Handler {
   public:
    void setPusher(Pusher *p) { pusher_ = p; }
    void setParticleBoundaries(BC_Particle **bc) { bc_ = bc; }
    void attach(Grid *g) { grid_ = g; }

    // Load: species as consecutive index blocks by density fraction, uniform
    // positions, Maxwellian velocities with v_th = UNIT_VTH sqrt(T/m), gamma =
    // sqrt(1 - v^2), and the mean velocity removed per species for a Poisson
    // start with periodic fields (src/particles/particle_handler.cpp:34-122),
    // sampled with the library's seeded per-particle streams.
    void Load(Input_Info_t *info, Domain *domain, uint64_t seed = 12345) {
        if (!grid_) throw std::runtime_error("Particle_Handler: attach(grid) before Load");
        int64_t npart = info->nparticles_domain;
        std::vector<int64_t> count(info->nspecies, 0);
        int ispec = 0;
        double cden = info->dens_frac[0];
        for (int64_t ip = 0; ip < npart; ip++) {
            if (ip >= cden * npart) {
                ispec += 1;
                cden += info->dens_frac[ispec];
            }
            if (ispec >= info->nspecies) throw std::runtime_error("Load: density fractions do not cover nparticles");
            count[ispec]++;
        }
        bool zero_mean = strcmp(info->fields_init, "poisson") == 0;
        for (int i = 0; i < 6; i++) zero_mean = zero_mean && strcmp(info->fields_bound[i], "periodic") == 0;
        for (int s = 0; s < info->nspecies; s++) {
            emoo_gen_params g;
            memset(&g, 0, sizeof(g));
            g.seed = seed;
            g.species = s;
            g.relativistic_gamma = 1;
            double vth = UNIT_VTH_() * sqrt(info->temp[s] / info->mass_ratio[s]);
            for (int d = 0; d < 3; d++) {
                g.x0[d] = domain->getxyz0()[d];
                g.L[d] = domain->getLxyz()[d];
                g.vth[d] = vth;
            }
            int64_t n = count[s];
            if (!zero_mean) {
                emoopic::check(emoo_load_generated(grid_->handle(), &g, n), "Load");
                continue;
            }
            std::vector<double> x(n), y(n), z(n), vx(n), vy(n), vz(n), ga(n);
            emoopic::check(emoo_generate_host(&g, 0, n, x.data(), y.data(), z.data(), vx.data(), vy.data(),
                                              vz.data(), ga.data()),
                           "Load");
            for (std::vector<double> *v : {&vx, &vy, &vz}) {  // zeroAvgChargeAndVelocity_
                double m = 0.0;
                for (double a : *v) m += a;
                m /= (double)(n ? n : 1);
                for (double &a : *v) a -= m;
            }
            emoopic::check(emoo_load_particles(grid_->handle(), s, n, x.data(), y.data(), z.data(), vx.data(),
                                               vy.data(), vz.data(), ga.data(), nullptr),
                           "Load");
        }
    }
    void Push(double dt) {
        grid_->check_dt(dt, "Push");
        emoopic::check(emoo_push(grid_->handle()), "Push");
    }
    long nParticles() {
        int64_t n = 0;
        emoo_num_particles(grid_->handle(), -1, &n);
        return (long)n;
    }
    void SortParticles(const Particle_Compare &) { emoopic::check(emoo_sort(grid_->handle()), "SortParticles"); }
    void InterpolateEB(Grid *) { emoopic::check(emoo_interpolate(grid_->handle()), "InterpolateEB"); }
    void depositRhoJ(Grid *, bool depositRho, Domain *, Input_Info_t *) {
        emoopic::check(emoo_deposit(grid_->handle(), depositRho ? 1 : 0), "depositRhoJ");
    }
    void executeParticleBoundaryConditions() {
        emoopic::check(emoo_apply_particle_bc(grid_->handle(), last_crossings_), "executeParticleBoundaryConditions");
    }
    void clearGhosts() {}  // particles leaving through absorbing sides are removed by the boundary call
    const int64_t *crossings() const { return last_crossings_; }

   private:
    static double UNIT_VTH_() { return emoopic::UNIT_VTH; }
    Pusher *pusher_ = nullptr;
    BC_Particle **bc_ = nullptr;
    Grid *grid_ = nullptr;
    int64_t last_crossings_[6] = {0, 0, 0, 0, 0, 0};
};

// ---------------------------------------------------------------- history
// OutputBoxQuantities (src/IO/output.hpp:12-27): history.dat every 10 steps.
class OutputBoxQuantities {
   public:
    OutputBoxQuantities(const char *fname, Grid *grid, Particle_Handler *, Input_Info_t *)
        : grid_(grid), fname_(fname) {}
    void output(double t, long i) {
        if (first_) {
            first_ = false;
            FILE *fp = fopen(fname_.c_str(), "w");
            if (fp) {
                fprintf(fp, "[1] time [2] part mom x [3] part mom y [4] part mom z [5] part Energy [6] B Energy "
                            "[7] E Energy [8] Total E\n");
                fclose(fp);
            }
        }
        if (i < next_) return;
        next_ += 10;
        double r[8];
        emoopic::check(emoo_history(grid_->handle(), r), "history");
        FILE *fp = fopen(fname_.c_str(), "a");
        if (!fp) return;
        fprintf(fp, "%e %.15e %.15e %.15e %.15e %.15e %.15e %.15e\n", t, r[1], r[2], r[3], r[4], r[5], r[6], r[7]);
        fclose(fp);
    }

   private:
    Grid *grid_;
    std::string fname_;
    bool first_ = true;
    long next_ = 0;
};

#endif
