// Host-only checks of the reference class mirror in include/emoopic.hpp: the
// string registries of the boundary factories. Built and run by
// tests/test_cpp_mirror.py; exits non-zero with a message on the first
// failed check. No GPU work.
#include <cstdio>
#include <cstring>
#include <string>

#include "emoopic.hpp"

namespace {

int failures = 0;

void expect(bool ok, const char *what) {
    if (!ok) {
        fprintf(stderr, "FAILED: %s\n", what);
        failures++;
    }
}

// a user boundary type declared under a new name, as a reference user would
// register one (RegisterParticleBoundary / RegisterFieldBoundary statics)
class BC_P_Wall : public BC_P_Reflecting {
   public:
    using BC_P_Reflecting::BC_P_Reflecting;
};
class BC_F_Laser : public BC_F_External {
   public:
    using BC_F_External::BC_F_External;
};
RegisterParticleBoundary reg_wall("wall", makeBCParticle<BC_P_Wall>);
RegisterFieldBoundary reg_laser("laser", makeBCField<BC_F_Laser>);

void set(char *dst, const char *s) { strncpy(dst, s, EMOO_NCHAR - 1); }

}  // namespace

int main() {
    Input_Info_t info;
    memset(&info, 0, sizeof(info));
    for (int d = 0; d < 3; d++) {
        info.nCell[d] = 4;
        info.Lxyz[d] = 4.0;
    }
    const char *pb[6] = {"wall", "wall", "periodic", "periodic", "absorbing", "reflecting"};
    const char *fb[6] = {"laser", "external", "periodic", "periodic", "periodic", "periodic"};
    for (int i = 0; i < 6; i++) {
        set(info.parts_bound[i], pb[i]);
        set(info.fields_bound[i], fb[i]);
    }
    Domain domain(&info);

    BC_Particle **bc = Part_BC_Factory::getInstance().constructConditions(&domain, &info);
    expect(bc[0]->type == "wall" && std::string(bc[0]->kind()) == "reflecting", "registered particle type");
    expect(std::string(info.parts_bound[0]) == "reflecting", "input side name becomes the device kind");
    expect(std::string(info.parts_bound[4]) == "absorbing", "built-in absorbing kind");
    for (int i = 0; i < 6; i++) delete bc[i];
    delete[] bc;

    bool found = false;
    for (const std::string *t : Part_BC_Factory::getInstance().types()) found = found || *t == "wall";
    expect(found, "types() lists a registered name");

    // the first declaration of a name stands
    Part_BC_Factory::getInstance().declare("periodic", makeBCParticle<BC_P_Reflecting>);
    set(info.parts_bound[2], "periodic");
    bc = Part_BC_Factory::getInstance().constructConditions(&domain, &info);
    expect(std::string(bc[2]->kind()) == "periodic", "a later declaration does not replace a name");
    for (int i = 0; i < 6; i++) delete bc[i];
    delete[] bc;

    set(info.parts_bound[3], "sticky");
    try {
        Part_BC_Factory::getInstance().constructConditions(&domain, &info);
        expect(false, "unknown particle boundary throws");
    } catch (const std::runtime_error &e) {
        expect(std::string(e.what()) == "Unable to find particle boundary sticky", "particle error text");
    }

    Field_BC_Factory::getInstance().Construct(&domain, nullptr, &info);
    expect(std::string(info.fields_bound[0]) == "laser", "Construct leaves the input as it is");
    Input_Info_t resolved = info;
    Field_BC_Factory::getInstance().resolve(&domain, &resolved);
    expect(std::string(resolved.fields_bound[0]) == "external", "registered field type resolves to its kind");
    set(info.fields_bound[5], "mirror");
    try {
        Field_BC_Factory::getInstance().Construct(&domain, nullptr, &info);
        expect(false, "unknown field boundary throws");
    } catch (const std::runtime_error &e) {
        expect(std::string(e.what()) == "Unable to find field boundary mirror", "field error text");
    }
    if (failures == 0) printf("ok\n");
    return failures ? 1 : 0;
}
