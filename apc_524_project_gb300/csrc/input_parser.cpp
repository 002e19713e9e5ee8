// input_parser.cpp - the reference's input.txt format (libconfig syntax) read
// into emoo_input_info, and the reference's input post-processing.
//
// emoo_read_input follows Input::readinfo (src/IO/readinfo.cpp:18-733): the
// same setting paths, the same defaults and the same required settings. Where
// the reference would abort (it catches a few SettingNotFoundException by
// pointer, so a missing `relativity`, `electrostatic` or `output_pCount`
// escapes the handler and terminates the program) this returns
// EMOO_ERR_INPUT with a message instead. emoo_process_info follows
// Input::ProcessInfo (src/IO/check.cpp:12-147).
//
// The parser covers the libconfig grammar the format uses: groups `{}`,
// arrays `[]`, lists `()`, integers (decimal, hex, 64-bit `L`), floats,
// booleans, strings (adjacent literals concatenate), `=` or `:`, optional `;`
// or `,` terminators, and `#`, `//`, `/* */` comments.
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <string>
#include <vector>

#include "emoo.h"

namespace {

struct Value {
    enum Type { None, Int, Int64, Float, Bool, String, Array, List, Group } type = None;
    long long i = 0;
    double f = 0.0;
    bool b = false;
    std::string s;
    std::vector<Value> elems;
    std::vector<std::pair<std::string, Value>> members;

    const Value *member(const std::string &name) const {
        for (const auto &m : members)
            if (m.first == name) return &m.second;
        return nullptr;
    }
    bool is_number() const { return type == Int || type == Int64 || type == Float; }
    bool is_aggregate() const { return type == Array || type == List; }
    int length() const { return is_aggregate() ? (int)elems.size() : (type == Group ? (int)members.size() : 0); }
    double as_double() const { return type == Float ? f : (double)i; }
    long long as_int() const { return type == Float ? (long long)f : i; }
};

struct Parser {
    const char *p;
    const char *end;
    int line = 1;
    std::string err;

    void skip() {
        for (;;) {
            while (p < end && isspace((unsigned char)*p)) {
                if (*p == '\n') line++;
                p++;
            }
            if (p < end && *p == '#') {
                while (p < end && *p != '\n') p++;
                continue;
            }
            if (p + 1 < end && p[0] == '/' && p[1] == '/') {
                while (p < end && *p != '\n') p++;
                continue;
            }
            if (p + 1 < end && p[0] == '/' && p[1] == '*') {
                p += 2;
                while (p + 1 < end && !(p[0] == '*' && p[1] == '/')) {
                    if (*p == '\n') line++;
                    p++;
                }
                p = p + 2 <= end ? p + 2 : end;
                continue;
            }
            break;
        }
    }

    bool fail(const char *m) {
        if (err.empty()) err = std::string(m) + " at line " + std::to_string(line);
        return false;
    }

    bool name(std::string &out) {
        skip();
        if (p >= end || !(isalpha((unsigned char)*p) || *p == '*')) return fail("expected a setting name");
        const char *s = p;
        while (p < end && (isalnum((unsigned char)*p) || *p == '_' || *p == '-' || *p == '*')) p++;
        out.assign(s, p);
        return true;
    }

    bool string_lit(std::string &out) {
        out.clear();
        bool any = false;
        for (;;) {
            skip();
            if (p >= end || *p != '"') break;
            any = true;
            p++;
            while (p < end && *p != '"') {
                if (*p == '\\' && p + 1 < end) {
                    p++;
                    char c = *p;
                    out.push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c == 'r' ? '\r' : c == 'f' ? '\f' : c);
                } else {
                    if (*p == '\n') line++;
                    out.push_back(*p);
                }
                p++;
            }
            if (p >= end) return fail("unterminated string");
            p++;
        }
        return any ? true : fail("expected a string");
    }

    bool scalar(Value &v) {
        skip();
        if (p >= end) return fail("unexpected end of input");
        if (*p == '"') {
            v.type = Value::String;
            return string_lit(v.s);
        }
        if (isalpha((unsigned char)*p)) {
            const char *s = p;
            while (p < end && isalpha((unsigned char)*p)) p++;
            std::string w(s, p);
            for (auto &c : w) c = (char)tolower((unsigned char)c);
            if (w == "true" || w == "false") {
                v.type = Value::Bool;
                v.b = w == "true";
                v.i = v.b;
                return true;
            }
            return fail("unknown word");
        }
        const char *s = p;
        if (p + 1 < end && p[0] == '0' && (p[1] == 'x' || p[1] == 'X')) {
            // libconfig's hex token takes no sign; without the L suffix it is a
            // 32-bit int (strtoul truncated), with it a 64-bit one
            p += 2;
            while (p < end && isxdigit((unsigned char)*p)) p++;
            std::string t(s, p);
            const unsigned long long u = strtoull(t.c_str(), nullptr, 16);
            if (p < end && *p == 'L') {
                p++;
                if (p < end && *p == 'L') p++;
                v.type = Value::Int64;
                v.i = (long long)u;
            } else {
                v.type = Value::Int;
                v.i = (int32_t)(uint32_t)(unsigned long)strtoul(t.c_str(), nullptr, 16);
            }
            return true;
        }
        if (*p == '+' || *p == '-') p++;
        {
            bool flt = false;
            while (p < end && (isdigit((unsigned char)*p) || *p == '.' || *p == 'e' || *p == 'E' ||
                               ((*p == '+' || *p == '-') && (p[-1] == 'e' || p[-1] == 'E')))) {
                if (*p == '.' || *p == 'e' || *p == 'E') flt = true;
                p++;
            }
            std::string t(s, p);
            if (t.empty() || t == "+" || t == "-") return fail("expected a value");
            if (flt) {
                v.type = Value::Float;
                v.f = strtod(t.c_str(), nullptr);
            } else if (p < end && *p == 'L') {
                // 64-bit integer token (libconfig: atoll)
                p++;
                if (p < end && *p == 'L') p++;
                v.type = Value::Int64;
                v.i = strtoll(t.c_str(), nullptr, 10);
            } else {
                // plain integer token: libconfig reads it with atoi, a 32-bit
                // int (larger values wrap; they are not promoted to 64 bits)
                v.type = Value::Int;
                v.i = (int32_t)(uint32_t)(unsigned long)strtol(t.c_str(), nullptr, 10);
            }
        }
        return true;
    }

    bool value(Value &v) {
        skip();
        if (p >= end) return fail("unexpected end of input");
        char c = *p;
        if (c == '{') {
            p++;
            v.type = Value::Group;
            return settings(v, '}');
        }
        if (c == '[' || c == '(') {
            char close = c == '[' ? ']' : ')';
            v.type = c == '[' ? Value::Array : Value::List;
            p++;
            skip();
            if (p < end && *p == close) {
                p++;
                return true;
            }
            for (;;) {
                Value e;
                if (!(c == '[' ? scalar(e) : value(e))) return false;
                // an array's elements all take the type of its first element
                // (libconfig's parser refuses anything else); lists mix types
                if (c == '[' && !v.elems.empty() && e.type != v.elems[0].type)
                    return fail("mismatched element type in array");
                v.elems.push_back(e);
                skip();
                if (p < end && *p == ',') {
                    p++;
                    continue;
                }
                if (p < end && *p == close) {
                    p++;
                    return true;
                }
                return fail("expected ',' or a closing bracket");
            }
        }
        return scalar(v);
    }

    bool settings(Value &grp, char close) {
        for (;;) {
            skip();
            if (p >= end) {
                if (close == 0) return true;
                return fail("unterminated group");
            }
            if (*p == close) {
                p++;
                return true;
            }
            std::string nm;
            if (!name(nm)) return false;
            skip();
            if (p < end && (*p == '=' || *p == ':')) p++;
            else return fail("expected '=' or ':'");
            Value v;
            if (!value(v)) return false;
            skip();
            if (p < end && (*p == ';' || *p == ',')) p++;
            grp.members.emplace_back(nm, v);
        }
    }
};

struct Reader {
    Value root;
    std::string msg;

    const Value *lookup(const char *path) const {
        const Value *v = &root;
        std::string s(path);
        size_t a = 0;
        while (v && a <= s.size()) {
            size_t b = s.find('.', a);
            std::string part = s.substr(a, b == std::string::npos ? std::string::npos : b - a);
            v = v->type == Value::Group ? v->member(part) : nullptr;
            if (b == std::string::npos) break;
            a = b + 1;
        }
        return v;
    }
};

void set_str(char *dst, const std::string &s) {
    strncpy(dst, s.c_str(), EMOO_NCHAR - 1);
    dst[EMOO_NCHAR - 1] = 0;
}

// Reads a per-species array of length nspecies (or a scalar when nspecies is 1).
template <typename T>
int species_array(const Reader &R, const char *path, int nspec, T *out, const char *what, bool required,
                  std::string &msg) {
    const Value *v = R.lookup(path);
    if (!v) {
        if (required) {
            msg = std::string("Error: ") + what + " not set in input file";
            return EMOO_ERR_INPUT;
        }
        return 1;  // not found, caller applies its default
    }
    if (v->is_aggregate()) {
        if (v->length() != nspec) {
            msg = std::string("Error: length of ") + what + " does not match nspecies!";
            return EMOO_ERR_INPUT;
        }
        for (int i = 0; i < nspec; i++) out[i] = (T)(std::is_integral<T>::value ? (double)v->elems[i].as_int()
                                                                              : v->elems[i].as_double());
        return EMOO_OK;
    }
    if (nspec == 1 && v->is_number()) {
        out[0] = (T)(std::is_integral<T>::value ? (double)v->as_int() : v->as_double());
        return EMOO_OK;
    }
    msg = std::string("Error: length of ") + what + " does not match nspecies!";
    return EMOO_ERR_INPUT;
}

int wave_array(const Reader &R, const char *path, int nw, double *out, const char *what, std::string &msg) {
    const Value *v = R.lookup(path);
    if (!v) {
        msg = std::string("Error: ") + what + " not set in input file";
        return EMOO_ERR_INPUT;
    }
    if (v->length() != nw) {
        msg = std::string("Error: length of ") + what + " does not match nwaves!";
        return EMOO_ERR_INPUT;
    }
    for (int i = 0; i < nw; i++) out[i] = v->elems[i].as_double();
    return EMOO_OK;
}

thread_local std::string g_last_message;

int read_info(const Reader &R, emoo_input_info *in) {
    std::string &msg = g_last_message;
    // domain (src/IO/readinfo.cpp:42-107)
    const Value *v = R.lookup("domain.nCell");
    if (!v) {
        msg = "Error: nCell not set in input file!";
        return EMOO_ERR_INPUT;
    }
    for (int i = 0; i < 3; i++) in->nCell[i] = (int)(v->length() == 3 ? v->elems[i].as_int()
                                                                      : (v->is_aggregate() ? v->elems[0].as_int() : v->as_int()));
    if ((v = R.lookup("domain.xyz0")))
        for (int i = 0; i < 3; i++) in->xyz0[i] = v->length() == 3 ? v->elems[i].as_double()
                                                                  : (v->is_aggregate() ? v->elems[0].as_double() : v->as_double());
    v = R.lookup("domain.Lxyz");
    if (!v) {
        msg = "Error: Lxyz not set in input file!";
        return EMOO_ERR_INPUT;
    }
    for (int i = 0; i < 3; i++) in->Lxyz[i] = v->length() == 3 ? v->elems[i].as_double()
                                                              : (v->is_aggregate() ? v->elems[0].as_double() : v->as_double());
    // serial build: one domain (src/IO/readinfo.cpp:142-145)
    in->nProc[0] = in->nProc[1] = in->nProc[2] = 1;
    // runtime (:147-206)
    if (!(v = R.lookup("runtime.nTimesteps"))) {
        msg = "Error: nTimesteps not set in input file";
        return EMOO_ERR_INPUT;
    }
    in->nt = (int)v->as_int();
    in->t0 = (v = R.lookup("runtime.startTime")) ? v->as_double() : 0.0;
    in->dens_phys = (v = R.lookup("initialization.particles.dens_phys")) ? v->as_double() : 0.0;
    in->debug = (v = R.lookup("runtime.debug")) ? (int)v->as_int() : 0;
    in->nstep_sort = (v = R.lookup("runtime.nstep_sort")) ? (int)v->as_int() : 100;
    int restart = (v = R.lookup("initialization.restart")) ? (int)v->as_int() : 0;
    in->restart = restart;
    // particles (:209-420)
    if (!(v = R.lookup("initialization.particles.relativity"))) {
        msg = "Error: relativity not set in input file (the reference terminates here)";
        return EMOO_ERR_INPUT;
    }
    in->relativity = (int)v->as_int();
    if (!(v = R.lookup("initialization.particles.nspecies"))) {
        msg = "Error: nSpecies not set in input file";
        return EMOO_ERR_INPUT;
    }
    int nspec = (int)v->as_int();
    in->nspecies = nspec;
    if (nspec < 1) {
        msg = "Error: no species in simulation ...";
        return EMOO_ERR_INPUT;
    }
    if (nspec > EMOO_NSPEC) {
        msg = "Error: More species are specified than NSPEC!";
        return EMOO_ERR_INPUT;
    }
    int rc;
    if ((rc = species_array(R, "initialization.particles.mass_ratio", nspec, in->mass_ratio, "mass_ratio", true, msg)) < 0) return rc;
    if ((rc = species_array(R, "initialization.particles.charge_ratio", nspec, in->charge_ratio, "charge_ratio", true, msg)) < 0) return rc;
    if ((rc = species_array(R, "initialization.particles.temperature", nspec, in->temp, "temperature", true, msg)) < 0) return rc;
    rc = species_array(R, "initialization.particles.dens_frac", nspec, in->dens_frac, "dens_frac", false, msg);
    if (rc < 0) return rc;
    if (rc == 1) {
        if (nspec == 1) in->dens_frac[0] = 1;
        else {
            msg = "Error: dens_frac not set in input file";
            return EMOO_ERR_INPUT;
        }
    }
    rc = species_array(R, "initialization.particles.isTestParticle", nspec, in->isTestParticle, "isTestParticle", false, msg);
    if (rc < 0) return rc;
    if (rc == 1)
        for (int i = 0; i < nspec; i++) in->isTestParticle[i] = 0;
    if (!(v = R.lookup("initialization.particles.nParticles_tot"))) {
        msg = "Error: nParticles_tot not set in input file";
        return EMOO_ERR_INPUT;
    }
    if (v->type == Value::Float) in->nparticles_tot = (int64_t)v->f;
    else in->nparticles_tot = v->i;
    if (v->type == Value::Int && in->nparticles_tot < 0) {
        msg = "Error: integer overflow...";
        return EMOO_ERR_INPUT;
    }
    if ((v = R.lookup("boundary.particles.conditions"))) {
        if (v->type != Value::Array) {
            msg = "Error: particle boundary conditions should be array of strings!";
            return EMOO_ERR_INPUT;
        }
        if (v->length() != 6) {
            msg = "Error: length of particle boundary condition does not match the number of dimensions!";
            return EMOO_ERR_INPUT;
        }
        for (int i = 0; i < 6; i++) {
            if (v->elems[i].type != Value::String) {
                msg = "Error: each element of particle boundary should be a string!";
                return EMOO_ERR_INPUT;
            }
            set_str(in->parts_bound[i], v->elems[i].s);
        }
    } else {
        for (int i = 0; i < 6; i++) set_str(in->parts_bound[i], "periodic");
    }
    // fields (:422-511)
    if (!(v = R.lookup("initialization.fields.electrostatic"))) {
        msg = "Error: electrostatic not set in input file (the reference terminates here)";
        return EMOO_ERR_INPUT;
    }
    in->electrostatic = (int)v->as_int();
    if (!(v = R.lookup("initialization.fields.init"))) {
        msg = "Error: field initialization method not set in input file!";
        return EMOO_ERR_INPUT;
    }
    if (v->type != Value::String) {
        msg = "Error: field initialization method should be a string!";
        return EMOO_ERR_INPUT;
    }
    set_str(in->fields_init, v->s);
    if ((v = R.lookup("initialization.fields.B0")) && v->length() == 3)
        for (int i = 0; i < 3; i++) in->B0[i] = v->elems[i].as_double();
    else
        for (int i = 0; i < 3; i++) in->B0[i] = 0.0;
    if ((v = R.lookup("initialization.fields.E0"))) {
        for (int i = 0; i < 3; i++) in->E0[i] = v->length() == 3 ? v->elems[i].as_double() : 0.0;
    } else {
        // the reference resets B0 here, not E0 (src/IO/readinfo.cpp:467)
        for (int i = 0; i < 3; i++) in->B0[i] = 0.0;
    }
    int isexternal = 0;
    if ((v = R.lookup("boundary.fields.conditions"))) {
        if (v->type != Value::Array) {
            msg = "Error: field boundary conditions should be array of strings!";
            return EMOO_ERR_INPUT;
        }
        if (v->length() != 6) {
            msg = "Error: length of field boundary condition does not match the number of dimensions!";
            return EMOO_ERR_INPUT;
        }
        for (int i = 0; i < 6; i++) {
            if (v->elems[i].type != Value::String) {
                msg = "Error: each element of field boundary should be a string!";
                return EMOO_ERR_INPUT;
            }
            set_str(in->fields_bound[i], v->elems[i].s);
            if (v->elems[i].s == "external") isexternal++;
        }
    } else {
        for (int i = 0; i < 6; i++) set_str(in->fields_bound[i], "periodic");
    }
    if (isexternal > 0) {  // (:513-686)
        int nw = 0;
        if ((v = R.lookup("boundary.fields.external.nwaves"))) {
            nw = (int)v->as_int();
            if (nw < 1) {
                msg = "Error: no external field specified ...";
                return EMOO_ERR_INPUT;
            }
            if (nw > EMOO_NWAVE) {
                msg = "Error: More external waves are specified than NWAVE!";
                return EMOO_ERR_INPUT;
            }
        }
        in->nwaves = nw;
        const Value *a = R.lookup("boundary.fields.external.inSide");
        if (!a) {
            msg = "Error: inSide not set in input file";
            return EMOO_ERR_INPUT;
        }
        if (a->length() != nw) {
            msg = "Error: length of inSide does not match nwaves!";
            return EMOO_ERR_INPUT;
        }
        for (int i = 0; i < nw; i++) in->inSide[i] = (int)a->elems[i].as_int();
        a = R.lookup("boundary.fields.external.inPolE");
        if (!a) {
            msg = "Error: inPolE not set in input file";
            return EMOO_ERR_INPUT;
        }
        if (a->length() != nw) {
            msg = "Error: length of inPol does not match nwaves!";
            return EMOO_ERR_INPUT;
        }
        for (int i = 0; i < nw; i++) in->inPolE[i] = (int)a->elems[i].as_int();
        if ((rc = wave_array(R, "boundary.fields.external.peakamps", nw, in->peakamps, "peakamps", msg))) return rc;
        if ((rc = wave_array(R, "boundary.fields.external.omegas", nw, in->omegas, "omegas", msg))) return rc;
        if ((rc = wave_array(R, "boundary.fields.external.phases", nw, in->phases, "phases", msg))) return rc;
        if ((rc = wave_array(R, "boundary.fields.external.invWidths", nw, in->invWidths, "invWidths", msg))) return rc;
        if ((rc = wave_array(R, "boundary.fields.external.delays", nw, in->delays, "delays", msg))) return rc;
        if (restart == 0 && strcmp(in->fields_init, "poisson") == 0) {
            const char *names[4] = {"bound_phi", "bound_Ax", "bound_Ay", "bound_Az"};
            double *dst[4] = {in->bound_phi, in->bound_Ax, in->bound_Ay, in->bound_Az};
            for (int q = 0; q < 4; q++) {
                std::string path = std::string("boundary.fields.external.poisson.") + names[q];
                const Value *b = R.lookup(path.c_str());
                if (!b) {
                    msg = std::string("Error: ") + names[q] + " not set in input file";
                    return EMOO_ERR_INPUT;
                }
                if (b->length() != 6) {
                    msg = std::string("Error: length of ") + names[q] + " is not 6!";
                    return EMOO_ERR_INPUT;
                }
                for (int i = 0; i < 6; i++) dst[q][i] = b->elems[i].as_double();
            }
        }
    } else {
        in->nwaves = 0;
    }
    // diagnostics (:691-727)
    in->nstep_fields = (v = R.lookup("diagnostics.nstep_fields")) ? (int)v->as_int() : 10;
    in->nstep_parts = (v = R.lookup("diagnostics.nstep_parts")) ? (int)v->as_int() : 10;
    in->nstep_restart = (v = R.lookup("diagnostics.nstep_restart")) ? (int)v->as_int() : 100;
    if (!(v = R.lookup("diagnostics.particles.output_pCount"))) {
        msg = "Error: output_pCount not set in input file (the reference terminates here)";
        return EMOO_ERR_INPUT;
    }
    in->output_pCount = (int)v->as_int();
    in->which_fields = (v = R.lookup("diagnostics.fields.which_fields")) ? (int)v->as_int() : -1;
    return EMOO_OK;
}

}  // namespace

extern "C" {

int emoo_parse_input(const char *text, emoo_input_info *out) {
    if (!text || !out) return EMOO_ERR_ARG;
    memset(out, 0, sizeof(*out));
    Parser P;
    P.p = text;
    P.end = text + strlen(text);
    Reader R;
    R.root.type = Value::Group;
    if (!P.settings(R.root, 0)) {
        g_last_message = "Parse error: " + P.err;
        return EMOO_ERR_INPUT;
    }
    g_last_message.clear();
    return read_info(R, out);
}

int emoo_read_input(const char *path, emoo_input_info *out) {
    if (!path || !out) return EMOO_ERR_ARG;
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        g_last_message = std::string("I/O error while reading file ") + path;
        return EMOO_ERR_INPUT;
    }
    std::string text;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, n);
    fclose(fp);
    return emoo_parse_input(text.c_str(), out);
}

const char *emoo_input_message(void) { return g_last_message.c_str(); }

// Input::ProcessInfo, src/IO/check.cpp:12-147 (one MPI rank).
int emoo_process_info(emoo_input_info *in) {
    if (!in) return EMOO_ERR_ARG;
    int err = 0;
    for (int i = 0; i < 3; i++) {
        int nproc = in->nProc[i] > 0 ? in->nProc[i] : 1;
        int resid = in->nCell[i] % nproc;
        if (resid) in->nCell[i] -= resid;
        if (in->nCell[i] <= 0) return EMOO_ERR_INPUT;
    }
    double vol = 1.0;
    for (int i = 0; i < 3; i++) vol *= in->Lxyz[i];
    if (!(vol > 0)) return EMOO_ERR_INPUT;
    if (in->nt < 0) in->nt = 1;
    double n0 = in->nparticles_tot / vol;
    double dens = in->dens_phys;
    if (dens < 0) dens = -dens;
    else if (dens == 0) dens = n0;
    in->dens_phys = dens;
    double ratio = n0 > 0 ? dens / n0 : -1.0;
    in->super_ratio = ratio;
    int nspec = in->nspecies;
    double cden = 0.0;
    for (int i = 0; i < nspec; i++) {
        if (in->dens_frac[i] < 0) return EMOO_ERR_INPUT;
        cden += in->dens_frac[i];
    }
    for (int i = 0; i < nspec; i++) {
        if (in->temp[i] < 0) in->temp[i] = -in->temp[i];
        if (in->mass_ratio[i] < 0) in->mass_ratio[i] = -in->mass_ratio[i];
        if (in->mass_ratio[i] == 0) err++;
    }
    if (ratio > 0) {
        for (int i = 0; i < nspec; i++) {
            in->dens_frac[i] /= cden;
            in->mass_ratio[i] *= ratio;
            in->charge_ratio[i] *= ratio;
            in->temp[i] *= ratio;
        }
    }
    for (int d = 0; d < 3; d++) {
        int fl = strcmp(in->fields_bound[2 * d], "periodic"), fr = strcmp(in->fields_bound[2 * d + 1], "periodic");
        int pl = strcmp(in->parts_bound[2 * d], "periodic"), pr = strcmp(in->parts_bound[2 * d + 1], "periodic");
        bool allp = !fl && !fr && !pl && !pr;
        bool nonep = fl && fr && pl && pr;
        if (!allp && !nonep) err++;
    }
    if (in->nwaves >= EMOO_NWAVE) return EMOO_ERR_INPUT;
    for (int i = 0; i < in->nwaves; i++)
        if (in->inPolE[i] < 0 || in->inPolE[i] > 3) return EMOO_ERR_INPUT;
    // nparticles_domain is left alone: the reference's Domain sets it
    // (src/domain/domain.cpp:100), not ProcessInfo
    return err ? EMOO_ERR_INPUT : EMOO_OK;
}

}  // extern "C"
