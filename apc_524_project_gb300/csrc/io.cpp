// io.cpp - output files: the field time series (raw files in the layout of
// the reference's Hdf5IO datasets) and restart files (no reference
// counterpart: the reference parses nstep_restart and writes nothing).
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

#include "emoo_internal.h"

using namespace emoo;

namespace {

// ---- field time series ---------------------------------------------------

struct FieldOut {
    const char *name;
    int id;       // field slot (B: the B slot, averaged with its B_tm1 slot)
    int off_axis;  // edge / face offsets: bit a set = d/2 along axis a
};

// Hdf5IO's datasets in its order (src/IO/hdf5io.cpp:108-141), with the
// offsets of Grid::getGridPhys (src/grid/grid.cpp:415-466): edgeX (Ex, Jx)
// x, faceX (Bx) y and z, vertex (rho) none.
const FieldOut FIELDS[10] = {
    {"Ex", EMOO_EX, 1}, {"Ey", EMOO_EY, 2}, {"Ez", EMOO_EZ, 4}, {"Bx", EMOO_BX, 6}, {"By", EMOO_BY, 5},
    {"Bz", EMOO_BZ, 3}, {"Jx", EMOO_JX, 1}, {"Jy", EMOO_JY, 2}, {"Jz", EMOO_JZ, 4}, {"rho", EMOO_RHO, 0},
};

bool selected(int which, int k) {
    if (which == EMOO_FIELDS_ALL) return true;
    if (k < 3) return which == EMOO_FIELDS_E;
    if (k < 6) return which == EMOO_FIELDS_B;
    if (k < 9) return which == EMOO_FIELDS_J;
    return which == EMOO_FIELDS_RHO;
}

int make_dir(const std::string &d) {
    if (mkdir(d.c_str(), 0777) == 0 || errno == EEXIST) return EMOO_OK;
    return EMOO_ERR_INPUT;
}

bool exists(const std::string &p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

int append(const std::string &path, const void *data, size_t bytes, bool start) {
    FILE *f = fopen(path.c_str(), start ? "wb" : "ab");
    if (!f) return EMOO_ERR_INPUT;
    const size_t w = fwrite(data, 1, bytes, f);
    const int rc = fclose(f);
    return (w == bytes && rc == 0) ? EMOO_OK : EMOO_ERR_INPUT;
}

// ---- restart files -------------------------------------------------------

constexpr char MAGIC[8] = {'E', 'M', 'O', 'O', 'R', 'S', 'T', '1'};

struct RestartHeader {
    char magic[8];
    int32_t version, precision, n[3], nspec;
    int32_t bswap, rho_stale, first_push, has_ids, has_gam, has_g0, dead_pending, pad;
    int64_t np, count[EMOO_NSPEC];
    double t, dt, dtp;
    int64_t step_index, next_hist, nhist_rows;
};

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

// device array <-> file through a host buffer
int put(FILE *f, const void *dev, size_t bytes, std::vector<char> &buf, cudaStream_t st) {
    if (!bytes) return EMOO_OK;
    buf.resize(bytes);
    EMOO_CUDA(cudaMemcpyAsync(buf.data(), dev, bytes, cudaMemcpyDeviceToHost, st));
    EMOO_CUDA(cudaStreamSynchronize(st));
    return fwrite(buf.data(), 1, bytes, f) == bytes ? EMOO_OK : EMOO_ERR_INPUT;
}

int get(FILE *f, void *dev, size_t bytes, std::vector<char> &buf, cudaStream_t st) {
    if (!bytes) return EMOO_OK;
    buf.resize(bytes);
    if (fread(buf.data(), 1, bytes, f) != bytes) return EMOO_ERR_INPUT;
    EMOO_CUDA(cudaMemcpyAsync(dev, buf.data(), bytes, cudaMemcpyHostToDevice, st));
    EMOO_CUDA(cudaStreamSynchronize(st));
    return EMOO_OK;
}

// The arrays of the restart file in order: fields, then particles. The
// optional particle arrays (FP64 gamma, the mixed form's loaded gamma before
// the first push, ids) are present as the header's flags say.
struct Arrays {
    std::vector<std::pair<void *, size_t>> fields;     // pointer, bytes
    std::vector<std::pair<void *, size_t>> particles;  // pointer, bytes per particle
};

Arrays state_arrays(emoo_handle *h, bool with_gam, bool with_g0, bool with_ids) {
    Arrays a;
    const size_t npts = (size_t)h->g.npts;
    if (h->precision == EMOO_FP64) {
        for (int id = 0; id <= EMOO_BZ_TM1; id++) a.fields.push_back({h->slot[id], sizeof(double) * npts});
        void *P[6] = {h->x, h->y, h->z, h->vx, h->vy, h->vz};
        for (void *p : P) a.particles.push_back({p, sizeof(double)});
        if (with_gam) a.particles.push_back({h->gam, sizeof(double)});
    } else {
        float *E[3], *Bs[6];
        long long *J[4];
        double q0;
        mixed_field_arrays(h, E, Bs);
        mixed_point_arrays(h, J, &q0);
        for (float *p : E) a.fields.push_back({p, sizeof(float) * npts});
        for (float *p : Bs) a.fields.push_back({p, sizeof(float) * npts});
        for (long long *p : J) a.fields.push_back({p, sizeof(long long) * npts});
        a.particles.push_back({h->cell, sizeof(int32_t)});
        void *P[6] = {h->ox, h->oy, h->oz, h->ux, h->uy, h->uz};
        for (void *p : P) a.particles.push_back({p, sizeof(float)});
        if (with_g0) a.particles.push_back({h->g0, sizeof(float)});
    }
    if (with_ids) a.particles.push_back({h->ids, sizeof(int64_t)});
    return a;
}

// Size in bytes of a restart file with this header: the header, the history
// rows, the fields and np particles, in the layout state_arrays gives.
int64_t restart_bytes(const RestartHeader &hd) {
    const int64_t npts = (int64_t)(hd.n[0] + 3) * (hd.n[1] + 3) * (hd.n[2] + 3);
    int64_t field = 0, part = 0;
    if (hd.precision == EMOO_FP64) {
        field = 13 * 8 * npts;
        part = 6 * 8 + (hd.has_gam ? 8 : 0);
    } else {
        field = 9 * 4 * npts + 4 * 8 * npts;
        part = 4 + 6 * 4 + (hd.has_g0 ? 4 : 0);
    }
    if (hd.has_ids) part += 8;
    return (int64_t)sizeof(RestartHeader) + hd.nhist_rows * 8 * (int64_t)sizeof(double) + field + hd.np * part;
}

bool flag(int32_t v) { return v == 0 || v == 1; }

// Reads the header of `path` and checks that it describes a well-formed file:
// known version and precision, grid sizes and species count in range, 0/1
// flags, gamma arrays present as the writer stores them, non-negative
// per-species counts (zero past nspec) that sum to np, and a file of exactly
// the size the header implies (so no array can be read short). Nothing but
// the header is read. EMOO_ERR_INPUT for anything else.
int read_header(const char *path, RestartHeader &hd) {
    File F;
    if (!(F.f = fopen(path, "rb"))) return EMOO_ERR_INPUT;
    if (fread(&hd, sizeof(hd), 1, F.f) != 1 || memcmp(hd.magic, MAGIC, 8) != 0 || hd.version != 1)
        return EMOO_ERR_INPUT;
    if ((hd.precision != EMOO_FP64 && hd.precision != EMOO_MIXED) || hd.nspec < 0 || hd.nspec > EMOO_NSPEC)
        return EMOO_ERR_INPUT;
    for (int d = 0; d < 3; d++)
        if (hd.n[d] < 1 || hd.n[d] > (1 << 16)) return EMOO_ERR_INPUT;
    if (!flag(hd.bswap) || !flag(hd.rho_stale) || !flag(hd.first_push) || !flag(hd.has_ids) ||
        !flag(hd.has_gam) || !flag(hd.has_g0) || !flag(hd.dead_pending))
        return EMOO_ERR_INPUT;
    if (hd.np < 0 || hd.np >= (int64_t)UINT32_MAX || hd.nhist_rows < 0 || hd.nhist_rows > ((int64_t)1 << 40))
        return EMOO_ERR_INPUT;
    int64_t sum = 0;
    for (int s = 0; s < EMOO_NSPEC; s++) {
        if (hd.count[s] < 0 || (s >= hd.nspec && hd.count[s] != 0)) return EMOO_ERR_INPUT;
        sum += hd.count[s];
    }
    if (sum != hd.np) return EMOO_ERR_INPUT;
    // the FP64 store always carries gamma once it holds particles; the mixed
    // form's loaded gamma exists only before its first push
    if (hd.precision == EMOO_FP64 && (hd.has_g0 || (hd.np > 0 && !hd.has_gam))) return EMOO_ERR_INPUT;
    if (hd.precision == EMOO_MIXED && (hd.has_gam || (hd.has_g0 && !hd.first_push))) return EMOO_ERR_INPUT;
    if (fseeko(F.f, 0, SEEK_END) != 0) return EMOO_ERR_INPUT;
    const off_t size = ftello(F.f);
    if (size < 0 || (int64_t)size != restart_bytes(hd)) return EMOO_ERR_INPUT;
    return EMOO_OK;
}

}  // namespace

extern "C" {

int emoo_write_fields(emoo_handle *h, const char *dir, int which) {
    if (!h || !dir || which < EMOO_FIELDS_RHO || which > EMOO_FIELDS_ALL) return EMOO_ERR_ARG;
    EMOO_CUDA(cudaSetDevice(h->dev));
    EMOO_TRY(host_store_sync(h));  // rho is deposited from the store
    const std::string d = std::string(dir) + "/";
    EMOO_TRY(make_dir(d));
    const bool start = !exists(d + "time.f64");
    const Geom &g = h->g;
    const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
    const size_t npts = (size_t)g.npts, nphys = (size_t)n0 * n1 * n2;
    std::vector<double> a(npts), b(npts), out(nphys);
    for (int k = 0; k < 10; k++) {
        if (!selected(which, k)) continue;
        const FieldOut &fo = FIELDS[k];
        EMOO_TRY(emoo_get_field(h, fo.id, a.data()));
        const bool avg = fo.id >= EMOO_BX && fo.id <= EMOO_BZ;
        if (avg) EMOO_TRY(emoo_get_field(h, fo.id - EMOO_BX + EMOO_BX_TM1, b.data()));
        size_t q = 0;
        for (int i = 1; i <= n0; i++)
            for (int j = 1; j <= n1; j++)
                for (int l = 1; l <= n2; l++) {
                    const size_t p = ((size_t)i * g.tot[1] + j) * g.tot[2] + l;
                    out[q++] = avg ? (a[p] + b[p]) / 2 : a[p];
                }
        EMOO_TRY(append(d + fo.name + ".f64", out.data(), sizeof(double) * nphys, start));
        if (start) {
            std::vector<double> xyz;
            for (int ax = 0; ax < 3; ax++) {
                const double off = ((fo.off_axis >> ax) & 1) ? h->g.d[ax] / 2 : 0.0;
                for (int i = 1; i <= g.n[ax]; i++) xyz.push_back(h->info.xyz0[ax] + off + h->g.d[ax] * (i - 1));
            }
            EMOO_TRY(append(d + fo.name + ".xyz", xyz.data(), sizeof(double) * xyz.size(), true));
        }
    }
    return append(d + "time.f64", &h->t, sizeof(double), start);
}

int emoo_write_restart(emoo_handle *h, const char *path) {
    if (!h || !path) return EMOO_ERR_ARG;
    EMOO_CUDA(cudaSetDevice(h->dev));
    EMOO_TRY(host_store_sync(h));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    RestartHeader hd;
    memset(&hd, 0, sizeof(hd));
    memcpy(hd.magic, MAGIC, 8);
    hd.version = 1;
    hd.precision = h->precision;
    for (int d = 0; d < 3; d++) hd.n[d] = h->g.n[d];
    hd.nspec = h->nspec;
    hd.bswap = h->bswap;
    hd.rho_stale = h->rho_stale;
    hd.first_push = h->first_push;
    hd.has_ids = h->opts.track_ids != 0;
    hd.has_gam = h->precision == EMOO_FP64 && h->gam != nullptr;
    hd.has_g0 = h->precision != EMOO_FP64 && h->first_push && h->g0;
    hd.dead_pending = h->dead_pending;
    hd.np = h->np;
    for (int s = 0; s < EMOO_NSPEC; s++) hd.count[s] = h->count[s];
    hd.t = h->t;
    hd.dt = h->dt;
    hd.dtp = h->dtp;
    hd.step_index = h->step_index;
    hd.next_hist = h->next_hist;
    hd.nhist_rows = (int64_t)(h->hist_rows.size() / 8);
    File F;
    if (!(F.f = fopen(path, "wb"))) return EMOO_ERR_INPUT;
    if (fwrite(&hd, sizeof(hd), 1, F.f) != 1) return EMOO_ERR_INPUT;
    if (hd.nhist_rows &&
        fwrite(h->hist_rows.data(), sizeof(double), h->hist_rows.size(), F.f) != h->hist_rows.size())
        return EMOO_ERR_INPUT;
    const Arrays A = state_arrays(h, hd.has_gam, hd.has_g0, hd.has_ids);
    std::vector<char> buf;
    for (const auto &f : A.fields) EMOO_TRY(put(F.f, f.first, f.second, buf, h->stream));
    for (const auto &p : A.particles) EMOO_TRY(put(F.f, p.first, p.second * (size_t)h->np, buf, h->stream));
    if (fclose(F.f) != 0) {
        F.f = nullptr;
        return EMOO_ERR_INPUT;
    }
    F.f = nullptr;
    return EMOO_OK;
}

int emoo_restart_info(const char *path, emoo_restart_desc *out) {
    if (!path || !out) return EMOO_ERR_ARG;
    RestartHeader hd;
    EMOO_TRY(read_header(path, hd));
    memset(out, 0, sizeof(*out));
    out->precision = hd.precision;
    for (int d = 0; d < 3; d++) out->n[d] = hd.n[d];
    out->nspec = hd.nspec;
    out->has_ids = hd.has_ids;
    out->np = hd.np;
    for (int s = 0; s < EMOO_NSPEC; s++) out->count[s] = hd.count[s];
    out->t = hd.t;
    out->step_index = hd.step_index;
    out->nhist_rows = hd.nhist_rows;
    return EMOO_OK;
}

int emoo_read_restart(emoo_handle *h, const char *path) {
    if (!h || !path) return EMOO_ERR_ARG;
    if (h->host_mode) return EMOO_ERR_STATE;  // it replaces the particle store
    // every check before the handle changes: a malformed file or one of
    // another configuration leaves the handle as it was
    RestartHeader hd;
    EMOO_TRY(read_header(path, hd));
    if (hd.precision != h->precision || hd.nspec != h->nspec || hd.n[0] != h->g.n[0] || hd.n[1] != h->g.n[1] ||
        hd.n[2] != h->g.n[2] || hd.has_ids != (h->opts.track_ids != 0))
        return EMOO_ERR_STATE;
    if (hd.has_g0 && h->info.relativity == 0) return EMOO_ERR_STATE;
    EMOO_CUDA(cudaSetDevice(h->dev));
    EMOO_CUDA(cudaStreamSynchronize(h->stream));
    File F;
    if (!(F.f = fopen(path, "rb")) || fseeko(F.f, (off_t)sizeof(hd), SEEK_SET) != 0) return EMOO_ERR_INPUT;
    std::vector<double> rows((size_t)hd.nhist_rows * 8);
    if (!rows.empty() && fread(rows.data(), sizeof(double), rows.size(), F.f) != rows.size()) return EMOO_ERR_INPUT;
    EMOO_TRY(reserve_store(h, std::max<int64_t>(hd.np, 1)));
    if (hd.has_g0 && !h->g0) EMOO_CUDA(cudaMalloc(&h->g0, sizeof(float) * (size_t)h->cap));
    // from here on the store is overwritten; an I/O error part-way leaves it
    // empty (no particles, fields to be set again), never inconsistent
    h->first_push = hd.first_push;
    int64_t off = 0;
    for (int s = 0; s < EMOO_NSPEC; s++) {
        h->off[s] = off;
        h->count[s] = hd.count[s];
        off += h->count[s];
    }
    h->off[EMOO_NSPEC] = off;
    h->np = hd.np;
    const Arrays A = state_arrays(h, hd.has_gam, hd.has_g0, hd.has_ids);
    std::vector<char> buf;
    int rc = EMOO_OK;
    for (const auto &f : A.fields)
        if (rc == EMOO_OK) rc = get(F.f, f.first, f.second, buf, h->stream);
    for (const auto &p : A.particles)
        if (rc == EMOO_OK) rc = get(F.f, p.first, p.second * (size_t)h->np, buf, h->stream);
    if (rc != EMOO_OK) {
        for (int s = 0; s <= EMOO_NSPEC; s++) h->off[s] = 0;
        for (int s = 0; s < EMOO_NSPEC; s++) h->count[s] = 0;
        h->np = 0;
        h->fields_initialised = 0;
        return rc;
    }
    h->bswap = hd.bswap;
    h->rho_stale = hd.rho_stale;
    h->t = hd.t;
    h->dt = hd.dt;
    h->dtp = hd.dtp;
    h->step_index = hd.step_index;
    h->next_hist = hd.next_hist;
    h->hist_rows = rows;
    h->dead_pending = hd.dead_pending;
    h->fields_initialised = 1;
    return EMOO_OK;
}

}  // extern "C"
