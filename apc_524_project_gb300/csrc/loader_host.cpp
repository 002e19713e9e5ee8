// loader_host.cpp - host-side seeded particle sampler (pure host code; the
// device sampler in loader.cu produces the same bits).
#include <stdint.h>

#include "emoo.h"
#include "loader_common.h"

extern "C" int emoo_generate_host(const emoo_gen_params *g, int64_t first, int64_t n, double *x, double *y, double *z,
                                  double *vx, double *vy, double *vz, double *gamma) {
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
