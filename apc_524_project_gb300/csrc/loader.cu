// loader.cu - device-side seeded particle sampler (same streams as the host
// sampler in loader_host.cpp; compiled with --fmad=false so both agree bit
// for bit). Writes straight into the handle's FP64 SoA or, for the mixed
// form, into a staging buffer that is converted to cell + offset form.
#include <cuda_runtime.h>

#include <algorithm>

#include "emoo_internal.h"
#include "loader_common.h"

namespace emoo {

namespace {

__global__ void k_generate(emoo_gen_params gp, int64_t first, int64_t n, double *x, double *y, double *z, double *vx,
                           double *vy, double *vz, double *g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double o[7];
        emoo_sample_particle(&gp, first + i, o);
        x[i] = o[0];
        y[i] = o[1];
        z[i] = o[2];
        vx[i] = o[3];
        vy[i] = o[4];
        vz[i] = o[5];
        if (g) g[i] = o[6];
    }
}

}  // namespace

// Generates particles [first, first+n) of stream gp into the FP64 arrays at
// particle index dst (FP64 form) or into seven FP64 staging arrays of n
// elements at h->pay (mixed form; the caller converts them).
int generate_device(emoo_handle *h, const emoo_gen_params *gp, int64_t first, int64_t n, int64_t dst) {
    if (n <= 0) return EMOO_OK;
    int nb = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    if (h->precision == EMOO_FP64) {
        h->launches++;
        k_generate<<<nb, 256, 0, h->stream>>>(*gp, first, n, h->x + dst, h->y + dst, h->z + dst, h->vx + dst,
                                              h->vy + dst, h->vz + dst, h->gam + dst);
    } else {
        double *b = (double *)h->pay;
        h->launches++;
        k_generate<<<nb, 256, 0, h->stream>>>(*gp, first, n, b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n,
                                              b + 6 * n);
    }
    EMOO_CUDA(cudaGetLastError());
    return EMOO_OK;
}

}  // namespace emoo
