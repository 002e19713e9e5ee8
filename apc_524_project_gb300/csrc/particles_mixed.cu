// particles_mixed.cu - mixed-precision form (placeholder until implemented).
#include "emoo_internal.h"

namespace emoo {
struct FieldsF32 {};
int mixed_alloc(emoo_handle *) { return EMOO_ERR_UNSUPPORTED; }
void mixed_free(emoo_handle *) {}
int mixed_from_f64(emoo_handle *, int64_t, int64_t, const double *, const double *, const double *, const double *,
                   const double *, const double *, const double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_to_f64(emoo_handle *, int64_t, int64_t, double *, double *, double *, double *, double *, double *,
                 double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_step(emoo_handle *, double, int) { return EMOO_ERR_UNSUPPORTED; }
int mixed_sort_keys(emoo_handle *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_get_field(emoo_handle *, int, double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_set_field(emoo_handle *, int, const double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_moments(emoo_handle *, double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_field_energy(emoo_handle *, double *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_ghost_fill(emoo_handle *) { return EMOO_ERR_UNSUPPORTED; }
int mixed_plane_sets(emoo_handle *, const PlaneSet *, int) { return EMOO_ERR_UNSUPPORTED; }
}  // namespace emoo
