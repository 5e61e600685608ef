// step_fixed.cu -- temporally blocked block-fixed-point upwind kernel.
#include "fdb_internal.h"

namespace fdb {

int fixed_supported(const Geom&, const Coeffs3&, int) {
  return fail(FDB_ERR_UNSUPPORTED, "fixed-point kernel not built yet");
}

int launch_advect_fixed(const Geom&, const Coeffs3&, int, int, double**, int*, double*, size_t,
                        cudaStream_t) {
  return fail(FDB_ERR_UNSUPPORTED, "fixed-point kernel not built yet");
}

}  // namespace fdb
