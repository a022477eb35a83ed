// Adjoint of the whole-domain MAC projection (see maestro_mac.h).
#include "mac_internal.cuh"

extern "C" int mac_macproject_adjoint_dense(mac_ctx* ctx, const double*, const double*,
                                            const double*, const double*, const double*,
                                            const double*, const double*, const double*,
                                            const double*, const double*, double*, double*,
                                            double*, double*, double*, double*, double*,
                                            mac_stats* stats) {
    if (stats) stats->status = MAC_ERR_UNSUPPORTED;
    return ctx ? MAC_ERR_UNSUPPORTED : MAC_ERR_INVALID;
}
