// Entry points declared in include/siml_gb300.h whose kernels are not built
// yet: they fail loudly with SIML_ERR_UNSUPPORTED.
#include "engine.h"

using namespace siml;

extern "C" {

int siml_batch_neighbors(siml_engine* h, int64_t, const int64_t*, const int64_t*, const int64_t*, const int64_t*,
                         const int64_t*, float, float, int64_t, int32_t*, float*, int32_t*, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_batch_neighbors: not available in this build");
}

}  // extern "C"
