// Entry points declared in include/siml_gb300.h whose kernels are not built
// yet: they fail loudly with SIML_ERR_UNSUPPORTED.
#include "engine.h"

using namespace siml;

extern "C" {

int siml_hist101(siml_engine* h, int64_t, int64_t, int32_t*, int64_t, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_hist101: not available in this build");
}
int siml_topk(siml_engine* h, int64_t, int64_t, int64_t, int32_t*, float*, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_topk: not available in this build");
}
int siml_hist_global(siml_engine* h, int64_t, int64_t, uint64_t*, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_hist_global: not available in this build");
}
int siml_batch_neighbors(siml_engine* h, int64_t, const int64_t*, const int64_t*, const int64_t*, const int64_t*,
                         const int64_t*, float, float, int64_t, int32_t*, float*, int32_t*, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_batch_neighbors: not available in this build");
}
int siml_row_histogram101(siml_engine* h, const float*, int64_t, int64_t, int64_t, uint32_t*, int) {
    clear_error();
    (void)h;
    return fail(SIML_ERR_UNSUPPORTED, "siml_row_histogram101: not available in this build");
}

}  // extern "C"
