// lowp_tc.cu -- placeholder translation unit, filled in by the tensor-core precision path.
#include "rbg_internal.h"

extern "C" int rbg_lskge3_lowp_workspace(int32_t, int64_t, int64_t, int64_t, size_t *bytes) {
    if (bytes) *bytes = 0;
    rbg::set_last_error("precision path not built yet");
    return RBG_ERROR_UNSUPPORTED;
}

extern "C" int rbg_lskge3_lowp(int32_t, int32_t, int32_t, int32_t, int64_t, int64_t, int64_t,
                               float, const rbg_dense_skop *, int64_t, int64_t, const float *,
                               int64_t, float, float *, int64_t, void *, size_t, rbg_stream_t) {
    rbg::set_last_error("precision path not built yet");
    return RBG_ERROR_UNSUPPORTED;
}
