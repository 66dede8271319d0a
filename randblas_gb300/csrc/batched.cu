// batched.cu -- placeholder translation unit, filled in by the batching path.
#include "rbg_internal.h"

extern "C" int rbg_lskge3_batched(int32_t, const rbg_batch_problem *, int64_t, int32_t,
                                  rbg_stream_t) {
    rbg::set_last_error("batching path not built yet");
    return RBG_ERROR_UNSUPPORTED;
}

extern "C" int rbg_batched_tile_configs(int32_t *count) {
    if (count) *count = 0;
    return RBG_SUCCESS;
}
