// march_ext128.cu — the extinction marchers of 128-thread CTAs (single frames and batches).
#include "march_ext.cuh"

namespace cvr {
CVR_EXTINCTION_INSTANCES(128)
}  // namespace cvr
