// march_ext64.cu — the extinction marchers of 64-thread CTAs (single frames and batches).
#include "march_ext.cuh"

namespace cvr {
CVR_EXTINCTION_INSTANCES(64)
}  // namespace cvr
