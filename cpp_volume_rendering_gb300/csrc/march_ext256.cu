// march_ext256.cu — the extinction marchers of 256-thread CTAs (single frames and batches).
#include "march_ext.cuh"

namespace cvr {
CVR_EXTINCTION_INSTANCES(256)
}  // namespace cvr
