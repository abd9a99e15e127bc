// Brick path (bit-sliced sweep): placeholder until the kernels land.
#include "dmc_internal.h"

namespace dmc {

bool brick_supports(const ExtractArgs &) { return false; }

dmc_status brick_run(Ctx *, const ExtractArgs &, cudaStream_t) { return DMC_ERR_UNSUPPORTED; }

}  // namespace dmc
