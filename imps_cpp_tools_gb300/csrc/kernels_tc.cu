// Placeholder for the tcgen05 split-BF16 engine (filled in below this line in a later step).
#include "imps_tc.h"
#include "imps_status.h"

namespace imps {
struct TcPlan { int dummy; };
int tc_create(TcPlan** out, const Plan&, cudaStream_t) { *out = nullptr; return IMPS_ERR_UNSUPPORTED; }
int tc_destroy(TcPlan* t) { delete t; return IMPS_OK; }
int tc_invalidate(TcPlan*) { return IMPS_OK; }
int tc_run_stage(TcPlan*, const Stage&, const imps_dslots&, cudaStream_t) { return IMPS_ERR_UNSUPPORTED; }
}  // namespace imps
