// rotation_tc.cu -- tcgen05 evaluation path (BF16 3-term split product, FP32 accumulation in
// tensor memory). Placeholder until the kernel lands: the entry points report UNSUPPORTED.
#include "common.cuh"
#include "host.h"

SPEO_DEFINE_DEVERR(speo_deverr_tc)

using namespace speo;

extern "C" int speo_evaluate_tc(const speo_segment *, const speo_work_item *, int, int, int, const float *, float *,
                                void *)
{
    return fail(SPEO_ERR_UNSUPPORTED, "speo_evaluate_tc: not built yet");
}

extern "C" int speo_tc_generation(const speo_segment *, const speo_work_item *, int, int, int, const float *,
                                  const float *, float *, float *, uint32_t *, float *, float *, void *)
{
    return fail(SPEO_ERR_UNSUPPORTED, "speo_generation(use_tc=1): not built yet");
}
