// pending.cpp -- entry points whose implementation lands in later translation units.
#include "acum_internal.h"
#include "ctx.h"

namespace acum {
}  // namespace acum

using namespace acum;

extern "C" int acum_batch_create(acum_batch**, int) { return fail(nullptr, ACUM_ERR_UNSUPPORTED, "not built yet"); }
extern "C" int acum_batch_destroy(acum_batch*) { return ACUM_OK; }
extern "C" const char* acum_batch_last_error(const acum_batch*) { return "not built yet"; }
extern "C" int acum_batch_add(acum_batch*, const acum_inputs*, int, const float*, int, const int*, const float*, int*)
{
    return ACUM_ERR_UNSUPPORTED;
}
extern "C" int acum_batch_prepare(acum_batch*) { return ACUM_ERR_UNSUPPORTED; }
extern "C" int acum_batch_run(acum_batch*, int, int) { return ACUM_ERR_UNSUPPORTED; }
extern "C" int acum_batch_result(acum_batch*, int, double*) { return ACUM_ERR_UNSUPPORTED; }
extern "C" int acum_batch_timing(const acum_batch*, double*, long long*) { return ACUM_ERR_UNSUPPORTED; }
extern "C" int acum_batch_set_tile(acum_batch*, int, int, int) { return ACUM_ERR_UNSUPPORTED; }
