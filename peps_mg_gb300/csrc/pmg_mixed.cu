// pmg_mixed.cu -- FP32 V-cycles inside FP64 defect correction (placeholder).
#include "pmg_ctx.h"

namespace pmg {

struct MixedState {};

int Ctx::solve_mixed(double *, double *, const double *, int, double, double, pmg_report_t *)
{
    set_error("mixed precision not built yet");
    return PMG_EINVAL;
}

void Ctx::destroy_mixed()
{
    delete mixed;
    mixed = nullptr;
}

}  // namespace pmg
