// exfem_f32.cu — FP32 increment form with Kahan-compensated displacements.
#include "exfem_ctx.h"

namespace exfem {

int f32_alloc(Ctx &c) { c.err = "FP32 form not built yet"; return EXFEM_E_UNSUPPORTED; }
int f32_init(Ctx &c) { c.err = "FP32 form not built yet"; return EXFEM_E_UNSUPPORTED; }
int f32_launch_step(Ctx &c, int) { c.err = "FP32 form not built yet"; return EXFEM_E_UNSUPPORTED; }
int f32_launch_sample0(Ctx &c, int) { c.err = "FP32 form not built yet"; return EXFEM_E_UNSUPPORTED; }
int f32_get_u(Ctx &c, int, std::vector<double> &) { c.err = "FP32 form not built yet"; return EXFEM_E_UNSUPPORTED; }

}  // namespace exfem
