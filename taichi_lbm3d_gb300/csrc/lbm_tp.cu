// K4: two-phase colour-gradient step (placeholder until the kernels land).
#include "lbm_internal.h"

int tp_launch_init(LbmHandle* h) { return lbm_set_err(h, LBM_EINVAL, "two-phase kernels not built yet"); }
int tp_launch_steps(LbmHandle* h, int32_t, bool) { return lbm_set_err(h, LBM_EINVAL, "two-phase kernels not built yet"); }
