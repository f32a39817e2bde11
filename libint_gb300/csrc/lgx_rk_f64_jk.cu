// FP64 register kernels, J/K digestion mode.
#include "lgx_rk.cuh"
#include "lgx_rk_dispatch.cuh"
LGX_RK_DEFINE_LAUNCHER(rk_launch_f64_jk, double, kModeJK)
