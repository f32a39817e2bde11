// FP64 register kernels, store and Schwarz modes.
#include "lgx_rk.cuh"
#include "lgx_rk_dispatch.cuh"
LGX_RK_DEFINE_LAUNCHER(rk_launch_f64_store, double, kModeStore)
LGX_RK_DEFINE_LAUNCHER(rk_launch_f64_schwarz, double, kModeSchwarz)
