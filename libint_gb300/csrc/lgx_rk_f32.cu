// FP32 register kernels (mixed-precision path), J/K digestion and store.
#include "lgx_rk.cuh"
#include "lgx_rk_dispatch.cuh"
LGX_RK_DEFINE_LAUNCHER(rk_launch_f32_jk, float, kModeJK)
LGX_RK_DEFINE_LAUNCHER(rk_launch_f32_store, float, kModeStore)
