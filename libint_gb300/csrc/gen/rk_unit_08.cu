// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 3, 0, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_2011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 1, 1, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
