// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_3030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 3, 0, 3, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 2, 0, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
