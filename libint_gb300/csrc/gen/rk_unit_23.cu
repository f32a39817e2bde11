// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_1121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0032(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 2, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 3, 0, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
