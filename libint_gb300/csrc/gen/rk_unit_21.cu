// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_1022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 2, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
