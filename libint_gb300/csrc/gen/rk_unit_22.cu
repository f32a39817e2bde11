// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_1031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 3, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 1, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
