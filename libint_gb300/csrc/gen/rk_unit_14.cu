// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 2, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 2, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 0, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
