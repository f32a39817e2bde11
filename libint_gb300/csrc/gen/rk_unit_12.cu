// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_1122(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 2, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 1, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 0, 0, kModeJK>(a, work, nsm, st);
}
}  // namespace lgx
