// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_1131(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 3, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 1, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 0, 0, kModeJK>(a, work, nsm, st);
}
}  // namespace lgx
