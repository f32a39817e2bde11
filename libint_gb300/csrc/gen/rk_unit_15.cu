// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 3, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 0, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 0, 0, kModeSchwarz>(a, work, nsm, st);
}
}  // namespace lgx
