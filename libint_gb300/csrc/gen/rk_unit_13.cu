// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_1131(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 3, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 1, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 0, kModeJK, false>(a, work, nsm, st);
}
}  // namespace lgx
