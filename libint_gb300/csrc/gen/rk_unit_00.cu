// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_0033(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 3, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 1, 1, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
