// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_1122(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 1, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
