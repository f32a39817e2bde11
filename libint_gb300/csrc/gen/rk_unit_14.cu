// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 3, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 1, 0, kModeJK, false>(a, work, nsm, st);
}
}  // namespace lgx
