// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_att_0033(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 3, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 3, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
