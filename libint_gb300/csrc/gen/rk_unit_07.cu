// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_2130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 1, 3, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1032(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_2030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 1, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 0, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 0, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
