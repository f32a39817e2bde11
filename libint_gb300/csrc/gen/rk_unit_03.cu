// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_1131(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 3, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_2130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 1, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 0, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
