// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 1, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0033(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 3, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_0032(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 2, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 0, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 1, 0, kModeJK, false>(a, work, nsm, st);
}
}  // namespace lgx
