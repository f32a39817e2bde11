// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_0033(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 3, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 2, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 3, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 0, kModeStoreB64, false>(a, work, nsm, st);
}
}  // namespace lgx
