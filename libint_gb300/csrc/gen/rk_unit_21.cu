// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jkb64_1032(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 3, 2, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 3, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 1, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeStoreB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 1, 1, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
