// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jkb64_0033(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 3, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_1130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 3, 0, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1120(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeStoreB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 0, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
