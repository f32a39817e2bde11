// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jkb64_1122(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 2, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 1, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_2030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 3, 0, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 2, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 3, 0, kModeStoreB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 2, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
