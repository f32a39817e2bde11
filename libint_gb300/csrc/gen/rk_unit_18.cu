// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 3, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1122(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_1031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 3, 1, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 3, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 1, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 0, kModeStore, false>(a, work, nsm, st);
}
}  // namespace lgx
