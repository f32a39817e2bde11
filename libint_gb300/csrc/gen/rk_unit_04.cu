// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 3, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_2030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 2, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 0, kModeSchwarz, false>(a, work, nsm, st);
}
}  // namespace lgx
