// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_3030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 3, 0, 3, 0, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1131(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 3, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_0032(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 0, 1, 0, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 0, 0, kModeJKB64, false>(a, work, nsm, st);
}
}  // namespace lgx
