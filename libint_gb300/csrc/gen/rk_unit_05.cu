// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_2031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 2, 0, 3, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_3030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 3, 0, 3, 0, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_1121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_1130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_0022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 2, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jkb64_0021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 1, kModeJKB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 1, kModeStoreB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 2, 0, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_0010(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
