// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2022(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 2, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_3021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 3, 0, 2, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_2021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 2, 1, kModeJK, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_2030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 0, 3, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeStore, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_0031(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 3, 1, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 0, kModeSchwarz, false>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_att_1020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 0, kModeJK, true>(a, work, nsm, st);
}
cudaError_t rk_launch_f_storeb64_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeStoreB64, false>(a, work, nsm, st);
}
cudaError_t rk_launch_d_jk_att_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 0, 0, kModeJK, true>(a, work, nsm, st);
}
}  // namespace lgx
