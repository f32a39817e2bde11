// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_f_jk_2121(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 2, 1, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1021(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 2, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_1111(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 1, 1, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 0, 1, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_store_0011(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 1, 1, kModeStore>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0000(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 0, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
