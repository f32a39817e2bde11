// GENERATED by libint_gb300/codegen/gen_rk.py -- do not edit.
#include "../lgx_rk.cuh"

namespace lgx {
cudaError_t rk_launch_d_jk_1131(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 1, 1, 3, 1, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_f_jk_1130(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 1, 1, 3, 0, kModeJK>(a, work, nsm, st);
}
cudaError_t rk_launch_d_schwarz_0030(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<double, 0, 0, 3, 0, kModeSchwarz>(a, work, nsm, st);
}
cudaError_t rk_launch_f_store_0020(const EriArgs& a, long long work, int nsm, cudaStream_t st) {
  return rk_launch_one<float, 0, 0, 2, 0, kModeStore>(a, work, nsm, st);
}
}  // namespace lgx
