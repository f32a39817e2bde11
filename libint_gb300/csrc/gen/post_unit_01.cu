// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.
#include "post_classes.cuh"

namespace lgx {
cudaError_t post_launch_f_3333(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<3, 3, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_f_3333(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<3, 3, 3, 3>>(block, smem);
}
cudaError_t post_launch_fb_3232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 2, 3, 2>>(a, grid, block, smem, st);
}
int post_occ_fb_3232(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 2, 3, 2>>(block, smem);
}
cudaError_t post_launch_fb_3033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 0, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_fb_3033(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 0, 3, 3>>(block, smem);
}
cudaError_t post_launch_f_2033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<2, 0, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_f_2033(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<2, 0, 3, 3>>(block, smem);
}
cudaError_t post_launch_d_2231(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<double, kModeJK, PostGen<2, 2, 3, 1>>(a, grid, block, smem, st);
}
int post_occ_d_2231(int block, size_t smem) {
  return occ_t<double, kModeJK, PostGen<2, 2, 3, 1>>(block, smem);
}
cudaError_t post_launch_fb_3122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 1, 2, 2>>(a, grid, block, smem, st);
}
int post_occ_fb_3122(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 1, 2, 2>>(block, smem);
}
cudaError_t post_launch_f_1132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<1, 1, 3, 2>>(a, grid, block, smem, st);
}
int post_occ_f_1132(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<1, 1, 3, 2>>(block, smem);
}
cudaError_t post_launch_d_2131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<double, kModeJK, PostGen<2, 1, 3, 1>>(a, grid, block, smem, st);
}
int post_occ_d_2131(int block, size_t smem) {
  return occ_t<double, kModeJK, PostGen<2, 1, 3, 1>>(block, smem);
}
cudaError_t post_launch_fb_3031(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 0, 3, 1>>(a, grid, block, smem, st);
}
int post_occ_fb_3031(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 0, 3, 1>>(block, smem);
}
}  // namespace lgx
