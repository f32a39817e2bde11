// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.
#include "post_classes.cuh"

namespace lgx {
cudaError_t post_launch_f_3233(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<3, 2, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_f_3233(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<3, 2, 3, 3>>(block, smem);
}
cudaError_t post_launch_fb_3133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 1, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_fb_3133(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 1, 3, 3>>(block, smem);
}
cudaError_t post_launch_f_2232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<2, 2, 3, 2>>(a, grid, block, smem, st);
}
int post_occ_f_2232(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<2, 2, 3, 2>>(block, smem);
}
cudaError_t post_launch_d_1133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<double, kModeJK, PostGen<1, 1, 3, 3>>(a, grid, block, smem, st);
}
int post_occ_d_1133(int block, size_t smem) {
  return occ_t<double, kModeJK, PostGen<1, 1, 3, 3>>(block, smem);
}
cudaError_t post_launch_f_2132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJK, PostGen<2, 1, 3, 2>>(a, grid, block, smem, st);
}
int post_occ_f_2132(int block, size_t smem) {
  return occ_t<float, kModeJK, PostGen<2, 1, 3, 2>>(block, smem);
}
cudaError_t post_launch_d_3032(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<double, kModeJK, PostGen<3, 0, 3, 2>>(a, grid, block, smem, st);
}
int post_occ_d_3032(int block, size_t smem) {
  return occ_t<double, kModeJK, PostGen<3, 0, 3, 2>>(block, smem);
}
cudaError_t post_launch_fb_3131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 1, 3, 1>>(a, grid, block, smem, st);
}
int post_occ_fb_3131(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 1, 3, 1>>(block, smem);
}
cudaError_t post_launch_d_2122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<double, kModeJK, PostGen<2, 1, 2, 2>>(a, grid, block, smem, st);
}
int post_occ_d_2122(int block, size_t smem) {
  return occ_t<double, kModeJK, PostGen<2, 1, 2, 2>>(block, smem);
}
cudaError_t post_launch_fb_3022(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  return launch_eri_t<float, kModeJKB64, PostGen<3, 0, 2, 2>>(a, grid, block, smem, st);
}
int post_occ_fb_3022(int block, size_t smem) {
  return occ_t<float, kModeJKB64, PostGen<3, 0, 2, 2>>(block, smem);
}
}  // namespace lgx
