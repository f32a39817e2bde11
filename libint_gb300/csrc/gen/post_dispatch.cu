// GENERATED by libint_gb300/codegen/gen_post.py -- do not edit.
// Run-time dispatch of the program kernels with generated post stages.
#include "../lgx_kernels.cuh"

namespace lgx {
cudaError_t post_launch_d_3333(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3333(int block, size_t smem);
cudaError_t post_launch_d_3033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3033(int block, size_t smem);
cudaError_t post_launch_d_2132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2132(int block, size_t smem);
cudaError_t post_launch_d_3122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3122(int block, size_t smem);
cudaError_t post_launch_d_2122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2122(int block, size_t smem);
cudaError_t post_launch_f_3333(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3333(int block, size_t smem);
cudaError_t post_launch_f_3033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3033(int block, size_t smem);
cudaError_t post_launch_f_2132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2132(int block, size_t smem);
cudaError_t post_launch_f_3122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3122(int block, size_t smem);
cudaError_t post_launch_f_2122(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2122(int block, size_t smem);
cudaError_t post_launch_d_3233(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3233(int block, size_t smem);
cudaError_t post_launch_d_2232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2232(int block, size_t smem);
cudaError_t post_launch_d_2033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2033(int block, size_t smem);
cudaError_t post_launch_d_3032(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3032(int block, size_t smem);
cudaError_t post_launch_d_1132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_1132(int block, size_t smem);
cudaError_t post_launch_d_2131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2131(int block, size_t smem);
cudaError_t post_launch_f_3233(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3233(int block, size_t smem);
cudaError_t post_launch_f_2232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2232(int block, size_t smem);
cudaError_t post_launch_f_2033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2033(int block, size_t smem);
cudaError_t post_launch_f_3032(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3032(int block, size_t smem);
cudaError_t post_launch_f_1132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_1132(int block, size_t smem);
cudaError_t post_launch_f_2131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2131(int block, size_t smem);
cudaError_t post_launch_d_2233(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2233(int block, size_t smem);
cudaError_t post_launch_d_3232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3232(int block, size_t smem);
cudaError_t post_launch_d_1133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_1133(int block, size_t smem);
cudaError_t post_launch_d_2231(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2231(int block, size_t smem);
cudaError_t post_launch_d_1033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_1033(int block, size_t smem);
cudaError_t post_launch_d_2032(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2032(int block, size_t smem);
cudaError_t post_launch_d_3031(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3031(int block, size_t smem);
cudaError_t post_launch_f_2233(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2233(int block, size_t smem);
cudaError_t post_launch_f_3232(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3232(int block, size_t smem);
cudaError_t post_launch_f_1133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_1133(int block, size_t smem);
cudaError_t post_launch_f_2231(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2231(int block, size_t smem);
cudaError_t post_launch_f_1033(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_1033(int block, size_t smem);
cudaError_t post_launch_f_2032(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2032(int block, size_t smem);
cudaError_t post_launch_f_3031(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3031(int block, size_t smem);
cudaError_t post_launch_d_3133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3133(int block, size_t smem);
cudaError_t post_launch_d_2133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2133(int block, size_t smem);
cudaError_t post_launch_d_3132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3132(int block, size_t smem);
cudaError_t post_launch_d_2222(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_2222(int block, size_t smem);
cudaError_t post_launch_d_3131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3131(int block, size_t smem);
cudaError_t post_launch_d_3022(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_d_3022(int block, size_t smem);
cudaError_t post_launch_f_3133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3133(int block, size_t smem);
cudaError_t post_launch_f_2133(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2133(int block, size_t smem);
cudaError_t post_launch_f_3132(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3132(int block, size_t smem);
cudaError_t post_launch_f_2222(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_2222(int block, size_t smem);
cudaError_t post_launch_f_3131(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3131(int block, size_t smem);
cudaError_t post_launch_f_3022(const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st);
int post_occ_f_3022(int block, size_t smem);

// Launches the J/K program kernel of (precision, class) with its
// generated post stage; cudaErrorNotSupported when there is none.
cudaError_t post_launch(bool fp32, int la, int lb, int lc, int ld, const EriArgs& a, int grid, int block, size_t smem, cudaStream_t st) {
  switch ((fp32 ? 4096 : 0) + ((la * 8 + lb) * 8 + lc) * 8 + ld) {
    case 1755: return post_launch_d_3333(a, grid, block, smem, st);
    case 1563: return post_launch_d_3033(a, grid, block, smem, st);
    case 1114: return post_launch_d_2132(a, grid, block, smem, st);
    case 1618: return post_launch_d_3122(a, grid, block, smem, st);
    case 1106: return post_launch_d_2122(a, grid, block, smem, st);
    case 5851: return post_launch_f_3333(a, grid, block, smem, st);
    case 5659: return post_launch_f_3033(a, grid, block, smem, st);
    case 5210: return post_launch_f_2132(a, grid, block, smem, st);
    case 5714: return post_launch_f_3122(a, grid, block, smem, st);
    case 5202: return post_launch_f_2122(a, grid, block, smem, st);
    case 1691: return post_launch_d_3233(a, grid, block, smem, st);
    case 1178: return post_launch_d_2232(a, grid, block, smem, st);
    case 1051: return post_launch_d_2033(a, grid, block, smem, st);
    case 1562: return post_launch_d_3032(a, grid, block, smem, st);
    case 602: return post_launch_d_1132(a, grid, block, smem, st);
    case 1113: return post_launch_d_2131(a, grid, block, smem, st);
    case 5787: return post_launch_f_3233(a, grid, block, smem, st);
    case 5274: return post_launch_f_2232(a, grid, block, smem, st);
    case 5147: return post_launch_f_2033(a, grid, block, smem, st);
    case 5658: return post_launch_f_3032(a, grid, block, smem, st);
    case 4698: return post_launch_f_1132(a, grid, block, smem, st);
    case 5209: return post_launch_f_2131(a, grid, block, smem, st);
    case 1179: return post_launch_d_2233(a, grid, block, smem, st);
    case 1690: return post_launch_d_3232(a, grid, block, smem, st);
    case 603: return post_launch_d_1133(a, grid, block, smem, st);
    case 1177: return post_launch_d_2231(a, grid, block, smem, st);
    case 539: return post_launch_d_1033(a, grid, block, smem, st);
    case 1050: return post_launch_d_2032(a, grid, block, smem, st);
    case 1561: return post_launch_d_3031(a, grid, block, smem, st);
    case 5275: return post_launch_f_2233(a, grid, block, smem, st);
    case 5786: return post_launch_f_3232(a, grid, block, smem, st);
    case 4699: return post_launch_f_1133(a, grid, block, smem, st);
    case 5273: return post_launch_f_2231(a, grid, block, smem, st);
    case 4635: return post_launch_f_1033(a, grid, block, smem, st);
    case 5146: return post_launch_f_2032(a, grid, block, smem, st);
    case 5657: return post_launch_f_3031(a, grid, block, smem, st);
    case 1627: return post_launch_d_3133(a, grid, block, smem, st);
    case 1115: return post_launch_d_2133(a, grid, block, smem, st);
    case 1626: return post_launch_d_3132(a, grid, block, smem, st);
    case 1170: return post_launch_d_2222(a, grid, block, smem, st);
    case 1625: return post_launch_d_3131(a, grid, block, smem, st);
    case 1554: return post_launch_d_3022(a, grid, block, smem, st);
    case 5723: return post_launch_f_3133(a, grid, block, smem, st);
    case 5211: return post_launch_f_2133(a, grid, block, smem, st);
    case 5722: return post_launch_f_3132(a, grid, block, smem, st);
    case 5266: return post_launch_f_2222(a, grid, block, smem, st);
    case 5721: return post_launch_f_3131(a, grid, block, smem, st);
    case 5650: return post_launch_f_3022(a, grid, block, smem, st);
  }
  return cudaErrorNotSupported;
}

int post_blocks_per_sm(bool fp32, int la, int lb, int lc, int ld, int block, size_t smem) {
  switch ((fp32 ? 4096 : 0) + ((la * 8 + lb) * 8 + lc) * 8 + ld) {
    case 1755: return post_occ_d_3333(block, smem);
    case 1563: return post_occ_d_3033(block, smem);
    case 1114: return post_occ_d_2132(block, smem);
    case 1618: return post_occ_d_3122(block, smem);
    case 1106: return post_occ_d_2122(block, smem);
    case 5851: return post_occ_f_3333(block, smem);
    case 5659: return post_occ_f_3033(block, smem);
    case 5210: return post_occ_f_2132(block, smem);
    case 5714: return post_occ_f_3122(block, smem);
    case 5202: return post_occ_f_2122(block, smem);
    case 1691: return post_occ_d_3233(block, smem);
    case 1178: return post_occ_d_2232(block, smem);
    case 1051: return post_occ_d_2033(block, smem);
    case 1562: return post_occ_d_3032(block, smem);
    case 602: return post_occ_d_1132(block, smem);
    case 1113: return post_occ_d_2131(block, smem);
    case 5787: return post_occ_f_3233(block, smem);
    case 5274: return post_occ_f_2232(block, smem);
    case 5147: return post_occ_f_2033(block, smem);
    case 5658: return post_occ_f_3032(block, smem);
    case 4698: return post_occ_f_1132(block, smem);
    case 5209: return post_occ_f_2131(block, smem);
    case 1179: return post_occ_d_2233(block, smem);
    case 1690: return post_occ_d_3232(block, smem);
    case 603: return post_occ_d_1133(block, smem);
    case 1177: return post_occ_d_2231(block, smem);
    case 539: return post_occ_d_1033(block, smem);
    case 1050: return post_occ_d_2032(block, smem);
    case 1561: return post_occ_d_3031(block, smem);
    case 5275: return post_occ_f_2233(block, smem);
    case 5786: return post_occ_f_3232(block, smem);
    case 4699: return post_occ_f_1133(block, smem);
    case 5273: return post_occ_f_2231(block, smem);
    case 4635: return post_occ_f_1033(block, smem);
    case 5146: return post_occ_f_2032(block, smem);
    case 5657: return post_occ_f_3031(block, smem);
    case 1627: return post_occ_d_3133(block, smem);
    case 1115: return post_occ_d_2133(block, smem);
    case 1626: return post_occ_d_3132(block, smem);
    case 1170: return post_occ_d_2222(block, smem);
    case 1625: return post_occ_d_3131(block, smem);
    case 1554: return post_occ_d_3022(block, smem);
    case 5723: return post_occ_f_3133(block, smem);
    case 5211: return post_occ_f_2133(block, smem);
    case 5722: return post_occ_f_3132(block, smem);
    case 5266: return post_occ_f_2222(block, smem);
    case 5721: return post_occ_f_3131(block, smem);
    case 5650: return post_occ_f_3022(block, smem);
  }
  return 0;
}

// Contracted-set size and the slots the generated post stage needs
// (accumulators + bra-stage output + shell set); false if none.
bool post_info(int la, int lb, int lc, int ld, int* nacc, int* slots) {
  switch (((la * 8 + lb) * 8 + lc) * 8 + ld) {
    case 539: *nacc = 222; *slots = 594; return true;
    case 602: *nacc = 414; *slots = 1152; return true;
    case 603: *nacc = 666; *slots = 1782; return true;
    case 1050: *nacc = 276; *slots = 686; return true;
    case 1051: *nacc = 444; *slots = 1064; return true;
    case 1106: *nacc = 496; *slots = 1336; return true;
    case 1113: *nacc = 400; *slots = 1090; return true;
    case 1114: *nacc = 736; *slots = 1966; return true;
    case 1115: *nacc = 1184; *slots = 3044; return true;
    case 1170: *nacc = 961; *slots = 2361; return true;
    case 1177: *nacc = 775; *slots = 1925; return true;
    case 1178: *nacc = 1426; *slots = 3476; return true;
    case 1179: *nacc = 2294; *slots = 5394; return true;
    case 1554: *nacc = 310; *slots = 702; return true;
    case 1561: *nacc = 250; *slots = 572; return true;
    case 1562: *nacc = 460; *slots = 1034; return true;
    case 1563: *nacc = 740; *slots = 1608; return true;
    case 1618: *nacc = 775; *slots = 1951; return true;
    case 1625: *nacc = 625; *slots = 1591; return true;
    case 1626: *nacc = 1150; *slots = 2872; return true;
    case 1627: *nacc = 1850; *slots = 4454; return true;
    case 1690: *nacc = 2116; *slots = 4986; return true;
    case 1691: *nacc = 3404; *slots = 7744; return true;
    case 1755: *nacc = 5476; *slots = 11552; return true;
  }
  return false;
}
}  // namespace lgx
