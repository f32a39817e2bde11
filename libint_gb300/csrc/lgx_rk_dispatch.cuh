// Launcher definitions for the register kernels: one function per
// (precision, mode) that selects the class instantiation at run time and
// reports the occupancy-derived grid.
#pragma once
#include "lgx_rk.cuh"

#define LGX_RK_DEFINE_LAUNCHER(NAME, T, MODE)                                         \
  namespace lgx {                                                                      \
  cudaError_t NAME(int la, int lb, int lc, int ld, const EriArgs& a, long long work,    \
                   int nsm, cudaStream_t st) {                                          \
    const int block = 128;                                                             \
    LGX_RK_CLASS_LIST(LGX_RK_LAUNCH_ONE_##MODE##_##T)                                  \
    return cudaErrorInvalidValue;                                                      \
  }                                                                                    \
  }

#define LGX_RK_LAUNCH_BODY(T, MODE, A, B, C, D)                                        \
  if (la == A && lb == B && lc == C && ld == D) {                                      \
    auto k = rk_kernel<T, A, B, C, D, MODE>;                                           \
    int occ = 0;                                                                       \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, block, 0) != cudaSuccess || \
        occ < 1)                                                                       \
      occ = 1;                                                                         \
    long long grid = (long long)nsm * occ;                                             \
    const long long need = (work * a.group + block - 1) / block;                       \
    if (need < grid) grid = need < 1 ? 1 : need;                                       \
    k<<<(unsigned)grid, block, 0, st>>>(a);                                            \
    return cudaGetLastError();                                                         \
  }

#define LGX_RK_LAUNCH_ONE_kModeJK_double(A, B, C, D) LGX_RK_LAUNCH_BODY(double, kModeJK, A, B, C, D)
#define LGX_RK_LAUNCH_ONE_kModeStore_double(A, B, C, D) LGX_RK_LAUNCH_BODY(double, kModeStore, A, B, C, D)
#define LGX_RK_LAUNCH_ONE_kModeSchwarz_double(A, B, C, D) LGX_RK_LAUNCH_BODY(double, kModeSchwarz, A, B, C, D)
#define LGX_RK_LAUNCH_ONE_kModeJK_float(A, B, C, D) LGX_RK_LAUNCH_BODY(float, kModeJK, A, B, C, D)
#define LGX_RK_LAUNCH_ONE_kModeStore_float(A, B, C, D) LGX_RK_LAUNCH_BODY(float, kModeStore, A, B, C, D)
