// The device Boys evaluators as a batch call (lgx_boys): each thread
// evaluates F_0..F_mmax(T) of one argument with exactly the function a class
// kernel uses, so that the evaluators can be checked on their own.
#include "lgx_boys.cuh"
#include "lgx_warp.cuh"

namespace lgx {
namespace {

template <int MMAX>
__device__ void rk_boys_to(int variant, const double* tay, const float* tab32, double T,
                           double* out) {
  if (variant == 1) {
    rk_boys<MMAX>(tay, T, 1.0, out);
  } else if (variant == 5) {  // rk_prim_b64's FP64 evaluator, rounded as it does
    double f[MMAX + 1];
    dsf Td;
    Td.hi = float(T);
    Td.lo = float(T - double(Td.hi));
    rk_boys_b64<MMAX>(tay, Td, f);
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) out[m] = double(d2f_int(f[m]));
  } else {
    float f[MMAX + 1];
    rk_boys<MMAX>(tab32, float(T), 1.0f, f);
#pragma unroll
    for (int m = 0; m <= MMAX; ++m) out[m] = double(f[m]);
  }
}

// Variant 6: the whole Boys path of the mixed scheme's register kernels
// from primitive-pair data: the bins' double-float records of (Pb, zeta)
// and (Pk, eta), the FP32 prologue's rho and 1/(zeta + eta), the
// double-float argument (ds_boys_arg) and the FP64 evaluator rounded to FP32.
template <int MMAX>
__device__ void rk_boys_pairs(const double* tay, const double* pz, double* out) {
  const PrimPairJKds b = make_jkds(pz[0], pz[1], pz[2], pz[3]);
  const PrimPairJKds k = make_jkds(pz[4], pz[5], pz[6], pz[7]);
  const float zeta = b.hi.w, eta = k.hi.w;
  const float rs = rsqrtf(zeta + eta);
  const float oogpq = rs * rs;
  const float rho = zeta * eta * oogpq;
  double f[MMAX + 1];
  rk_boys_b64<MMAX>(tay, ds_boys_arg(b.hi, b.lo, k.hi, k.lo, rho, oogpq), f);
#pragma unroll
  for (int m = 0; m <= MMAX; ++m) out[m] = double(d2f_int(f[m]));
}

__global__ void boys_eval_kernel(const double* tab, const double* tay, const float* tab32,
                                 const double* inv_odd, int variant, const double* Targ,
                                 long long n, int mmax, double* F) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double out[kBoysMaxM + 1];
  if (variant == 6) {
    const double* pz = Targ + 8 * i;
    switch (mmax) {
      case 0: rk_boys_pairs<0>(tay, pz, out); break;
      case 1: rk_boys_pairs<1>(tay, pz, out); break;
      case 2: rk_boys_pairs<2>(tay, pz, out); break;
      case 3: rk_boys_pairs<3>(tay, pz, out); break;
      case 4: rk_boys_pairs<4>(tay, pz, out); break;
      case 5: rk_boys_pairs<5>(tay, pz, out); break;
      default: rk_boys_pairs<6>(tay, pz, out); break;
    }
    for (int m = 0; m <= mmax; ++m) F[i * (mmax + 1) + m] = out[m];
    return;
  }
  const double T = Targ[i];
  if (variant == 0) {
    boys_to_stage(tab, inv_odd, T, mmax, 1.0, out);
  } else if (variant == 2) {
    float f[kBoysMaxM + 1];
    boys_to_stage(tab32, float(T), mmax, 1.0f, f);
    for (int m = 0; m <= mmax; ++m) out[m] = double(f[m]);
  } else if (variant == 4) {  // the program kernels' mixed-scheme evaluator
    float f[kBoysMaxM + 1];
    dsf Td;
    Td.hi = float(T);
    Td.lo = float(T - double(Td.hi));
    boys_b64_stage(tay, inv_odd, Td, mmax, 1.0f, f);
    for (int m = 0; m <= mmax; ++m) out[m] = double(f[m]);
  } else {
    switch (mmax) {
      case 0: rk_boys_to<0>(variant, tay, tab32, T, out); break;
      case 1: rk_boys_to<1>(variant, tay, tab32, T, out); break;
      case 2: rk_boys_to<2>(variant, tay, tab32, T, out); break;
      case 3: rk_boys_to<3>(variant, tay, tab32, T, out); break;
      case 4: rk_boys_to<4>(variant, tay, tab32, T, out); break;
      case 5: rk_boys_to<5>(variant, tay, tab32, T, out); break;
      default: rk_boys_to<6>(variant, tay, tab32, T, out); break;
    }
  }
  for (int m = 0; m <= mmax; ++m) F[i * (mmax + 1) + m] = out[m];
}

}  // namespace

// variant: 0 program kernel FP64, 1 register kernel FP64 (mmax <= 6),
// 2 program kernel FP32, 3 register kernel FP32 (mmax <= 6), 4 and 5 the
// mixed scheme's FP64 evaluators of the program and register kernels
// (rounded to FP32), 6 the mixed register kernels' path from pair data (T holds 8
// values per argument: Pb.xyz, zeta, Pk.xyz, eta); the caller checks the
// ranges.
cudaError_t launch_boys_eval(const double* tab, const double* tay, const float* tab32,
                             const double* inv_odd, int variant, const double* T, long long n,
                             int mmax, double* F, cudaStream_t st) {
  const int block = 128;
  const long long grid = (n + block - 1) / block;
  boys_eval_kernel<<<(unsigned)grid, block, 0, st>>>(tab, tay, tab32, inv_odd, variant, T, n,
                                                     mmax, F);
  return cudaGetLastError();
}

}  // namespace lgx
