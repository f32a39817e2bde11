// Kernels of the ERI path other than the register kernels: the generic
// instances of the program kernel (lgx_warp.cuh), ShellPair precomputation,
// the J/K finalisation and the launchers used by lgx_api.cu.
#include "lgx_warp.cuh"

namespace lgx {

// ---------------------------------------------------------- pair kernel
// ShellPair::init for every pair (s1 >= s2) of the basis, one thread per
// primitive pair (shell.h:1138-1256, Original/Conservative screening).
__global__ void shellpair_kernel(DevBasis b, const PairRec* pairs, int npairs, PrimPairRec* pp,
                                 PrimPairJKds* ppds, const int* pp_pair, long long npp,
                                 double ln_prec, int method) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= npp) return;
  const int pi = pp_pair[t];
  const PairRec pr = pairs[pi];
  const int k = int(t - pr.pp_off);
  const int s1 = pr.s1, s2 = pr.s2;
  const int n2 = b.nprim[s2];
  const int p1 = k / n2, p2 = k % n2;
  const double a1 = b.alpha[b.prim_off[s1] + p1];
  const double a2 = b.alpha[b.prim_off[s2] + p2];
  const double c1 = b.coeff[b.prim_off[s1] + p1];
  const double c2 = b.coeff[b.prim_off[s2] + p2];
  double A[3], B[3], AB2 = 0;
  for (int x = 0; x < 3; ++x) {
    A[x] = b.O[3 * s1 + x];
    B[x] = b.O[3 * s2 + x];
    AB2 += (A[x] - B[x]) * (A[x] - B[x]);
  }
  // a pair of two unit shells (exponent 0, Shell::unit()) has no Gaussian
  // product; no braket uses it, so it is stored as a dropped pair
  const bool degenerate = !(a1 + a2 > 0.0);
  const double gamma = a1 + a2, oog = degenerate ? 0.0 : 1.0 / gamma;
  const double rho = a1 * a2 * oog;
  const double mrAB2 = -rho * AB2;
  double ln_scr = mrAB2 + log(fabs(c1)) + log(fabs(c2));
  PrimPairRec r;
  for (int x = 0; x < 3; ++x) r.P[x] = (AB2 == 0.0) ? A[x] : (a1 * A[x] + a2 * B[x]) * oog;
  double nonsph = 0;
  if (degenerate) ln_scr = -1.0e300;
  bool drop = degenerate || (method == 0 && ln_scr < ln_prec);
  if (method == 1) {
    double mPA = 0, mPB = 0;
    for (int x = 0; x < 3; ++x) {
      mPA = fmax(mPA, fabs(r.P[x] - A[x]));
      mPB = fmax(mPB, fabs(r.P[x] - B[x]));
    }
    const int l1 = b.l[s1], l2 = b.l[s2];
    // l! (l <= 4: the Cartesian raised shells of deriv 2 reach g)
    const double fl1 = l1 < 2 ? 1.0 : (l1 == 2 ? 2.0 : (l1 == 3 ? 6.0 : 24.0));
    const double fl2 = l2 < 2 ? 1.0 : (l2 == 2 ? 2.0 : (l2 == 3 ? 6.0 : 24.0));
    const double t1 = pow(mPA, l1) * pow(mPB, l2);
    const double t2 = fl1 * fl2 * pow(oog, l1 + l2);
    nonsph = fmax(t1, t2);
    ln_scr += 1.777485947591722872387900 + log(oog) + log(fmax(nonsph, 1.0)) +
              log(double(b.nprim[s1] * b.nprim[s2]));
    drop = degenerate || ln_scr < ln_prec;
  }
  r.Kc = degenerate ? 0.0 : 5.9149671727956128778 * exp(mrAB2) * oog * c1 * c2;
  r.oog = oog;
  r.zeta = gamma;
  r.a1 = a1;
  r.a2 = a2;
  r.ln_scr = drop ? -1.0e300 : ln_scr;
  r.fKc = float(r.Kc);
  r.fzeta = float(gamma);
  r.foog = float(oog);
  r.fln_scr = drop ? -3.0e38f : float(ln_scr);
  for (int x = 0; x < 3; ++x) {
    r.fPA1[x] = float(r.P[x] - A[x]);
    r.fPA2[x] = float(r.P[x] - B[x]);
  }
  r.fa1 = float(a1);
  r.fa2 = float(a2);
  r.fnonsph = float(nonsph);
  r.pad = 0.f;
  pp[t] = r;
  ppds[t] = make_jkds(r.P[0], r.P[1], r.P[2], gamma);
}

// FP32 J/K records: record r takes primitive pair src[r] & 0x7fffffff,
// oriented on its second centre when the sign bit is set.
__global__ void jk_records_kernel(const PrimPairRec* __restrict__ pp, const int* __restrict__ src,
                                  long long n, PrimPairJK32* __restrict__ out,
                                  PrimPairJKds* __restrict__ outds) {
  const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const unsigned v = unsigned(src[r]);
  const PrimPairRec& q = pp[v & 0x7fffffffu];
  const bool sw = (v >> 31) != 0;
  PrimPairJK32 o;
  o.k = make_float4(q.fKc, q.fzeta, q.foog, q.fln_scr);
  o.pa = sw ? make_float4(q.fPA2[0], q.fPA2[1], q.fPA2[2], q.fnonsph)
            : make_float4(q.fPA1[0], q.fPA1[1], q.fPA1[2], q.fnonsph);
  out[r] = o;
  outds[r] = make_jkds(q.P[0], q.P[1], q.P[2], q.zeta);
}

cudaError_t launch_jk_records(const PrimPairRec* pp, const int* src, long long n,
                              PrimPairJK32* out, PrimPairJKds* outds, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int block = 256;
  jk_records_kernel<<<(unsigned)((n + block - 1) / block), block, 0, st>>>(pp, src, n, out,
                                                                           outds);
  return cudaGetLastError();
}

// Infinity norms of the shell blocks of D (compute_shellblock_norm,
// tests/hartree-fock/hartree-fock++.cc:939-957): out[s1 * ns + s2] =
// max |D(i, j)| over the functions i of shell s1 and j of shell s2.
__global__ void shell_block_norm_kernel(DevBasis b, const double* __restrict__ D, int nbf,
                                        double* __restrict__ out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int ns = b.nshell;
  if (t >= (long long)ns * ns) return;
  const int s1 = int(t / ns), s2 = int(t - (long long)s1 * ns);
  const int o1 = b.bf_off[s1], o2 = b.bf_off[s2];
  const int n1 = b.pure[s1] ? 2 * b.l[s1] + 1 : ncart_of(b.l[s1]);
  const int n2 = b.pure[s2] ? 2 * b.l[s2] + 1 : ncart_of(b.l[s2]);
  double m = 0.0;
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n2; ++j) m = fmax(m, fabs(D[(size_t)(o1 + i) * nbf + o2 + j]));
  out[t] = m;
}

cudaError_t launch_shell_block_norm(const DevBasis& b, const double* D, int nbf, double* out,
                                    cudaStream_t st) {
  const long long n = (long long)b.nshell * b.nshell;
  if (n == 0) return cudaSuccess;
  const int block = 256;
  shell_block_norm_kernel<<<(unsigned)((n + block - 1) / block), block, 0, st>>>(b, D, nbf, out);
  return cudaGetLastError();
}

// J = (Jacc + Jacc^T)/4, K = (Kacc + Kacc^T)/8 (hartree-fock++.cc:1766 with
// the G = 2J - K split).
__global__ void jk_finalize_kernel(const double* Jacc, const double* Kacc, double* J, double* K,
                                   int nbf) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)nbf * nbf) return;
  const int i = int(t / nbf), j = int(t % nbf);
  J[t] = 0.25 * (Jacc[(size_t)i * nbf + j] + Jacc[(size_t)j * nbf + i]);
  K[t] = 0.125 * (Kacc[(size_t)i * nbf + j] + Kacc[(size_t)j * nbf + i]);
}

// ----------------------------------------------------------- launchers

cudaError_t launch_eri(const EriArgs& a, int mode, bool fp32, int grid, int block, size_t smem,
                       cudaStream_t st) {
  if (a.op != 0) {  // erf / erfc: the attenuated instantiations
    if (!fp32) {
      switch (mode) {
        case kModeStore: return launch_eri_t<double, kModeStore, PostInterpAtten>(a, grid, block, smem, st);
        case kModeSchwarz: return launch_eri_t<double, kModeSchwarz, PostInterpAtten>(a, grid, block, smem, st);
        case kModeJK: return launch_eri_t<double, kModeJK, PostInterpAtten>(a, grid, block, smem, st);
        case kModeGrad: return launch_eri_t<double, kModeGrad, PostInterpAtten>(a, grid, block, smem, st);
      }
    } else {
      switch (mode) {
        case kModeStore: return launch_eri_t<float, kModeStore, PostInterpAtten>(a, grid, block, smem, st);
        case kModeJK: return launch_eri_t<float, kModeJK, PostInterpAtten>(a, grid, block, smem, st);
      }
    }
    return cudaErrorInvalidValue;
  }
  if (!fp32) {
    switch (mode) {
      case kModeStore: return launch_eri_t<double, kModeStore>(a, grid, block, smem, st);
      case kModeSchwarz: return launch_eri_t<double, kModeSchwarz>(a, grid, block, smem, st);
      case kModeJK: return launch_eri_t<double, kModeJK>(a, grid, block, smem, st);
      case kModeGrad: return launch_eri_t<double, kModeGrad>(a, grid, block, smem, st);
    }
  } else {
    switch (mode) {
      case kModeStore: return launch_eri_t<float, kModeStore>(a, grid, block, smem, st);
      case kModeJK: return launch_eri_t<float, kModeJK>(a, grid, block, smem, st);
      case kModeStoreB64: return launch_eri_t<float, kModeStoreB64>(a, grid, block, smem, st);
      case kModeJKB64: return launch_eri_t<float, kModeJKB64>(a, grid, block, smem, st);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_shellpairs(const DevBasis& b, const PairRec* pairs, int npairs,
                              PrimPairRec* pp, PrimPairJKds* ppds, const int* pp_pair,
                              long long npp, double ln_prec, int method, cudaStream_t st) {
  if (npp == 0) return cudaSuccess;
  const int block = 256;
  const long long grid = (npp + block - 1) / block;
  shellpair_kernel<<<(unsigned)grid, block, 0, st>>>(b, pairs, npairs, pp, ppds, pp_pair, npp,
                                                     ln_prec, method);
  return cudaGetLastError();
}

// Drops the primitive pairs of one shell pair (n records) whose screening
// logarithm is below ln_prec: the pair table built at a tighter precision,
// cut to a caller's ShellPair data at ln_prec (shell.h:1138-1256).
__global__ void drop_pairs_kernel(PrimPairRec* pp, int n, double ln_prec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && pp[t].ln_scr < ln_prec) {
    pp[t].ln_scr = -1.0e300;
    pp[t].fln_scr = -3.0e38f;
  }
}

cudaError_t launch_drop_pairs(PrimPairRec* pp, int n, double ln_prec, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  drop_pairs_kernel<<<(n + 127) / 128, 128, 0, st>>>(pp, n, ln_prec);
  return cudaGetLastError();
}

cudaError_t launch_jk_finalize(const double* Jacc, const double* Kacc, double* J, double* K,
                               int nbf, cudaStream_t st) {
  const long long n = (long long)nbf * nbf;
  const int block = 256;
  jk_finalize_kernel<<<(unsigned)((n + block - 1) / block), block, 0, st>>>(Jacc, Kacc, J, K,
                                                                           nbf);
  return cudaGetLastError();
}

// Bytes of per-warp staging (rows primitive quartets + the factor table)
// for the program kernel in FP64 or FP32.
size_t stage_bytes_per_warp(bool fp32, int rows) {
  return size_t((rows * kStage + kKtab + 3) & ~3) * (fp32 ? sizeof(float) : sizeof(double));
}

__global__ void d2f_kernel(const double* src, float* dst, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) dst[t] = float(src[t]);
}

cudaError_t launch_d2f(const double* src, float* dst, long long n, cudaStream_t st) {
  const int block = 256;
  d2f_kernel<<<(unsigned)((n + block - 1) / block), block, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

// One contracted Cartesian shell set from caller-supplied primitive data
// (libint's generated per-quartet entry libint2_build_eri / _eri1: the
// caller fills the Libint_t prefactors and (00|00)^(m) of every primitive
// quartet, engine.impl.h:1389-1757, and the library contracts them,
// dg.cc:1177-1189).  The host packs the rows in the canonical orientation;
// the block stages them in batches of stage_rows (<= 32), runs the class's
// VRR program and post program with every level spread over all its
// threads, and stores the Cartesian sets in the caller's shell order, the
// derivative sets of centre C by translational invariance.
__global__ void __launch_bounds__(kBlockThreads) prim_set_kernel(PrimSetArgs a) {
  extern __shared__ double smem_d[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const DevProg& P = a.prog;
  const int R = a.stage_rows;
  const int stage_per = (R * kStage + kKtab + 3) & ~3;
  double* slots;
  if (a.warp_rows) {
    // warp w: stage at w * (stage_per + slot_stride), its accumulators after it;
    // rows w, w + nwarps, ... in batches of up to R per warp
    const int w = tid >> 5, lane = tid & 31, nw = nt >> 5;
    double* wstage = smem_d + size_t(w) * (stage_per + a.slot_stride);
    double* wslots = wstage + stage_per;
    for (int i = lane; i < P.nacc; i += 32) wslots[i] = 0.0;
    __syncwarp();
    const int mine = a.nrows > w ? (a.nrows - w + nw - 1) / nw : 0;  // rows of this warp
    for (int base = 0; base < mine; base += R) {
      const int n = min(R, mine - base);
      for (int i = lane; i < n * kStage; i += 32) {
        const int r = i / kStage, c = i - r * kStage;
        wstage[i] = a.rows[(size_t)(w + (base + r) * nw) * kStage + c];
      }
      __syncwarp();
      const unsigned ballot = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
      vrr_consume<double, WarpGrp>(P, wstage, ballot, wslots, wstage + R * kStage, lane);
      __syncwarp();
    }
    __syncthreads();
    slots = smem_d + stage_per;  // warp 0's accumulators receive the sum
    for (int i = tid; i < P.nacc; i += nt) {
      double v = slots[i];
      for (int u = 1; u < nw; ++u) v += smem_d[size_t(u) * (stage_per + a.slot_stride) + stage_per + i];
      slots[i] = v;
    }
    __syncthreads();
  } else {
    double* stage = smem_d;
    double* ktab = stage + R * kStage;
    slots = a.slots ? a.slots : smem_d + stage_per;
    for (int i = tid; i < P.nacc; i += nt) slots[i] = 0.0;
    __syncthreads();
    for (int base = 0; base < a.nrows; base += R) {
      const int n = min(R, a.nrows - base);
      const double* src = a.rows + (size_t)base * kStage;
      for (int i = tid; i < n * kStage; i += nt) stage[i] = src[i];
      __syncthreads();
      const unsigned ballot = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
      vrr_consume<double, BlockGrp>(P, stage, ballot, slots, ktab, tid);
      __syncthreads();
    }
  }
  QuartetGeom<double> g;
  for (int x = 0; x < 3; ++x) {
    g.AB[x] = a.AB[x];
    g.CD[x] = a.CD[x];
  }
  const int dims[4] = {ncart_of(P.la), ncart_of(P.lb), ncart_of(P.lc), ncart_of(P.ld)};
  int tn[4];
  for (int t = 0; t < 4; ++t) tn[a.perm[t]] = dims[t];
  const int n4 = P.ncart4;
  auto caller_index = [&](int e) {
    int ci[4];
    int r = e;
    ci[3] = r % dims[3]; r /= dims[3];
    ci[2] = r % dims[2]; r /= dims[2];
    ci[1] = r % dims[1]; ci[0] = r / dims[1];
    int it[4];
    for (int t = 0; t < 4; ++t) it[a.perm[t]] = ci[t];
    return ((it[0] * tn[1] + it[1]) * tn[2] + it[2]) * tn[3] + it[3];
  };
  for (int ph = 0; ph < P.nphases; ++ph) {
    run_post_phase<double, BlockGrp>(P, ph, g, slots, tid);
    const int ctr = P.deriv ? (ph == 0 ? 0 : (ph == 1 ? 1 : 3)) : 0;
    for (int s = 0; s < P.sets_per_phase; ++s) {
      const double* cart = slots + P.cart_out + s * n4;
      double* cb = slots + P.cbuf + s * n4;
      double* o = a.out + (size_t)(P.deriv ? a.perm[ctr] * 3 + s : 0) * n4;
      for (int e = tid; e < n4; e += nt) {
        o[caller_index(e)] = cart[e];
        if (P.deriv) cb[e] = (ph == 0 ? 0.0 : cb[e]) - cart[e];
      }
      __syncthreads();
      if (P.deriv && ph == P.nphases - 1) {
        double* oc = a.out + (size_t)(a.perm[2] * 3 + s) * n4;
        for (int e = tid; e < n4; e += nt) oc[caller_index(e)] = cb[e];
        __syncthreads();
      }
    }
  }
}

// Store mode for short explicit lists (a few quartets, e.g. one shell set
// or the raised / lowered quartets of a second-derivative set): one block
// per contracted quartet instead of one warp, so a single quartet's VRR
// and post-program levels, transform and store are spread over all the
// block's threads.  Warp 0 runs the primitive-quartet prologues (<= 32
// staged rows per batch, ballot-compacted as in the warp kernel).  FP64;
// ATT: attenuated operator.  Same output layout as eri_warp_kernel's store.
template <bool ATT>
__global__ void __launch_bounds__(kBlockThreads) eri_block_store_kernel(EriArgs a) {
  extern __shared__ double smem_d[];
  __shared__ unsigned s_ballot;
  __shared__ int s_kept;
  const int tid = threadIdx.x, nt = blockDim.x;
  const DevProg& P = a.prog;
  const int R = a.stage_rows;
  const int stage_per = (R * kStage + kKtab + 3) & ~3;
  double* stage = smem_d;
  double* ktab = stage + R * kStage;
  // warp_rows: warp w owns the shared-memory region w * (stage_per +
  // slot_stride) (its staging rows, then its accumulators); the post program
  // runs on warp 0's region after the accumulators are summed into it
  double* slots = a.global_slots
                      ? reinterpret_cast<double*>(a.gscratch) + size_t(blockIdx.x) * a.slot_stride
                      : smem_d + stage_per;
  const int w = tid >> 5, lane = tid & 31, nw = nt >> 5;
  double* wstage = smem_d + size_t(w) * (stage_per + a.slot_stride);
  double* wslots = wstage + stage_per;
  for (long long q = blockIdx.x; q < a.nitems; q += gridDim.x) {
    const QuartetItem it = a.items[q];
    QuartetGeom<double> g;
    load_geom<double>(a, it.bra_pair, it.ket_pair, it.flags & 1, (it.flags >> 1) & 1, g);
    const int nq = g.nbpp * g.nkpp;
    const double npbraket = double(nq);
    if (a.warp_rows) {
      for (int i = lane; i < P.nacc; i += 32) wslots[i] = 0.0;
      if (tid == 0) s_kept = 0;
      __syncthreads();
      const int mine = nq > w ? (nq - w + nw - 1) / nw : 0;  // primitive quartets w + k nw
      int kept_w = 0;
      for (int base = 0; base < mine; base += R) {
        bool keep = false;
        if (lane < R && base + lane < mine)
          keep = prologue<ATT>(a, g, w + (base + lane) * nw, npbraket, wstage + lane * kStage);
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        kept_w += __popc(b);
        __syncwarp();
        vrr_consume<double, WarpGrp>(P, wstage, b, wslots, wstage + R * kStage, lane);
        __syncwarp();
      }
      if (lane == 0) atomicAdd(&s_kept, kept_w);
      __syncthreads();
      for (int i = tid; i < P.nacc; i += nt) {
        double v = slots[i];
        for (int u = 1; u < nw; ++u) v += smem_d[size_t(u) * (stage_per + a.slot_stride) + stage_per + i];
        slots[i] = v;
      }
      __syncthreads();
    } else {
      for (int i = tid; i < P.nacc; i += nt) slots[i] = 0.0;
      if (tid == 0) s_kept = 0;
      __syncthreads();
      for (int base = 0; base < nq; base += R) {
        if (tid < 32) {
          bool keep = false;
          if (tid < R && base + tid < nq)
            keep = prologue<ATT>(a, g, base + tid, npbraket, stage + tid * kStage);
          const unsigned b = __ballot_sync(0xffffffffu, keep);
          if (tid == 0) {
            s_ballot = b;
            s_kept += __popc(b);
          }
        }
        __syncthreads();
        vrr_consume<double, BlockGrp>(P, stage, s_ballot, slots, ktab, tid);
        __syncthreads();
      }
    }
    const int kept = s_kept;
    if (a.is_null && tid == 0) a.is_null[it.pad] = kept == 0 ? 1 : 0;
    if (kept == 0) continue;  // block-uniform
    const int lsh[4] = {P.la, P.lb, P.lc, P.ld};
    int pure[4];
    for (int t = 0; t < 4; ++t) pure[t] = a.basis.pure[g.sh[t]];
    const int fl = it.flags >> 2;
    const bool sbk = fl & 1, stb = (fl >> 1) & 1, stk = (fl >> 2) & 1;
    int perm[4];
    perm[0] = sbk ? (stk ? 3 : 2) : (stb ? 1 : 0);
    perm[1] = sbk ? (stk ? 2 : 3) : (stb ? 0 : 1);
    perm[2] = sbk ? (stb ? 1 : 0) : (stk ? 3 : 2);
    perm[3] = sbk ? (stb ? 0 : 1) : (stk ? 2 : 3);
    for (int ph = 0; ph < P.nphases; ++ph) {
      run_post_phase<double, BlockGrp>(P, ph, g, slots, tid);
      const int ctr = P.deriv ? (ph == 0 ? 0 : (ph == 1 ? 1 : 3)) : 0;
      for (int s = 0; s < P.sets_per_phase; ++s) {
        int dims[4] = {ncart_of(P.la), ncart_of(P.lb), ncart_of(P.lc), ncart_of(P.ld)};
        double* cart = slots + P.cart_out + s * P.ncart4;
        const double* V =
            sph_transform<double, BlockGrp>(a, lsh, pure, dims, cart, slots + P.sph_tmp, tid);
        const int nsph4 = dims[0] * dims[1] * dims[2] * dims[3];
        int tn[4];
        for (int t = 0; t < 4; ++t) tn[perm[t]] = dims[t];
        auto caller_index = [&](int e) {
          int ci[4];
          int r = e;
          ci[3] = r % dims[3]; r /= dims[3];
          ci[2] = r % dims[2]; r /= dims[2];
          ci[1] = r % dims[1]; ci[0] = r / dims[1];
          int ix[4];
          for (int t = 0; t < 4; ++t) ix[perm[t]] = ci[t];
          return ((ix[0] * tn[1] + ix[1]) * tn[2] + ix[2]) * tn[3] + ix[3];
        };
        const int ts = P.deriv ? perm[ctr] * 3 + s : 0;
        double* o = a.out + it.out + (size_t)ts * nsph4;
        double* cb = slots + P.cbuf + s * P.ncart4;
        for (int e = tid; e < nsph4; e += nt) {
          o[caller_index(e)] = V[e];
          if (P.deriv) cb[e] = (ph == 0 ? 0.0 : cb[e]) - V[e];
        }
        __syncthreads();
        if (P.deriv && ph == P.nphases - 1) {
          double* oc = a.out + it.out + (size_t)(perm[2] * 3 + s) * nsph4;
          for (int e = tid; e < nsph4; e += nt) oc[caller_index(e)] = cb[e];
        }
        __syncthreads();
      }
    }
  }
}

cudaError_t launch_eri_block_store(const EriArgs& a, int grid, size_t smem, cudaStream_t st) {
  auto k = a.op != 0 ? eri_block_store_kernel<true> : eri_block_store_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, kBlockThreads, smem, st>>>(a);
  return cudaGetLastError();
}

// One block of kBlockThreads; smem = staging (stage_bytes_per_warp) + the
// slots when they live in shared memory (a.slots == nullptr).
cudaError_t launch_prim_set(const PrimSetArgs& a, size_t smem, cudaStream_t st) {
  cudaError_t e =
      cudaFuncSetAttribute(prim_set_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  prim_set_kernel<<<1, kBlockThreads, smem, st>>>(a);
  return cudaGetLastError();
}


int eri_blocks_per_sm(int mode, bool fp32, int block, size_t smem) {
  if (!fp32) {
    switch (mode) {
      case kModeStore: return occ_t<double, kModeStore>(block, smem);
      case kModeSchwarz: return occ_t<double, kModeSchwarz>(block, smem);
      case kModeJK: return occ_t<double, kModeJK>(block, smem);
      case kModeGrad: return occ_t<double, kModeGrad>(block, smem);
    }
  } else {
    switch (mode) {
      case kModeStore: return occ_t<float, kModeStore>(block, smem);
      case kModeJK: return occ_t<float, kModeJK>(block, smem);
      case kModeStoreB64: return occ_t<float, kModeStoreB64>(block, smem);
      case kModeJKB64: return occ_t<float, kModeJKB64>(block, smem);
    }
  }
  return 1;
}

}  // namespace lgx
