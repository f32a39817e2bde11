// C ABI of liblgx (include/lgx.h): contexts, basis and shell-pair state,
// class programs, launch configuration and the batched / J/K passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_kernels.cuh"
#include "lgx_program.h"

namespace lgx {
cudaError_t launch_eri(const EriArgs& a, int mode, bool fp32, int grid, int block,
                       size_t smem, cudaStream_t st);
cudaError_t launch_shellpairs(const DevBasis& b, const PairRec* pairs, int npairs,
                              PrimPairRec* pp, PrimPairJKds* ppds, const int* pp_pair,
                              long long npp, double ln_prec, int method, cudaStream_t st);
cudaError_t launch_jk_finalize(const double* Jacc, const double* Kacc, double* J,
                               double* K, int nbf, cudaStream_t st);
cudaError_t launch_drop_pairs(PrimPairRec* pp, int n, double ln_prec, cudaStream_t st);
size_t stage_bytes_per_warp(bool fp32, int rows);
int eri_blocks_per_sm(int mode, bool fp32, int block, size_t smem);
cudaError_t launch_d2f(const double* src, float* dst, long long n, cudaStream_t st);
cudaError_t launch_shell_block_norm(const DevBasis& b, const double* D, int nbf, double* out,
                                    cudaStream_t st);
cudaError_t launch_boys_eval(const double* tab, const double* tay, const float* tab32,
                             const double* inv_odd, int variant, const double* T, long long n,
                             int mmax, double* F, cudaStream_t st);
cudaError_t launch_prim_set(const PrimSetArgs& a, size_t smem, cudaStream_t st);
cudaError_t launch_eri_block_store(const EriArgs& a, int grid, size_t smem, cudaStream_t st);
cudaError_t rk_launch(bool fp32, int mode, bool att, int la, int lb, int lc, int ld, const EriArgs& a,
                      long long work, int nsm, cudaStream_t st);
bool rk_available(bool fp32, int mode, bool att, int la, int lb, int lc, int ld);
cudaError_t launch_jk_records(const PrimPairRec* pp, const int* src, long long n,
                              PrimPairJK32* out, PrimPairJKds* outds, cudaStream_t st);
cudaError_t post_launch(bool fp32, int mode, int la, int lb, int lc, int ld, const EriArgs& a,
                        int grid, int block, size_t smem, cudaStream_t st);
int post_blocks_per_sm(bool fp32, int mode, int la, int lb, int lc, int ld, int block,
                       size_t smem);
bool post_info(int la, int lb, int lc, int ld, int* nacc, int* slots);
}  // namespace lgx

using namespace lgx;

namespace {

const char* kVersion = "lgx 0.1 (sm_103a)";

struct DBuf {
  void* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
    if (e == cudaSuccess) n = std::max<size_t>(bytes, 256);
    return e;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};


struct ProgDev {
  ClassProgramHost host;
  DevProg dev;
  DBuf buf;
};

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
inline int nfunc(int l, int pure) { return pure ? 2 * l + 1 : ncart(l); }
inline long long pidx(int s1, int s2) {  // s1 >= s2
  return (long long)s1 * (s1 + 1) / 2 + s2;
}

struct BasisDev {
  int nshell = 0, nprim_total = 0, nbf = 0, natoms = 0;
  std::vector<int> l, pure, nprim, prim_off, bf_off, atom;
  std::vector<double> O, alpha, coeff;
  DBuf ints, dbls, flts;
  DevBasis dev{};
  // pairs
  std::vector<PairRec> hpairs;
  std::vector<unsigned char> hswap;
  long long npp = 0;
  DBuf pairs, pprims, ppds, pp_pair, pair_swap;
  bool pairs_ok = false;
  unsigned long long pairs_version = 0;  // bumped whenever pprims is rewritten
  double pairs_lnprec = 0;
  int pairs_method = -1;
  // Schwarz
  std::vector<double> Kpair;  // per pair index
  DBuf Kd;                    // Kpair on the device
  bool schwarz_ok = false;
  bool std_pure = true;  // every shell has pure == (l >= 2)
  double avg_npp = 1;    // mean primitive pairs per shell pair
};

struct BinHost {
  double nq_avg = 1;  // mean primitive quartets per shell quartet (unscreened)
  int cls;  // class index
  int la, lb, lc, ld;
  int bra_class, ket_class;
  long long total[2];   // [0] FP64 space, [1] FP32 space
  long long integrals[2];
  double last_ms[2] = {0, 0};  // device time of the space's launch in the last pass
  DBuf seg_start[2], seg_bra[2], seg_j0[2];
  int nseg[2];
};

struct BinCache {
  bool valid = false;
  double thresh = -1, mixed = -1;
  int mode = -1;
  unsigned long long subset_version = ~0ull;  // pair subset the bins were built for
  DBuf class_lists;                 // pair ids of every pair class, sorted
  std::vector<long long> class_off; // offsets of each class in class_lists
  // FP32 records per list position (PrimPairJK32 layout) and their source
  DBuf rec_idx, rec_src, recs, recsds;
  long long nrec = 0;
  unsigned long long rec_version = ~0ull;  // pairs_version the records hold
  std::vector<std::unique_ptr<BinHost>> bins;
  long long quartets[2] = {0, 0};
};

}  // namespace

// Launch variant of one class bin: the register kernel with G lanes per
// quartet, or the program kernel with interpreted or generated post stage
// and R staging rows.
struct Variant {
  int kind = 0;   // 0 register kernel, 1 program kernel, 2 program kernel + generated post
  int group = 1;  // register kernel: lanes per quartet
  int rows = 0;   // program kernel: staging rows (0: from the contraction depth)
};

// Launch record of one enqueued pass (kept with a captured pass graph).
struct PassRec {
  int bin, sp;
  bool fp32;
  Variant v;
  int mode;  // kernel mode of the launch
};
struct PassRecs {
  std::vector<PassRec> recs;
  long long integrals = 0, launches = 0;
  size_t nslots = 0;
  bool count = false;
  bool timed = false;  // per-launch events were recorded (ctx->lev)
  bool split = false;  // FP64 / FP32 launches on parallel streams
};

// Identity of a captured J/K pass: every pointer and setting its nodes use.
struct PassKey {
  const void* ptr[9] = {};
  double thresh = 0, mixed = 0;
  int mode = -1;
  unsigned long long version = 0;
  bool operator==(const PassKey& o) const {
    for (int i = 0; i < 9; ++i)
      if (ptr[i] != o.ptr[i]) return false;
    return thresh == o.thresh && mixed == o.mixed && mode == o.mode && version == o.version;
  }
};

struct lgx_context {
  int device = 0;
  int nsm = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  std::string err;
  DBuf boys, boys_tay, boys32, sph_off, sph_c, sph_cd, sph_cf, Df, inv_odd;
  std::map<int, std::unique_ptr<ProgDev>> progs;
  bool use_rk = true;  // register kernels for the small classes
  bool use_post = true;  // generated post stages for the large J/K classes
  bool tune = true;      // per-class launch-shape tuning on the first pass
  long long tune_min = 4096;  // bins with fewer quartets keep the default variant
  // tuned launch variant per (class, deriv, mode, precision)
  std::map<int, struct Variant> tuned;
  DBuf tuneJ, tuneK;
  // captured J/K pass (replayed while its key matches) and its records
  bool use_graphs = true;
  unsigned long long version = 0;  // bumped when bins, tuning or basis change
  cudaGraphExec_t jk_exec = nullptr;
  PassKey jk_key;
  PassRecs jk_recs;
  // mixed passes: the FP64 and the FP32 class launches run on two streams
  // forked from and joined back into `stream` (parallel branches of the
  // captured pass), so that FP32 launches use the issue slots that the
  // FP64-pipe-bound launches leave idle; FP64 launches then hold at most
  // fp64_bps blocks per SM (0: no cap).  `launch_stream` / `scratch` are
  // the stream and the program-kernel slot scratch of the launch being
  // enqueued (the FP32 branch has its own scratch).
  static constexpr int kMaxBranches = 4;  // streams per precision
  bool overlap = true;
  int branches = 3;
  // 0: longest first onto the least-loaded branch, issued longest first;
  // 1: round-robin in bin order (default: best or level on (H2O)32 cc-pVDZ,
  // (H2O)8 and (H2O)64 cc-pVTZ); 2: as 0 but issued in bin order
  int branch_policy = 1;
  int fp64_bps = 0;
  int fp32_bps = 0;  // as fp64_bps, for the FP32 launches of a mixed pass
  cudaStream_t s64[kMaxBranches] = {}, s32[kMaxBranches] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[2 * kMaxBranches] = {};
  cudaStream_t launch_stream = nullptr;
  DBuf gscratch_br[2 * kMaxBranches];  // program-kernel slot scratch per branch
  DBuf* scratch = nullptr;
  // identity of the branch scratch buffers (their addresses enter a
  // captured pass): changes whenever one of them is reallocated
  const void* scratch_sig() const {
    unsigned long long h = 1469598103934665603ull;
    for (const auto& b : gscratch_br) h = (h ^ reinterpret_cast<uintptr_t>(b.p)) * 1099511628211ull;
    return reinterpret_cast<const void*>(uintptr_t(h));
  }
  // per-launch timing events of the batched passes (a start and an end
  // event around each class launch, on the launch's stream; inside a
  // captured pass they are event-record nodes) and the per-launch
  // statistics of the last pass
  std::vector<cudaEvent_t> lev;
  std::vector<lgx_launch_stats> last_launches;
  bool noalloc = false;  // set during lgx_jk_device_noalloc: no device allocation
  // work chunks a program-kernel warp may take per launch before it raises
  // the watchdog flag (< 0: derived from the launch's work; lgx_set_watchdog)
  long long watchdog_chunks = -1;
  // shell pairs a J/K pass is restricted to (lgx_set_pair_subset; one flag
  // per pair index, empty: every pair) and a version bumped on each change
  std::vector<unsigned char> pair_subset;
  unsigned long long subset_version = 0;
  // density-weighted screening of the J/K passes (lgx_set_fock_precision):
  // Fock precision (0: off) and the shell-block norms of D it uses
  double fock_prec = 0.0;
  DBuf Dsh;
  // two-body operator of every pass (lgx_set_operator): LGX_OP_* and omega
  int op = LGX_OP_COULOMB;
  double omega = 0.0;
  BasisDev basis, small;
  DBuf gscratch, counter, errflag, primcount;
  DBuf items, out, isnull;
  DBuf Jacc, Kacc, Dd, Jd, Kd, gJ, gK;
  DBuf prim_rows, prim_slots;  // lgx_compute_primitive_set
  DBuf boysT, boysF;           // lgx_boys
  DBuf xcounters;              // explicit lists: one work counter per class launch
  BinCache bins;
  std::mutex mu;
};

namespace {

lgx_status fail(lgx_context* c, lgx_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}
#define CK(expr)                                                              \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return fail(ctx, LGX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Precision modes (LGX_FP64, LGX_MIXED, LGX_MIXED_FP32_BOYS): whether a pass
// splits off an FP32 space, and the kernel mode of its FP32 launches.  The
// mixed scheme's FP32 kernels evaluate the Boys function in FP64 for the
// Coulomb operator; the attenuated operators' FP32 kernels keep it in FP32.
bool mixed_mode(int mode) { return mode == LGX_MIXED || mode == LGX_MIXED_FP32_BOYS; }
bool valid_mode(int mode) { return mode == LGX_FP64 || mixed_mode(mode); }
int fp32_kernel_mode(const lgx_context* ctx, int mode, int base_mode) {
  if (!mixed_mode(mode)) return -1;
  const bool b64 = mode == LGX_MIXED && ctx->op == LGX_OP_COULOMB;
  if (base_mode == kModeJK) return b64 ? kModeJKB64 : kModeJK;
  return b64 ? kModeStoreB64 : kModeStore;
}

// ------------------------------------------------------- host constants
// Boys table: F_m(k/64), m < kBoysCols, from the Maclaurin series (top m)
// and downward recursion in long double.
std::vector<double> make_boys_table() {
  std::vector<double> t(size_t(kBoysRows) * kBoysCols);
  for (int k = 0; k < kBoysRows; ++k) {
    const long double T = (long double)k * kBoysDT;
    const int M = kBoysCols - 1;
    long double term = 1.0L / (2 * M + 1), sum = term;
    for (int i = 1; i < 4000; ++i) {
      term *= 2 * T / (2 * M + 2 * i + 1);
      sum += term;
      if (term < sum * 1e-22L) break;
    }
    const long double eT = expl(-T);
    long double f = eT * sum;
    t[size_t(k) * kBoysCols + M] = (double)f;
    for (int m = M - 1; m >= 0; --m) {
      f = (2 * T * f + eT) / (2 * m + 1);
      t[size_t(k) * kBoysCols + m] = (double)f;
    }
  }
  return t;
}

double fac(int n) {
  double r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}
double dfac(int n) {
  double r = 1;
  for (int i = n; i > 1; i -= 2) r *= i;
  return r;
}
double binom(int n, int k) { return (k < 0 || k > n) ? 0.0 : fac(n) / (fac(k) * fac(n - k)); }
int par(int k) { return (k % 2) ? -1 : 1; }

// Real solid harmonics in Cartesian Gaussians sharing the x^l normalization
// (Schlegel & Frisch, IJQC 54, 83 (1995), eq. 15; the coefficient set of
// SolidHarmonicsCoefficients::coeff, solidharmonics.h:114-174).
double solid_coeff(int l, int m, int lx, int ly, int lz) {
  const int am = std::abs(m);
  if ((lx + ly - am) % 2) return 0.0;
  const int j = (lx + ly - am) / 2;
  if (j < 0) return 0.0;
  const int i = am - lx;
  if ((m >= 0) != (std::abs(i) % 2 == 0)) return 0.0;
  double pf = std::sqrt(fac(2 * lx) * fac(2 * ly) * fac(2 * lz) / fac(2 * l) * fac(l - am) /
                        fac(l) / fac(l + am) / (fac(lx) * fac(ly) * fac(lz)));
  pf /= double(1 << l);
  pf *= (m < 0) ? par((i - 1) / 2) : par(i / 2);
  double sum = 0;
  for (int ii = j; ii <= (l - am) / 2; ++ii) {
    const double t = binom(l, ii) * binom(ii, j) * par(ii) * fac(2 * (l - ii)) /
                     fac(l - am - 2 * ii);
    double s1 = 0;
    for (int k = 0; k <= std::min(j, lx / 2); ++k)
      if (lx - 2 * k <= am) s1 += binom(j, k) * binom(am, lx - 2 * k) * par(k);
    sum += t * s1;
  }
  sum *= std::sqrt(dfac(2 * l - 1) / (dfac(2 * lx - 1) * dfac(2 * ly - 1) * dfac(2 * lz - 1)));
  return m == 0 ? pf * sum : M_SQRT2 * pf * sum;
}

std::vector<double> make_sph_table() {
  std::vector<double> t(110, 0.0);
  for (int l = 0; l <= 3; ++l) {
    const int nc = ncart(l);
    for (int p = 0; p < 2 * l + 1; ++p) {
      int c = 0;
      for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly, ++c)
          t[sph_off(l) + p * nc + c] = solid_coeff(l, p - l, lx, ly, l - lx - ly);
    }
  }
  return t;
}

// ------------------------------------------------------------ programs
lgx_status get_prog(lgx_context* ctx, int la, int lb, int lc, int ld, int deriv,
                    ProgDev** out) {
  const int ci = class_index(la, lb, lc, ld);
  if (ci < 0) return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "angular momentum beyond LGX_MAX_L");
  const int key = ci * 2 + deriv;
  auto it = ctx->progs.find(key);
  if (it != ctx->progs.end()) {
    *out = it->second.get();
    return LGX_OK;
  }
  if (ctx->noalloc)
    return fail(ctx, LGX_ERR_INVALID_ARG,
                "class program not prepared: call lgx_jk_device once with the same settings");
  auto pd = std::make_unique<ProgDev>();
  try {
    pd->host = build_class_program(la, lb, lc, ld, deriv);
  } catch (const std::exception& e) {
    return fail(ctx, LGX_ERR_INVALID_ARG, e.what());
  }
  const auto& H = pd->host;
  // layout: [ints: vrr_lev, acc_lev, post_lev, phase_lev] [pad16] [vrr_ops] [acc_ops] [pad16] [post_ops]
  std::vector<uint32_t> blob;
  auto pad16 = [&]() {
    while (blob.size() % 4) blob.push_back(0);
  };
  const size_t o_vlev = blob.size();
  for (int v : H.vrr_lev) blob.push_back(uint32_t(v));
  const size_t o_alev = blob.size();
  for (int v : H.acc_lev) blob.push_back(uint32_t(v));
  const size_t o_plev = blob.size();
  for (int v : H.post_lev) blob.push_back(uint32_t(v));
  const size_t o_phlev = blob.size();
  for (int v : H.phase_lev) blob.push_back(uint32_t(v));
  pad16();
  // 16-bit slot indices when every slot fits (halves the op stream)
  const bool compact = H.total_slots() < 65536;
  const size_t o_vops = blob.size();
  if (compact) {
    for (size_t i = 0; i < H.vrr_ops.size(); i += 8) {
      const uint32_t* w = &H.vrr_ops[i];
      blob.push_back(w[0] | (w[1] << 16));
      blob.push_back(w[2] | (w[3] << 16));
      blob.push_back(w[4] | (w[5] << 16));
      blob.push_back(w[6]);
    }
  } else {
    blob.insert(blob.end(), H.vrr_ops.begin(), H.vrr_ops.end());
  }
  pad16();
  const size_t o_aops = blob.size();
  blob.insert(blob.end(), H.acc_ops.begin(), H.acc_ops.end());
  pad16();
  const size_t o_pops = blob.size();
  if (compact) {
    for (size_t i = 0; i < H.post_ops.size(); i += 4) {
      const uint32_t* w = &H.post_ops[i];
      if (w[3] > 0xFFFFu) return fail(ctx, LGX_ERR_INVALID_ARG, "post op word out of range");
      blob.push_back(w[0] | (w[1] << 16));
      blob.push_back(w[2] | (w[3] << 16));
    }
  } else {
    blob.insert(blob.end(), H.post_ops.begin(), H.post_ops.end());
  }
  pad16();
  CK(pd->buf.ensure(blob.size() * 4));
  CK(cudaMemcpyAsync(pd->buf.p, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const uint32_t* base = pd->buf.as<uint32_t>();
  DevProg& D = pd->dev;
  D.la = la; D.lb = lb; D.lc = lc; D.ld = ld; D.deriv = deriv; D.mmax = H.mmax;
  D.nacc = H.nacc; D.nwork = H.nwork; D.leaf_slot0 = H.leaf_slot0;
  D.nphases = H.nphases; D.sets_per_phase = H.sets_per_phase; D.ncart4 = H.ncart4;
  D.cart_out = H.cart_out; D.cbuf = H.cbuf; D.sph_tmp = H.sph_tmp;
  D.nlev = int(H.vrr_lev.size()) - 1;
  D.npost_lev = int(H.post_lev.size()) - 1;
  D.vrr_lev = reinterpret_cast<const int*>(base + o_vlev);
  D.acc_lev = reinterpret_cast<const int*>(base + o_alev);
  D.post_lev = reinterpret_cast<const int*>(base + o_plev);
  D.phase_lev = reinterpret_cast<const int*>(base + o_phlev);
  D.compact = compact ? 1 : 0;
  D.vrr_ops = reinterpret_cast<const uint4*>(base + o_vops);
  D.acc_ops = reinterpret_cast<const uint2*>(base + o_aops);
  D.post_ops = reinterpret_cast<const uint4*>(base + o_pops);
  D.post_ops_c = reinterpret_cast<const uint2*>(base + o_pops);
  *out = pd.get();
  ctx->progs.emplace(key, std::move(pd));
  return LGX_OK;
}

// ---------------------------------------------------------------- basis
// lmax: LGX_MAX_L for callers' bases; one more for the Cartesian raised
// shells of the second-derivative composition.
lgx_status upload_basis(lgx_context* ctx, BasisDev& B, int nshell, const int32_t* l,
                        const int32_t* pure, const int32_t* nprim, const int32_t* atom,
                        const double* origins, const double* alpha, const double* coeff,
                        int lmax = kMaxL) {
  if (nshell <= 0 || !l || !pure || !nprim || !origins || !alpha || !coeff)
    return fail(ctx, LGX_ERR_INVALID_ARG, "lgx_set_basis: null array or empty basis");
  B.nshell = nshell;
  B.l.assign(l, l + nshell);
  B.pure.assign(pure, pure + nshell);
  B.nprim.assign(nprim, nprim + nshell);
  B.atom.assign(nshell, 0);
  if (atom) B.atom.assign(atom, atom + nshell);
  B.prim_off.resize(nshell);
  B.bf_off.resize(nshell);
  int np = 0, nbf = 0, natoms = 0;
  for (int s = 0; s < nshell; ++s) {
    if (l[s] < 0 || l[s] > lmax || (pure[s] && l[s] > kMaxL))
      return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "shell angular momentum exceeds LGX_MAX_L");
    if (nprim[s] <= 0 || nprim[s] > kMaxNprim)
      return fail(ctx, LGX_ERR_TOO_LARGE, "shell contraction depth exceeds LGX_MAX_NPRIM");
    if (B.atom[s] < 0) return fail(ctx, LGX_ERR_INVALID_ARG, "negative atom index");
    B.prim_off[s] = np;
    B.bf_off[s] = nbf;
    np += nprim[s];
    nbf += nfunc(l[s], pure[s]);
    natoms = std::max(natoms, B.atom[s] + 1);
  }
  B.nprim_total = np;
  B.nbf = nbf;
  B.natoms = natoms;
  B.std_pure = true;
  for (int s = 0; s < nshell; ++s)
    if ((pure[s] != 0) != (l[s] >= 2)) B.std_pure = false;
  B.O.assign(origins, origins + 3 * nshell);
  B.alpha.assign(alpha, alpha + np);
  B.coeff.assign(coeff, coeff + np);
  // device copies: ints [l|pure|nprim|prim_off|bf_off|atom], doubles [O|alpha|coeff]
  std::vector<int> hi;
  hi.reserve(6 * nshell);
  for (auto* v : {&B.l, &B.pure, &B.nprim, &B.prim_off, &B.bf_off, &B.atom})
    hi.insert(hi.end(), v->begin(), v->end());
  std::vector<double> hd;
  hd.reserve(3 * nshell + 2 * np);
  hd.insert(hd.end(), B.O.begin(), B.O.end());
  hd.insert(hd.end(), B.alpha.begin(), B.alpha.end());
  hd.insert(hd.end(), B.coeff.begin(), B.coeff.end());
  CK(B.ints.ensure(hi.size() * sizeof(int)));
  CK(B.dbls.ensure(hd.size() * sizeof(double)));
  CK(cudaMemcpyAsync(B.ints.p, hi.data(), hi.size() * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(B.dbls.p, hd.data(), hd.size() * sizeof(double), cudaMemcpyHostToDevice,
                     ctx->stream));
  const int* ib = B.ints.as<int>();
  const double* db = B.dbls.as<double>();
  B.dev.nshell = nshell;
  B.dev.l = ib;
  B.dev.pure = ib + nshell;
  B.dev.nprim = ib + 2 * nshell;
  B.dev.prim_off = ib + 3 * nshell;
  B.dev.bf_off = ib + 4 * nshell;
  B.dev.atom = ib + 5 * nshell;
  B.dev.O = db;
  B.dev.alpha = db + 3 * nshell;
  B.dev.coeff = db + 3 * nshell + np;
  {
    std::vector<float> hf(6 * size_t(nshell));
    for (int i = 0; i < 3 * nshell; ++i) {
      const float hi = float(B.O[i]);
      hf[i] = hi;
      hf[3 * nshell + i] = float(B.O[i] - double(hi));
    }
    CK(B.flts.ensure(hf.size() * sizeof(float)));
    CK(cudaMemcpyAsync(B.flts.p, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice,
                       ctx->stream));
    B.dev.Ohi = B.flts.as<float>();
    B.dev.Olo = B.flts.as<float>() + 3 * nshell;
  }
  B.pairs_ok = false;
  B.schwarz_ok = false;
  // pair table layout (all s1 >= s2)
  const long long npairs = (long long)nshell * (nshell + 1) / 2;
  B.hpairs.resize(npairs);
  B.hswap.resize(npairs);
  long long off = 0;
  for (int s1 = 0; s1 < nshell; ++s1)
    for (int s2 = 0; s2 <= s1; ++s2) {
      PairRec& r = B.hpairs[pidx(s1, s2)];
      r.s1 = s1;
      r.s2 = s2;
      r.pp_off = int(off);
      r.npp = nprim[s1] * nprim[s2];
      off += r.npp;
      B.hswap[pidx(s1, s2)] = (l[s2] > l[s1]) ? 1 : 0;
    }
  if (off > std::numeric_limits<int>::max())
    return fail(ctx, LGX_ERR_TOO_LARGE, "too many primitive pairs");
  B.npp = off;
  std::vector<int> ppp(off);
  for (long long p = 0; p < npairs; ++p)
    for (int k = 0; k < B.hpairs[p].npp; ++k) ppp[B.hpairs[p].pp_off + k] = int(p);
  CK(B.pairs.ensure(npairs * sizeof(PairRec)));
  CK(B.pp_pair.ensure(off * sizeof(int)));
  CK(B.pprims.ensure(off * sizeof(PrimPairRec)));
  CK(B.ppds.ensure(off * sizeof(PrimPairJKds)));
  CK(B.pair_swap.ensure(npairs));
  CK(cudaMemcpyAsync(B.pairs.p, B.hpairs.data(), npairs * sizeof(PairRec),
                     cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(B.pp_pair.p, ppp.data(), off * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(B.pair_swap.p, B.hswap.data(), npairs, cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LGX_OK;
}

// FP32 J/K records of the current bins from the current primitive pairs.
lgx_status ensure_jk_records(lgx_context* ctx, BasisDev& B) {
  BinCache& C = ctx->bins;
  if (C.rec_version == B.pairs_version) return LGX_OK;
  CK(launch_jk_records(B.pprims.as<PrimPairRec>(), C.rec_src.as<int>(), C.nrec,
                       C.recs.as<PrimPairJK32>(), C.recsds.as<PrimPairJKds>(), ctx->stream));
  C.rec_version = B.pairs_version;
  return LGX_OK;
}

lgx_status ensure_pairs(lgx_context* ctx, BasisDev& B, double ln_prec, int method) {
  if (B.pairs_ok && B.pairs_lnprec == ln_prec && B.pairs_method == method) return LGX_OK;
  CK(launch_shellpairs(B.dev, B.pairs.as<PairRec>(), int(B.hpairs.size()),
                       B.pprims.as<PrimPairRec>(), B.ppds.as<PrimPairJKds>(),
                       B.pp_pair.as<int>(), B.npp, ln_prec, method, ctx->stream));
  B.pairs_ok = true;
  ++B.pairs_version;
  B.pairs_lnprec = ln_prec;
  B.pairs_method = method;
  return LGX_OK;
}

// ------------------------------------------------------ launch helpers
struct Launch {
  int grid, block, wpb, stride, rows;
  size_t smem;
  bool global;
};

// Program-kernel launch shape: staging rows (primitive quartets prepared per
// batch; a few suffice for the nearly uncontracted high-L classes and leave
// shared memory to more resident warps) and warps per block, chosen for the
// most resident warps per SM; rows_hint > 0 forces the row count.
lgx_status plan_launch(lgx_context* ctx, const ProgDev& P, int mode, bool fp32,
                       long long nwork, double nq_avg, int rows_hint, bool gen, Launch& L) {
  const size_t elt = fp32 ? 4 : 8;
  L.stride = (P.host.total_slots() + 1) & ~1;
  if (gen) {  // accumulators + VRR work, or accumulators + generated post regions
    int nacc = 0, slots = 0;
    post_info(P.host.la, P.host.lb, P.host.lc, P.host.ld, &nacc, &slots);
    if (nacc != P.host.nacc)
      return fail(ctx, LGX_ERR_INVALID_ARG, "generated post stage does not match the class program");
    L.stride = (std::max(P.host.nacc + P.host.vrr_work, slots) + 1) & ~1;
  }
  auto occupancy = [&](int block, size_t smem) {
    return gen ? post_blocks_per_sm(fp32, mode, P.host.la, P.host.lb, P.host.lc, P.host.ld, block,
                                    smem)
               : eri_blocks_per_sm(mode, fp32, block, smem);
  };
  const size_t slot_bytes = size_t(L.stride) * elt;
  L.rows = rows_hint > 0 ? rows_hint : (nq_avg > 12 ? 32 : (nq_avg > 6 ? 16 : 8));
  const size_t stage = stage_bytes_per_warp(fp32, L.rows);
  const size_t smem_cap = std::min<size_t>(ctx->smem_optin, 200 * 1024);
  L.global = slot_bytes > 40 * 1024;
  int best_warps = -1, bps = 1;
  for (int wpb : {4, 2, 1}) {
    const size_t smem = wpb * (stage + (L.global ? 0 : slot_bytes));
    if (smem > smem_cap) continue;
    const int b = std::max(1, occupancy(32 * wpb, smem));
    if (b * wpb > best_warps) {
      best_warps = b * wpb;
      bps = b;
      L.wpb = wpb;
      L.smem = smem;
    }
  }
  if (best_warps < 0) {  // not even one warp's slots fit: global slots
    L.global = true;
    L.wpb = 4;
    L.smem = L.wpb * stage;
    bps = std::max(1, occupancy(32 * L.wpb, L.smem));
  }
  L.block = 32 * L.wpb;
  long long grid = (long long)ctx->nsm * bps;
  const long long need = (nwork + L.wpb - 1) / L.wpb;
  grid = std::max<long long>(1, std::min(grid, need));
  if (L.global) {
    const size_t per_block = size_t(L.wpb) * slot_bytes;
    const size_t cap = size_t(2) << 30;  // 2 GiB of per-warp slot scratch at most
    grid = std::min<long long>(grid, std::max<size_t>(1, cap / per_block));
    DBuf& scr = ctx->scratch ? *ctx->scratch : ctx->gscratch;
    if (ctx->noalloc) {  // use the slot scratch a previous pass left, never grow it
      if (scr.n < per_block)
        return fail(ctx, LGX_ERR_INVALID_ARG,
                    "slot scratch not prepared: call lgx_jk_device once with the same settings");
      grid = std::min<long long>(grid, (long long)(scr.n / per_block));
    } else {
      CK(scr.ensure(size_t(grid) * per_block));
    }
  }
  L.grid = int(grid);
  return LGX_OK;
}

// Register kernels exist for the generated classes (deriv 0; see
// codegen/gen_rk.py for the limits per mode) with the standard pure flags;
// everything else runs on the warp-cooperative program kernel.
// Context and basis pointers every kernel launch needs.
void fill_common(const lgx_context* ctx, const BasisDev& B, EriArgs& a) {
  a.basis = B.dev;
  a.pairs = B.pairs.as<PairRec>();
  a.pprims = B.pprims.as<PrimPairRec>();
  a.ppds = B.ppds.as<PrimPairJKds>();
  a.pair_swap = B.pair_swap.as<unsigned char>();
  a.boys = ctx->boys.as<double>();
  a.boys_tay = ctx->boys_tay.as<double>();
  a.boys32 = ctx->boys32.as<float>();
  a.inv_odd = ctx->inv_odd.as<double>();
  a.sph_off = ctx->sph_off.as<int>();
  a.sph_c = ctx->sph_c.as<int>();
  a.sph_cd = ctx->sph_cd.as<double>();
  a.sph_cf = ctx->sph_cf.as<float>();
  a.error_flag = ctx->errflag.as<int>();
  a.op = ctx->op;
  a.omega2 = ctx->omega * ctx->omega;
  a.fprecision = float(a.precision);
  a.fln_prec = float(std::max(a.ln_prec, -1.0e30));
}

bool rk_eligible(const lgx_context* ctx, const BasisDev& B, const ProgDev& P, int mode,
                 bool fp32) {
  if (!ctx->use_rk || !B.std_pure || P.host.deriv != 0) return false;
  const bool att = ctx->op != LGX_OP_COULOMB;  // attenuated: J/K register kernels only
  return rk_available(fp32, mode, att, P.host.la, P.host.lb, P.host.lc, P.host.ld);
}

int choose_group(double nq_avg) {
  int g = 1;
  while (g < 32 && g * 2 <= nq_avg * 0.5) g *= 2;
  return g;
}

bool post_gen_ok(const lgx_context* ctx, const BasisDev& B, const ProgDev& P, int mode) {
  int nacc = 0, slots = 0;
  return ctx->use_post && mode_jk(mode) && B.std_pure && P.host.deriv == 0 &&
         ctx->op == LGX_OP_COULOMB &&
         post_info(P.host.la, P.host.lb, P.host.lc, P.host.ld, &nacc, &slots);
}

// Default variant of a class bin (before or without tuning).
Variant default_variant(const lgx_context* ctx, const BasisDev& B, const ProgDev& P, int mode,
                        bool fp32, bool implicit, double nq_avg) {
  Variant v;
  if (rk_eligible(ctx, B, P, mode, fp32)) {
    v.kind = 0;
    v.group = implicit ? 1 : choose_group(nq_avg);
  } else {
    v.kind = post_gen_ok(ctx, B, P, mode) ? 2 : 1;
  }
  return v;
}

lgx_status run_rk(lgx_context* ctx, BasisDev& B, const ProgDev& P, int mode, bool fp32,
                  EriArgs a, long long nwork, int group) {
  fill_common(ctx, B, a);
  a.group = group;
  CK(rk_launch(fp32, mode, a.op != LGX_OP_COULOMB, P.host.la, P.host.lb, P.host.lc, P.host.ld, a,
               nwork, ctx->nsm,
               ctx->launch_stream ? ctx->launch_stream : ctx->stream));
  return LGX_OK;
}

// Short explicit FP64 store lists (at most one quartet per SM): one block
// of kBlockThreads per quartet (eri_block_store_kernel), the slots in shared
// memory when they fit, else in per-block global scratch.
lgx_status run_block_store(lgx_context* ctx, BasisDev& B, const ProgDev& P, EriArgs a,
                           long long nwork) {
  fill_common(ctx, B, a);
  a.prog = P.dev;
  a.slot_stride = (P.host.total_slots() + 1) & ~1;
  const size_t slot_bytes = size_t(a.slot_stride) * sizeof(double);
  const size_t smem_cap = std::min<size_t>(ctx->smem_optin, 200 * 1024);
  const int grid = int(std::max<long long>(1, nwork));
  a.global_slots = 0;
  // small classes: each warp contracts its own primitive quartets (8 staged
  // rows and the accumulators per warp in shared memory), no block-wide
  // barrier per recurrence level
  const size_t per_warp = stage_bytes_per_warp(false, 8) + slot_bytes;
  if ((kBlockThreads / 32) * per_warp <= smem_cap) {
    a.warp_rows = 1;
    a.stage_rows = 8;
    CK(launch_eri_block_store(a, grid, (kBlockThreads / 32) * per_warp,
                              ctx->launch_stream ? ctx->launch_stream : ctx->stream));
    return LGX_OK;
  }
  a.warp_rows = 0;
  a.stage_rows = 32;
  const size_t stage = stage_bytes_per_warp(false, a.stage_rows);
  size_t smem = stage + slot_bytes;
  if (smem > smem_cap) {
    DBuf& scr = ctx->scratch ? *ctx->scratch : ctx->gscratch;
    if (ctx->noalloc && scr.n < size_t(grid) * slot_bytes)
      return fail(ctx, LGX_ERR_INVALID_ARG, "slot scratch not prepared");
    if (!ctx->noalloc) CK(scr.ensure(size_t(grid) * slot_bytes));
    a.gscratch = scr.p;
    a.global_slots = 1;
    smem = stage;
  }
  CK(launch_eri_block_store(a, grid, smem, ctx->launch_stream ? ctx->launch_stream : ctx->stream));
  return LGX_OK;
}

lgx_status run_eri(lgx_context* ctx, BasisDev& B, const ProgDev& P, int mode, bool fp32,
                   EriArgs a, long long nwork, double nq_avg = 1.0,
                   const Variant* var = nullptr) {
  const Variant v = var ? *var : default_variant(ctx, B, P, mode, fp32, a.implicit, nq_avg);
  if (v.kind == 0) return run_rk(ctx, B, P, mode, fp32, a, nwork, v.group);
  if (v.kind == 1 && mode == kModeStore && !fp32 && !a.implicit && nwork <= ctx->nsm)
    return run_block_store(ctx, B, P, a, nwork);
  const bool gen = v.kind == 2;
  Launch L;
  lgx_status s = plan_launch(ctx, P, mode, fp32, nwork, nq_avg, v.rows, gen, L);
  if (s != LGX_OK) return s;
  fill_common(ctx, B, a);
  a.prog = P.dev;
  const bool own_counter = a.counter == nullptr;  // else zeroed by the caller
  if (own_counter) a.counter = ctx->counter.as<unsigned long long>();
  a.slot_stride = L.stride;
  a.stage_rows = L.rows;
  a.global_slots = L.global ? 1 : 0;
  a.gscratch = (ctx->scratch ? ctx->scratch : &ctx->gscratch)->p;
  if (a.max_bps > 0) L.grid = std::min(L.grid, ctx->nsm * a.max_bps);
  cudaStream_t lst = ctx->launch_stream ? ctx->launch_stream : ctx->stream;
  const long long nwarps = (long long)L.grid * L.wpb;
  a.chunk = int(std::max<long long>(1, std::min<long long>(32, nwork / (nwarps * 8))));
  // every warp takes at most all chunks of the launch (plus slack); a test
  // hook (lgx_set_watchdog) can lower the bound to make the watchdog fire
  a.max_chunks = ctx->watchdog_chunks >= 0 ? ctx->watchdog_chunks : nwork / a.chunk + 2;
  if (own_counter) CK(cudaMemsetAsync(ctx->counter.p, 0, sizeof(unsigned long long), lst));
  if (gen)
    CK(post_launch(fp32, mode, P.host.la, P.host.lb, P.host.lc, P.host.ld, a, L.grid, L.block, L.smem,
                   lst));
  else
    CK(launch_eri(a, mode, fp32, L.grid, L.block, L.smem, lst));
  return LGX_OK;
}

lgx_status check_errflag(lgx_context* ctx) {
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, ctx->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (flag) {
    CK(cudaMemsetAsync(ctx->errflag.p, 0, sizeof(int), ctx->stream));
    return fail(ctx, LGX_ERR_WATCHDOG, "device work loop exceeded its bound");
  }
  return LGX_OK;
}

// Canonical quartet (engine.impl.h:1181-1211) -> work item.
struct Canon {
  int c[4];  // canonical shells
  int flags;
  int la, lb, lc, ld;
};
Canon canonicalize(const BasisDev& B, const int* s) {
  const int l0 = B.l[s[0]], l1 = B.l[s[1]], l2 = B.l[s[2]], l3 = B.l[s[3]];
  const bool stb = l0 < l1, stk = l2 < l3, sbk = l0 + l1 > l2 + l3;
  int perm[4];
  perm[0] = sbk ? (stk ? 3 : 2) : (stb ? 1 : 0);
  perm[1] = sbk ? (stk ? 2 : 3) : (stb ? 0 : 1);
  perm[2] = sbk ? (stb ? 1 : 0) : (stk ? 3 : 2);
  perm[3] = sbk ? (stb ? 0 : 1) : (stk ? 2 : 3);
  Canon q;
  for (int k = 0; k < 4; ++k) q.c[k] = s[perm[k]];
  const bool bsw = q.c[0] < q.c[1];  // stored pair has s1 >= s2
  const bool ksw = q.c[2] < q.c[3];
  q.flags = (bsw ? 1 : 0) | (ksw ? 2 : 0) |
            ((sbk ? 1 : 0) | (stb ? 2 : 0) | (stk ? 4 : 0)) << 2;
  q.la = B.l[q.c[0]];
  q.lb = B.l[q.c[1]];
  q.lc = B.l[q.c[2]];
  q.ld = B.l[q.c[3]];
  return q;
}

// Explicit quartet list -> grouped launches (store mode).
// mode32: kernel mode of the FP32 items (quartets with K12 K34 <
// mixed_thresh; kModeStore or kModeStoreB64), used when mixed_thresh > 0.
lgx_status run_explicit(lgx_context* ctx, BasisDev& B, const int32_t* quartets, long long n,
                        int deriv, int mode, double mixed_thresh, const int64_t* offsets,
                        double* d_out, int* d_isnull, double precision, int screening,
                        double* d_kschwarz, int mode32 = kModeStore) {
  // class key of each quartet from a (la, lb, lc, ld) table, counting
  // passes, and a stable scatter of the work items into one array grouped by
  // key (ascending key order, as the launches below go); long lists split
  // both passes over the host threads (per-thread counts merged so that the
  // items of a class keep the list order, packed offsets fixed up by the
  // chunks' prefix sums)
  constexpr int LK = kMaxLInternal + 1;
  struct ClassTables {
    std::vector<int> key;          // (la, lb, lc, ld) -> class index
    std::vector<std::array<int, 4>> shape;  // class index -> (la, lb, lc, ld)
  };
  static const ClassTables kTab = [] {
    ClassTables t;
    t.key.assign(LK * LK * LK * LK, -1);
    t.shape.resize(num_classes());
    for (int la = 0; la < LK; ++la)
      for (int lb = 0; lb < LK; ++lb)
        for (int lc = 0; lc < LK; ++lc)
          for (int ld = 0; ld < LK; ++ld) {
            const int ci = class_index(la, lb, lc, ld);
            t.key[((la * LK + lb) * LK + lc) * LK + ld] = ci;
            if (ci >= 0) t.shape[ci] = {la, lb, lc, ld};
          }
    return t;
  }();
  const int nkeys = 2 * num_classes();
  struct G {
    size_t count = 0, begin = 0;
    double nq = 0;
    int la = 0, lb = 0, lc = 0, ld = 0;
    bool fp32 = false;
  };
  const size_t nn = size_t(std::max<long long>(n, 0));
  std::vector<QuartetItem> items(nn);
  std::vector<int> keys(nn);
  const int nthr = nn >= 65536 ? int(std::max(1u, std::min(16u, std::thread::hardware_concurrency())))
                               : 1;
  const size_t chunk = (nn + nthr - 1) / std::max(1, nthr);
  std::vector<std::vector<size_t>> cnt(nthr, std::vector<size_t>(nkeys, 0));
  std::vector<std::vector<double>> nqs(nthr, std::vector<double>(nkeys, 0.0));
  std::vector<long long> span(nthr, 0);  // packed output length of each chunk
  std::vector<int> bad(nthr, 0);          // 1: shell index out of range, 2: l beyond the build
  const long long nsets = deriv ? 12 : 1;
  auto pass1 = [&](int t) {
    const size_t q0 = std::min(nn, size_t(t) * chunk), q1 = std::min(nn, q0 + chunk);
    long long run_off = 0;
    for (size_t q = q0; q < q1; ++q) {
      const int* s = quartets + 4 * q;
      for (int k = 0; k < 4; ++k)
        if (s[k] < 0 || s[k] >= B.nshell) {
          bad[t] = 1;
          return;
        }
      const Canon c = canonicalize(B, s);
      QuartetItem& it = items[q];
      it.bra_pair = int(pidx(std::max(c.c[0], c.c[1]), std::min(c.c[0], c.c[1])));
      it.ket_pair = int(pidx(std::max(c.c[2], c.c[3]), std::min(c.c[2], c.c[3])));
      it.flags = c.flags;
      it.pad = int(q);
      if (mode == kModeSchwarz) {
        it.out = offsets ? offsets[q] : (long long)q;
      } else if (offsets) {
        it.out = offsets[q];
      } else {
        long long nv = 1;
        for (int k = 0; k < 4; ++k) nv *= nfunc(B.l[s[k]], B.pure[s[k]]);
        it.out = run_off;  // chunk-relative; the chunk's base is added in the scatter
        run_off += nv * nsets;
      }
      bool fp32 = false;
      if (mode == kModeStore && mixed_thresh > 0 && B.schwarz_ok) {
        const double bound = B.Kpair[it.bra_pair] * B.Kpair[it.ket_pair];
        fp32 = bound < mixed_thresh;
      }
      const int ci = kTab.key[((c.la * LK + c.lb) * LK + c.lc) * LK + c.ld];
      if (ci < 0) {
        bad[t] = 2;
        return;
      }
      const int key = ci * 2 + (fp32 ? 1 : 0);
      keys[q] = key;
      ++cnt[t][key];
      nqs[t][key] += double(B.hpairs[it.bra_pair].npp) * double(B.hpairs[it.ket_pair].npp);
    }
    span[t] = run_off;
  };
  auto run_threads = [&](auto&& fn) {
    if (nthr == 1) {
      fn(0);
      return;
    }
    std::vector<std::thread> th;
    th.reserve(nthr);
    for (int t = 0; t < nthr; ++t) th.emplace_back(fn, t);
    for (auto& x : th) x.join();
  };
  run_threads(pass1);
  for (int t = 0; t < nthr; ++t) {
    if (bad[t] == 1) return fail(ctx, LGX_ERR_INVALID_ARG, "quartet shell index out of range");
    if (bad[t] == 2) return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "angular momentum beyond LGX_MAX_L");
  }
  std::vector<long long> base(nthr, 0);  // packed output offset of each chunk
  for (int t = 1; t < nthr; ++t) base[t] = base[t - 1] + span[t - 1];
  // class order ascending; within a class, chunk order (= list order)
  std::vector<G> gk(nkeys);
  std::vector<std::vector<size_t>> pos(nthr, std::vector<size_t>(nkeys, 0));
  size_t total = 0;
  std::vector<int> order;  // keys with work, ascending
  for (int k = 0; k < nkeys; ++k) {
    G& g = gk[k];
    g.begin = total;
    for (int t = 0; t < nthr; ++t) {
      pos[t][k] = total;
      total += cnt[t][k];
      g.nq += nqs[t][k];
    }
    g.count = total - g.begin;
    if (g.count) {
      const auto& sh = kTab.shape[k / 2];
      g.la = sh[0]; g.lb = sh[1]; g.lc = sh[2]; g.ld = sh[3];
      g.fp32 = (k & 1) != 0;
      order.push_back(k);
    }
  }
  CK(ctx->items.ensure(std::max<size_t>(total, 1) * sizeof(QuartetItem)));
  std::vector<QuartetItem> all(total);
  const bool packed = !offsets && mode != kModeSchwarz;
  auto scatter = [&](int t) {
    const size_t q0 = std::min(nn, size_t(t) * chunk), q1 = std::min(nn, q0 + chunk);
    std::vector<size_t>& p = pos[t];
    for (size_t q = q0; q < q1; ++q) {
      QuartetItem it = items[q];
      if (packed) it.out += base[t];
      all[p[keys[q]]++] = it;
    }
  };
  run_threads(scatter);
  CK(cudaMemcpyAsync(ctx->items.p, all.data(), total * sizeof(QuartetItem),
                     cudaMemcpyHostToDevice, ctx->stream));
  // the class launches run on parallel branches (streams forked from and
  // joined back into ctx->stream, one work counter and one program-kernel
  // slot scratch per launch / branch): a short list, such as the raised and
  // lowered quartets of a second-derivative set, then costs its slowest
  // class rather than the sum of its classes
  const int ng = int(order.size());
  const int nbr = std::min(ng, lgx_context::kMaxBranches);
  const bool split = ctx->overlap && nbr > 1;
  CK(ctx->xcounters.ensure(size_t(ng) * sizeof(unsigned long long)));
  CK(cudaMemsetAsync(ctx->xcounters.p, 0, size_t(ng) * sizeof(unsigned long long), ctx->stream));
  if (split) {
    CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
    for (int b = 0; b < nbr; ++b) {
      CK(cudaStreamWaitEvent(ctx->s64[b], ctx->ev_fork, 0));
      CK(cudaStreamWaitEvent(ctx->s32[b], ctx->ev_fork, 0));
    }
  }
  struct Restore {  // launch stream / scratch back to the context defaults
    lgx_context* c;
    ~Restore() {
      c->launch_stream = nullptr;
      c->scratch = nullptr;
    }
  } restore{ctx};
  size_t gi = 0;
  lgx_status s = LGX_OK;
  for (const int key : order) {
    const G& grp = gk[key];
    ProgDev* P = nullptr;
    s = get_prog(ctx, grp.la, grp.lb, grp.lc, grp.ld, deriv, &P);
    if (s != LGX_OK) break;
    const bool fp32 = grp.fp32;
    if (split) {
      const int b = int(gi) % nbr;
      ctx->launch_stream = fp32 ? ctx->s32[b] : ctx->s64[b];
      ctx->scratch = (fp32 || b > 0) ? &ctx->gscratch_br[(fp32 ? nbr : 0) + b] : &ctx->gscratch;
    }
    EriArgs a{};
    a.counter = ctx->xcounters.as<unsigned long long>() + gi;
    a.precision = precision;
    a.ln_prec = precision > 0 ? std::log(precision) : -std::numeric_limits<double>::max();
    a.screening = screening;
    a.items = ctx->items.as<QuartetItem>() + grp.begin;
    a.nitems = (long long)grp.count;
    a.implicit = 0;
    a.out = d_out;
    a.is_null = d_isnull;
    a.kschwarz = d_kschwarz;
    const double nq = grp.nq / double(std::max<size_t>(1, grp.count));
    s = run_eri(ctx, B, *P, fp32 ? mode32 : mode, fp32, a, a.nitems, nq);
    if (s != LGX_OK) break;
    ++gi;
  }
  if (split) {  // joined on every path, so ctx->stream orders after all branch work
    for (int b = 0; b < nbr; ++b) {
      CK(cudaEventRecord(ctx->ev_join[2 * b], ctx->s64[b]));
      CK(cudaEventRecord(ctx->ev_join[2 * b + 1], ctx->s32[b]));
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[2 * b], 0));
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[2 * b + 1], 0));
    }
  }
  return s;
}

lgx_status ensure_schwarz(lgx_context* ctx, BasisDev& B) {
  if (B.schwarz_ok) return LGX_OK;
  lgx_status s = ensure_pairs(ctx, B, -std::numeric_limits<double>::max(), 0);
  if (s != LGX_OK) return s;
  const long long npairs = (long long)B.hpairs.size();
  std::vector<int32_t> q(4 * npairs);
  for (long long p = 0; p < npairs; ++p) {
    q[4 * p] = B.hpairs[p].s1;
    q[4 * p + 1] = B.hpairs[p].s2;
    q[4 * p + 2] = B.hpairs[p].s1;
    q[4 * p + 3] = B.hpairs[p].s2;
  }
  // kept on the device too: the density-weighted J/K screening reads it
  CK(B.Kd.ensure(npairs * sizeof(double)));
  s = run_explicit(ctx, B, q.data(), npairs, 0, kModeSchwarz, 0.0, nullptr, nullptr, nullptr,
                   0.0, 0, B.Kd.as<double>());
  if (s != LGX_OK) return s;
  B.Kpair.resize(npairs);
  CK(cudaMemcpyAsync(B.Kpair.data(), B.Kd.p, npairs * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  s = check_errflag(ctx);
  if (s != LGX_OK) return s;
  B.schwarz_ok = true;
  // the J/K passes use libint's default primitive screening (precision eps)
  return LGX_OK;
}

// ------------------------------------------------------------ J/K bins
int pair_class(int lhi, int llo) { return lhi * (lhi + 1) / 2 + llo; }  // 10 classes

lgx_status build_bins(lgx_context* ctx, BasisDev& B, double thresh, int mode, double mixed) {
  BinCache& C = ctx->bins;
  if (C.valid && C.thresh == thresh && C.mode == mode && C.mixed == mixed &&
      C.subset_version == ctx->subset_version)
    return LGX_OK;
  C.valid = false;
  C.bins.clear();
  const long long npairs = (long long)B.hpairs.size();
  double Kmax = 0;
  for (double k : B.Kpair) Kmax = std::max(Kmax, k);
  // significant pairs per pair class, ordered by (contraction depth, K desc)
  std::vector<std::vector<int>> lists(10);
  for (long long p = 0; p < npairs; ++p) {
    if (B.Kpair[p] * Kmax < thresh) continue;
    if (!ctx->pair_subset.empty() && !ctx->pair_subset[p]) continue;
    const int s1 = B.hpairs[p].s1, s2 = B.hpairs[p].s2;
    const int lhi = std::max(B.l[s1], B.l[s2]), llo = std::min(B.l[s1], B.l[s2]);
    lists[pair_class(lhi, llo)].push_back(int(p));
  }
  std::vector<std::vector<int>> groups(10);  // group boundaries (depth runs)
  for (int c = 0; c < 10; ++c) {
    auto& v = lists[c];
    std::stable_sort(v.begin(), v.end(), [&](int a, int b) {
      if (B.hpairs[a].npp != B.hpairs[b].npp) return B.hpairs[a].npp < B.hpairs[b].npp;
      return B.Kpair[a] > B.Kpair[b];
    });
    groups[c].push_back(0);
    for (size_t i = 1; i < v.size(); ++i)
      if (B.hpairs[v[i]].npp != B.hpairs[v[i - 1]].npp) groups[c].push_back(int(i));
    groups[c].push_back(int(v.size()));
  }
  C.class_off.assign(11, 0);
  std::vector<int> flat;
  for (int c = 0; c < 10; ++c) {
    C.class_off[c] = (long long)flat.size();
    flat.insert(flat.end(), lists[c].begin(), lists[c].end());
  }
  C.class_off[10] = (long long)flat.size();
  CK(C.class_lists.ensure(std::max<size_t>(1, flat.size()) * sizeof(int)));
  if (!flat.empty())
    CK(cudaMemcpyAsync(C.class_lists.p, flat.data(), flat.size() * sizeof(int),
                       cudaMemcpyHostToDevice, ctx->stream));
  {
    // FP32 record layout: per class, per depth group [g0, g1) of npp n, the
    // record of (position i, primitive pair ip) at base + ip * (g1 - g0) + (i - g0)
    std::vector<int2> idx(std::max<size_t>(1, flat.size()));
    std::vector<int> src;
    for (int c = 0; c < 10; ++c) {
      const auto& v = lists[c];
      const auto& g = groups[c];
      for (size_t gi = 0; gi + 1 < g.size(); ++gi) {
        const int g0 = g[gi], g1 = g[gi + 1];
        if (g1 <= g0) continue;
        const int n = B.hpairs[v[g0]].npp;
        const long long base = (long long)src.size();
        if (base + (long long)n * (g1 - g0) > std::numeric_limits<int>::max())
          return fail(ctx, LGX_ERR_TOO_LARGE, "too many primitive-pair records");
        src.resize(base + (size_t)n * (g1 - g0));
        for (int i = g0; i < g1; ++i) {
          const int pr = v[i];
          idx[C.class_off[c] + i] = make_int2(int(base + (i - g0)), g1 - g0);
          const unsigned sw = B.hswap[pr] ? 0x80000000u : 0u;
          for (int ip = 0; ip < n; ++ip)
            src[base + (size_t)ip * (g1 - g0) + (i - g0)] =
                int(unsigned(B.hpairs[pr].pp_off + ip) | sw);
        }
      }
    }
    C.nrec = (long long)src.size();
    CK(C.rec_idx.ensure(idx.size() * sizeof(int2)));
    CK(C.rec_src.ensure(std::max<size_t>(1, src.size()) * sizeof(int)));
    CK(C.recs.ensure(std::max<size_t>(1, src.size()) * sizeof(PrimPairJK32)));
    CK(C.recsds.ensure(std::max<size_t>(1, src.size()) * sizeof(PrimPairJKds)));
    CK(cudaMemcpyAsync(C.rec_idx.p, idx.data(), idx.size() * sizeof(int2),
                       cudaMemcpyHostToDevice, ctx->stream));
    if (!src.empty())
      CK(cudaMemcpyAsync(C.rec_src.p, src.data(), src.size() * sizeof(int),
                         cudaMemcpyHostToDevice, ctx->stream));
    C.rec_version = ~0ull;
  }
  int cls_l[10][2];
  for (int lhi = 0; lhi <= 3; ++lhi)
    for (int llo = 0; llo <= lhi; ++llo) {
      cls_l[pair_class(lhi, llo)][0] = lhi;
      cls_l[pair_class(lhi, llo)][1] = llo;
    }
  auto nf_pair = [&](int p) {
    return (long long)nfunc(B.l[B.hpairs[p].s1], B.pure[B.hpairs[p].s1]) *
           nfunc(B.l[B.hpairs[p].s2], B.pure[B.hpairs[p].s2]);
  };
  C.quartets[0] = C.quartets[1] = 0;
  for (int x = 0; x < 10; ++x)
    for (int y = 0; y < 10; ++y) {
      const int Lx = cls_l[x][0] + cls_l[x][1], Ly = cls_l[y][0] + cls_l[y][1];
      if (!(Lx < Ly || (Lx == Ly && x <= y))) continue;
      const auto& bra = lists[x];
      const auto& ket = lists[y];
      if (bra.empty() || ket.empty()) continue;
      auto bin = std::make_unique<BinHost>();
      bin->la = cls_l[x][0]; bin->lb = cls_l[x][1];
      bin->lc = cls_l[y][0]; bin->ld = cls_l[y][1];
      bin->bra_class = x;
      bin->ket_class = y;
      // kets j in [k0, k1) (one depth group, K desc) with K_i*K_j >= t
      auto count_ge = [&](double Ki, double t, int k0, int k1) -> int {
        if (Ki <= 0) return 0;
        const double need = t / Ki;
        int lo = k0, hi = k1;
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (B.Kpair[ket[mid]] >= need) lo = mid + 1; else hi = mid;
        }
        return lo - k0;
      };
      std::vector<long long> st[2];
      std::vector<int> sb[2], sj[2];
      for (int sp = 0; sp < 2; ++sp) st[sp].push_back(0);
      double nq_sum = 0, nq_w = 0;
      const auto& gb = groups[x];
      const auto& gk = groups[y];
      for (size_t bgi = 0; bgi + 1 < gb.size(); ++bgi)
        for (size_t kgi = 0; kgi + 1 < gk.size(); ++kgi) {
          if (x == y && kgi > bgi) continue;  // unique quartets: ket index <= bra index
          const int k0 = gk[kgi], k1 = gk[kgi + 1];
          for (int i = gb[bgi]; i < gb[bgi + 1]; ++i) {
            const double Ki = B.Kpair[bra[i]];
            int n = count_ge(Ki, thresh, k0, k1);
            if (x == y && kgi == bgi) n = std::min(n, i - k0 + 1);
            if (n <= 0) continue;
            int m = n;
            if (mode == LGX_MIXED) m = std::min(n, count_ge(Ki, mixed, k0, k1));
            if (m > 0) {
              st[0].push_back(st[0].back() + m);
              sb[0].push_back(i);
              sj[0].push_back(k0);
            }
            if (n - m > 0) {
              st[1].push_back(st[1].back() + (n - m));
              sb[1].push_back(i);
              sj[1].push_back(k0 + m);
            }
            nq_sum += double(n) * B.hpairs[bra[i]].npp * B.hpairs[ket[k0]].npp;
            nq_w += n;
          }
        }
      bin->nq_avg = nq_w > 0 ? nq_sum / nq_w : 1.0;
      const long long nfq = nf_pair(bra[0]) * nf_pair(ket[0]);
      for (int sp = 0; sp < 2; ++sp) {
        bin->nseg[sp] = int(sb[sp].size());
        bin->total[sp] = st[sp].back();
        bin->integrals[sp] = bin->total[sp] * nfq;
        C.quartets[sp] += bin->total[sp];
        if (bin->nseg[sp] == 0) continue;
        CK(bin->seg_start[sp].ensure(st[sp].size() * sizeof(long long)));
        CK(bin->seg_bra[sp].ensure(sb[sp].size() * sizeof(int)));
        CK(bin->seg_j0[sp].ensure(sj[sp].size() * sizeof(int)));
        CK(cudaMemcpyAsync(bin->seg_start[sp].p, st[sp].data(), st[sp].size() * sizeof(long long),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(bin->seg_bra[sp].p, sb[sp].data(), sb[sp].size() * sizeof(int),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(bin->seg_j0[sp].p, sj[sp].data(), sj[sp].size() * sizeof(int),
                           cudaMemcpyHostToDevice, ctx->stream));
      }
      C.bins.push_back(std::move(bin));
    }
  CK(cudaStreamSynchronize(ctx->stream));
  C.valid = true;
  ++ctx->version;
  C.thresh = thresh;
  C.mode = mode;
  C.mixed = mixed;
  C.subset_version = ctx->subset_version;
  return LGX_OK;
}

// Algorithmic FP operations of the per-primitive-quartet prologue, counted
// from the equations of libint's primitive data (engine.impl.h:1389-1466),
// each add, multiply, divide, square root or exponential one operation and
// an FMA two:
//   zeta + eta, 1/(zeta + eta), rho = zeta eta / (zeta + eta)        4
//   P - Q, |P - Q|^2, T = rho |P - Q|^2                              9
//   pfac = K_ab K_cd / sqrt(zeta + eta)                               3
//   F_mmax(T) by the order-6 Taylor step, e^{-T}, 2T, and the downward
//   recursion F_m = (2T F_{m+1} + e^{-T}) / (2m + 1)          14 + 3 mmax
//   (00|00)^(m) = pfac F_m                                      mmax + 1
//   W - P, W - Q (eta / (zeta + eta), zeta / (zeta + eta), 6 products) 8
//   P - A, Q - C                                                      6
//   1/2zeta, 1/2eta, 1/2(zeta + eta), rho/zeta, rho/eta               5
// = 50 + 4 mmax.  The mixed scheme's FP32 kernels with the Boys function in
// FP64 form rho, P - Q, T and F_m(T) again in FP64 (27 + 3 mmax on the FP64
// pipe) besides the FP32 quantities the VRR uses; prologue_flops64 is that
// FP64 share.
double prologue_flops(int mmax, bool b64) {
  return 50.0 + 4.0 * mmax + (b64 ? 13.0 : 0.0);
}
double prologue_flops64(int mmax, bool b64) { return b64 ? 27.0 + 3.0 * mmax : 0.0; }

// FP operations of the Cartesian -> solid-harmonic transform of one set.
double sph_flops(int la, int lb, int lc, int ld, const int* pure) {
  const int l[4] = {la, lb, lc, ld};
  int dims[4];
  for (int k = 0; k < 4; ++k) dims[k] = ncart(l[k]);
  double f = 0;
  for (int k = 0; k < 4; ++k) {
    if (!pure[k]) continue;
    double rest = 1;
    for (int t = 0; t < 4; ++t)
      if (t != k) rest *= dims[t];
    f += 2.0 * (2 * l[k] + 1) * dims[k] * rest;
    dims[k] = 2 * l[k] + 1;
  }
  return f;
}

int tune_key(const BinHost& bin, int deriv, int mode, bool fp32, int op) {
  return (((class_index(bin.la, bin.lb, bin.lc, bin.ld) * 2 + deriv) * 8 + mode) * 2 +
          (fp32 ? 1 : 0)) * 4 + op;
}

// Work description of precision space sp of a class bin.
void bin_args(const BinCache& C, const BinHost& bin, int sp, EriArgs& a) {
  a.implicit = 1;
  a.jk32 = C.recs.as<PrimPairJK32>();
  a.jkds = C.recsds.as<PrimPairJKds>();
  a.bin.bra_rec = C.rec_idx.as<int2>() + C.class_off[bin.bra_class];
  a.bin.ket_rec = C.rec_idx.as<int2>() + C.class_off[bin.ket_class];
  a.bin.bra_pairs = C.class_lists.as<int>() + C.class_off[bin.bra_class];
  a.bin.ket_pairs = C.class_lists.as<int>() + C.class_off[bin.ket_class];
  a.bin.seg_start = bin.seg_start[sp].as<long long>();
  a.bin.seg_bra = bin.seg_bra[sp].as<int>();
  a.bin.seg_j0 = bin.seg_j0[sp].as<int>();
  a.bin.nseg = bin.nseg[sp];
  a.bin.total = bin.total[sp];
}

// Per-class launch-shape autotuner: for every (class, precision) of the
// pass without a tuned variant, times the candidate variants (register
// kernel lanes per quartet; program kernel with interpreted or generated
// post stage and its staging rows) on a leading sample of the bin's
// quartets, into scratch accumulators, and keeps the fastest.  Runs once per
// basis; later passes reuse the choice.
// mode32: kernel mode of the FP32 precision space (kModeJK, or kModeJKB64
// for the mixed scheme with the Boys function in FP64), or -1 when the pass
// runs every quartet in FP64.
lgx_status tune_bins(lgx_context* ctx, BasisDev& B, int mode, int deriv, int mode32,
                     EriArgs base) {
  if (!ctx->tune || ctx->noalloc) return LGX_OK;
  const BinCache& C = ctx->bins;
  const size_t nn = std::max(size_t(B.nbf) * B.nbf, size_t(3 * B.natoms + 64));
  bool scratch = false;
  for (size_t bi = 0; bi < C.bins.size(); ++bi) {
    const BinHost& bin = *C.bins[bi];
    ProgDev* P = nullptr;
    lgx_status s = get_prog(ctx, bin.la, bin.lb, bin.lc, bin.ld, deriv, &P);
    if (s != LGX_OK) return s;
    for (int sp = 0; sp < 2; ++sp) {
      if (bin.total[sp] == 0) continue;
      const bool fp32 = (sp == 1) && mode32 >= 0;
      const int kmode = fp32 ? mode32 : mode;
      const int key = tune_key(bin, deriv, kmode, fp32, ctx->op);
      if (ctx->tuned.count(key)) continue;
      std::vector<Variant> cand;
      const Variant d = default_variant(ctx, B, *P, kmode, fp32, true, bin.nq_avg);
      cand.push_back(d);
      if (d.kind == 0) {
        for (int g = 2; g <= 8 && g <= 2 * bin.nq_avg; g *= 2) cand.push_back({0, g, 0});
      } else {
        for (int kind = 1; kind <= d.kind; ++kind) {
          cand.push_back({kind, 1, 8});
          if (bin.nq_avg > 4) cand.push_back({kind, 1, 32});
        }
      }
      const long long cap = d.kind == 0 ? (1LL << 22) : (1LL << 17);
      const long long sample = std::min<long long>(bin.total[sp], cap);
      if (cand.size() < 2 || sample < ctx->tune_min) {
        ctx->tuned[key] = d;
        ++ctx->version;
        continue;
      }
      if (!scratch) {
        CK(ctx->tuneJ.ensure(nn * sizeof(double)));
        CK(ctx->tuneK.ensure(nn * sizeof(double)));
        scratch = true;
      }
      EriArgs a = base;
      bin_args(C, bin, sp, a);
      a.bin.total = sample;
      a.prim_count = nullptr;
      if (mode == kModeJK) {
        a.Jacc = ctx->tuneJ.as<double>();
        a.Kacc = ctx->tuneK.as<double>();
      } else {
        a.gJ = ctx->tuneJ.as<double>();
        a.gK = ctx->tuneK.as<double>();
      }
      float best = 0;
      Variant bestv = d;
      for (size_t ci = 0; ci < cand.size(); ++ci) {
        float ms = 0;
        for (int rep = 0; rep < 2; ++rep) {  // the second run is timed
          CK(cudaEventRecord(ctx->ev0, ctx->stream));
          s = run_eri(ctx, B, *P, kmode, fp32, a, sample, bin.nq_avg, &cand[ci]);
          if (s != LGX_OK) return s;
          CK(cudaEventRecord(ctx->ev1, ctx->stream));
        }
        CK(cudaEventSynchronize(ctx->ev1));
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (ci == 0 || ms < best) {
          best = ms;
          bestv = cand[ci];
        }
      }
      ctx->tuned[key] = bestv;
      ++ctx->version;
    }
  }
  return check_errflag(ctx);
}

// Enqueues the launches of one screened pass (every class bin and
// precision space) on ctx->stream with no host synchronisation, so that the
// same sequence can be captured into a CUDA graph.  Work counters and
// primitive counters live in ctx->primcount ([0, nslots) primitive quartets,
// [nslots, 2 nslots) work counters) and are zeroed by the first node.
lgx_status enqueue_bins(lgx_context* ctx, BasisDev& B, int mode, int deriv, int mode32,
                        EriArgs base, PassRecs& pr) {
  BinCache& C = ctx->bins;
  pr = PassRecs{};
  // the launches of the pass: one per class bin and precision space
  struct Job {
    size_t bi;
    int sp;
    bool fp32;
    double est;  // expected device time (ms, or a relative cost before any pass)
    int branch;
  };
  std::vector<Job> jobs;
  for (size_t bi = 0; bi < C.bins.size(); ++bi) {
    const BinHost& bin = *C.bins[bi];
    for (int sp = 0; sp < 2; ++sp) {
      if (bin.total[sp] == 0) continue;
      const bool fp32 = (sp == 1) && mode32 >= 0;
      const double est = bin.last_ms[sp] > 0
                             ? bin.last_ms[sp]
                             : 1e-9 * double(bin.total[sp]) * bin.nq_avg * (fp32 ? 1.0 : 8.0);
      jobs.push_back({bi, sp, fp32, est, 0});
    }
  }
  const size_t nlaunch = jobs.size();
  // Parallel branches: each precision's launches spread over nbr streams
  // (round-robin, or longest first onto the least-loaded branch with the
  // bins' device times of the previous pass as estimates), so that the
  // tails of the persistent class launches overlap with other launches and
  // FP32 launches run beside FP64-pipe-bound ones.
  const bool split = ctx->overlap && !ctx->noalloc && nlaunch > 1;
  pr.split = split;
  const int nbr = std::max(1, std::min(ctx->branches, lgx_context::kMaxBranches));
  if (split && ctx->branch_policy == 1) {  // round-robin in bin order
    int nxt[2] = {0, 0};
    for (auto& j : jobs) j.branch = nxt[j.fp32 ? 1 : 0]++ % nbr;
  } else if (split) {  // longest first onto the least-loaded branch
    std::vector<size_t> ord(jobs.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](size_t x, size_t y) { return jobs[x].est > jobs[y].est; });
    double load[2][lgx_context::kMaxBranches] = {};
    for (size_t i : ord) {
      Job& j = jobs[i];
      double* l = load[j.fp32 ? 1 : 0];
      int b = 0;
      for (int k = 1; k < nbr; ++k)
        if (l[k] < l[b]) b = k;
      j.branch = b;
      l[b] += j.est;
    }
    if (ctx->branch_policy == 0)  // issue longest first too (else in bin order)
      std::stable_sort(jobs.begin(), jobs.end(),
                       [](const Job& x, const Job& y) { return x.est > y.est; });
  }
  // per-launch events persist in the context (a captured pass refers to
  // them); the no-allocation path only uses events that already exist
  pr.timed = ctx->lev.size() >= 2 * nlaunch;
  if (!pr.timed && !ctx->noalloc) {
    while (ctx->lev.size() < 2 * nlaunch) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      ctx->lev.push_back(e);
    }
    pr.timed = true;
  }
  pr.nslots = 2 * C.bins.size() + 1;
  pr.count = !ctx->noalloc || ctx->primcount.n >= 2 * pr.nslots * sizeof(unsigned long long);
  unsigned long long* counters = nullptr;
  if (pr.count) {
    CK(ctx->primcount.ensure(2 * pr.nslots * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(ctx->primcount.p, 0, 2 * pr.nslots * sizeof(unsigned long long),
                       ctx->stream));
    counters = ctx->primcount.as<unsigned long long>() + pr.nslots;
  }
  // inside a capture the timing events become event-record nodes of the graph
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(ctx->stream, &cap));
  const unsigned evflags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0;
  CK(cudaEventRecordWithFlags(ctx->ev0, ctx->stream, evflags));
  if (split) {
    CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
    for (int b = 0; b < nbr; ++b) {
      CK(cudaStreamWaitEvent(ctx->s64[b], ctx->ev_fork, 0));
      CK(cudaStreamWaitEvent(ctx->s32[b], ctx->ev_fork, 0));
    }
  }
  struct Restore {  // launch stream / scratch back to the context defaults
    lgx_context* c;
    ~Restore() {
      c->launch_stream = nullptr;
      c->scratch = nullptr;
    }
  } restore{ctx};
  for (const Job& j : jobs) {
    BinHost& bin = *C.bins[j.bi];
    ProgDev* P = nullptr;
    lgx_status s = get_prog(ctx, bin.la, bin.lb, bin.lc, bin.ld, deriv, &P);
    if (s != LGX_OK) return s;
    const int sp = j.sp;
    const bool fp32 = j.fp32;
    const int kmode = fp32 ? mode32 : mode;
    EriArgs a = base;
    bin_args(C, bin, sp, a);
    a.prim_count = pr.count ? ctx->primcount.as<unsigned long long>() + 2 * j.bi + sp : nullptr;
    a.counter = counters ? counters + 2 * j.bi + sp : nullptr;
    const auto tv = ctx->tuned.find(tune_key(bin, deriv, kmode, fp32, ctx->op));
    const Variant v = tv != ctx->tuned.end()
                          ? tv->second
                          : default_variant(ctx, B, *P, kmode, fp32, true, bin.nq_avg);
    cudaStream_t st = ctx->stream;
    if (split) {
      const int b = j.branch;
      st = fp32 ? ctx->s32[b] : ctx->s64[b];
      // program-kernel slot scratch: one region per branch
      ctx->scratch = (fp32 || b > 0) ? &ctx->gscratch_br[(fp32 ? nbr : 0) + b] : &ctx->gscratch;
      if (!fp32 && mode32 >= 0) a.max_bps = ctx->fp64_bps;
      if (fp32) a.max_bps = ctx->fp32_bps;
    }
    ctx->launch_stream = st;
    const size_t li = pr.recs.size();
    if (pr.timed) CK(cudaEventRecordWithFlags(ctx->lev[2 * li], st, evflags));
    s = run_eri(ctx, B, *P, kmode, fp32, a, bin.total[sp], bin.nq_avg, &v);
    if (s != LGX_OK) return s;
    if (pr.timed) CK(cudaEventRecordWithFlags(ctx->lev[2 * li + 1], st, evflags));
    pr.integrals += bin.integrals[sp];
    ++pr.launches;
    pr.recs.push_back({int(j.bi), sp, fp32, v, kmode});
  }
  if (split) {
    for (int b = 0; b < nbr; ++b) {
      CK(cudaEventRecord(ctx->ev_join[2 * b], ctx->s64[b]));
      CK(cudaEventRecord(ctx->ev_join[2 * b + 1], ctx->s32[b]));
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[2 * b], 0));
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[2 * b + 1], 0));
    }
  }
  CK(cudaEventRecordWithFlags(ctx->ev1, ctx->stream, evflags));
  return LGX_OK;
}

// After the pass: per-launch statistics (device time between the launch
// events, quartets, primitive quartets, algorithmic FP operations), kept in
// ctx->last_launches and printed per class with LGX_CLASS_PROFILE=1 (the
// counterpart of libint's per-class Engine timers, engine.h:862-890), and
// the statistics of the whole pass.
bool class_profile();
lgx_status finish_bins(lgx_context* ctx, BasisDev& B, int deriv, bool allow_fp32,
                       const PassRecs& pr, lgx_jk_stats* stats) {
  BinCache& C = ctx->bins;
  const auto& recs = pr.recs;
  const size_t nslots = pr.nslots;
  CK(cudaEventSynchronize(ctx->ev1));
  std::vector<unsigned long long> pc(nslots, 0);
  if (pr.count)
    CK(cudaMemcpy(pc.data(), ctx->primcount.p, nslots * sizeof(unsigned long long),
                  cudaMemcpyDeviceToHost));
  ctx->last_launches.clear();
  long long prims = 0;
  double f64 = 0, f32 = 0;
  for (size_t i = 0; i < recs.size(); ++i) {
    const PassRec& r = recs[i];
    const BinHost& bin = *C.bins[r.bin];
    ProgDev* P = nullptr;
    lgx_status s = get_prog(ctx, bin.la, bin.lb, bin.lc, bin.ld, deriv, &P);
    if (s != LGX_OK) return s;
    const unsigned long long np = pc[2 * r.bin + r.sp];
    prims += (long long)np;
    const int pure[4] = {bin.la > 1, bin.lb > 1, bin.lc > 1, bin.ld > 1};
    const double q = double(bin.total[r.sp]);
    const int nsets = deriv ? 12 : 1;
    double nsph = 1;
    const int lq[4] = {bin.la, bin.lb, bin.lc, bin.ld};
    for (int k = 0; k < 4; ++k) nsph *= pure[k] ? 2 * lq[k] + 1 : ncart(lq[k]);
    // VRR + post stage + transform, then the prologue and the digestion,
    // which run in the launch's precision too (the FP64 Boys share of the
    // mixed scheme's FP32 kernels on the FP64 pipe)
    const bool b64 = mode_b64(r.mode);
    const double flops =
        double(np) * (double(P->host.vrr_flops) + prologue_flops(P->host.mmax, b64)) +
        q * (double(P->host.post_flops) + nsets * sph_flops(bin.la, bin.lb, bin.lc, bin.ld, pure) +
             nsets * 12.0 * nsph);
    const double flops_on64 = r.fp32 ? double(np) * prologue_flops64(P->host.mmax, b64) : flops;
    f64 += flops_on64;
    f32 += flops - flops_on64;
    lgx_launch_stats ls{};
    ls.la = bin.la; ls.lb = bin.lb; ls.lc = bin.lc; ls.ld = bin.ld;
    ls.fp32 = r.fp32 ? 1 : 0;
    ls.kernel = r.v.kind;
    ls.shape = r.v.kind == 0 ? r.v.group : r.v.rows;
    ls.deriv = deriv;
    ls.quartets = bin.total[r.sp];
    ls.prim_quartets = (long long)np;
    ls.integrals = (long long)(q * nsph);
    ls.flops = flops;
    ls.flops_fp64 = flops_on64;
    ls.ms = -1.0;
    if (pr.timed) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, ctx->lev[2 * i], ctx->lev[2 * i + 1]));
      ls.ms = ms;
      C.bins[r.bin]->last_ms[r.sp] = ms;
    }
    ctx->last_launches.push_back(ls);
    if (class_profile()) {
      char kind[32];
      if (r.v.kind == 0) snprintf(kind, sizeof(kind), "rk/G%d", r.v.group);
      else snprintf(kind, sizeof(kind), "%s/R%d", r.v.kind == 2 ? "gen" : "prog", r.v.rows);
      fprintf(stderr, "lgx-class (%d%d|%d%d) %s %s quartets %lld prims %.0f nq_avg %.1f  %.3f ms"
              "  %.1f GFLOP %.3f TFLOP/s\n",
              bin.la, bin.lb, bin.lc, bin.ld, r.fp32 ? "fp32" : "fp64", kind,
              (long long)bin.total[r.sp], double(np), bin.nq_avg, ls.ms, 1e-9 * flops,
              ls.ms > 0 ? 1e-9 * flops / ls.ms : 0.0);
    }
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    stats->flops_fp64 = f64;
    stats->flops_fp32 = f32;
    stats->quartets_fp64 = C.quartets[0] + (allow_fp32 ? 0 : C.quartets[1]);
    stats->quartets_fp32 = allow_fp32 ? C.quartets[1] : 0;
    stats->integrals = pr.integrals;
    stats->prim_quartets = prims;
    stats->kernel_ms = ms;
    stats->launches = pr.launches;
  }
  return LGX_OK;
}

bool class_profile() {
  static const bool prof = getenv("LGX_CLASS_PROFILE") && getenv("LGX_CLASS_PROFILE")[0] == '1';
  return prof;
}

lgx_status run_bins(lgx_context* ctx, BasisDev& B, int mode, int deriv, int mode32,
                    EriArgs base, lgx_jk_stats* stats) {
  PassRecs pr;
  lgx_status s = enqueue_bins(ctx, B, mode, deriv, mode32, base, pr);
  if (s != LGX_OK) return s;
  return finish_bins(ctx, B, deriv, mode32 >= 0, pr, stats);
}

// Cartesian component index and exponents in the standard order
// (cgshell_ordering.h:125-131): lx descending, then ly descending.
int cart_idx(int l, int lx, int ly) {
  const int i = l - lx;
  return i * (i + 1) / 2 + (i - ly);
}
void cart_exp(int l, int c, int* e) {
  int i = 0;
  while ((i + 1) * (i + 2) / 2 <= c) ++i;
  const int ly = i - (c - i * (i + 1) / 2);
  e[0] = l - i;
  e[1] = ly;
  e[2] = l - e[0] - e[1];
}

// The 78 second-derivative sets (libint's CartesianDerivIterator<4>(2)
// order) from the first-derivative sets d1 of the quartets with shell X
// raised (12 sets of su[X] values at offu[X]) and lowered (sd[X] values at
// offd[X]; l = 0 has none):
//   d/dY_j d/dX_i (..x..) = d/dY_j (..X'(x+1_i)..) - x_i d/dY_j (..X_(x-1_i)..)
// composed in Cartesian components, then transformed to solid harmonics
// for the pure shell X.  n[] are the caller's set dimensions, nv their
// product; the raised / lowered shells are Cartesian.
void compose_deriv2(const int lx[4], const int n[4], const int pure[4], const double* d1,
                    const int64_t offu[4], const int64_t offd[4], const size_t su[4],
                    const size_t sd[4], size_t nv, double* out) {
  std::vector<double> cart;
  int set = 0;
  for (int c1 = 0; c1 < 12; ++c1)
    for (int c2 = c1; c2 < 12; ++c2, ++set) {
      const int X = c1 / 3, i = c1 % 3;
      int dc[4] = {n[0], n[1], n[2], n[3]}, du[4] = {n[0], n[1], n[2], n[3]},
          dd[4] = {n[0], n[1], n[2], n[3]};
      dc[X] = ncart(lx[X]);
      du[X] = ncart(lx[X] + 1);
      dd[X] = lx[X] > 0 ? ncart(lx[X] - 1) : 0;
      const double* U = d1 + offu[X] + size_t(c2) * su[X];
      const double* Dn = lx[X] > 0 ? d1 + offd[X] + size_t(c2) * sd[X] : nullptr;
      cart.assign(size_t(dc[0]) * dc[1] * dc[2] * dc[3], 0.0);
      int ix[4];
      size_t o = 0;
      for (ix[0] = 0; ix[0] < dc[0]; ++ix[0])
        for (ix[1] = 0; ix[1] < dc[1]; ++ix[1])
          for (ix[2] = 0; ix[2] < dc[2]; ++ix[2])
            for (ix[3] = 0; ix[3] < dc[3]; ++ix[3], ++o) {
              int e[3];
              cart_exp(lx[X], ix[X], e);
              int iu[4] = {ix[0], ix[1], ix[2], ix[3]};
              int eu[3] = {e[0], e[1], e[2]};
              ++eu[i];
              iu[X] = cart_idx(lx[X] + 1, eu[0], eu[1]);
              double v = U[((size_t(iu[0]) * du[1] + iu[1]) * du[2] + iu[2]) * du[3] + iu[3]];
              if (e[i] > 0) {
                int id[4] = {ix[0], ix[1], ix[2], ix[3]};
                int ed[3] = {e[0], e[1], e[2]};
                --ed[i];
                id[X] = cart_idx(lx[X] - 1, ed[0], ed[1]);
                v -= e[i] * Dn[((size_t(id[0]) * dd[1] + id[1]) * dd[2] + id[2]) * dd[3] + id[3]];
              }
              cart[o] = v;
            }
      double* dst = out + size_t(set) * nv;
      if (!pure[X]) {
        std::memcpy(dst, cart.data(), nv * sizeof(double));
        continue;
      }
      size_t outer = 1, inner = 1;
      for (int t = 0; t < X; ++t) outer *= size_t(dc[t]);
      for (int t = X + 1; t < 4; ++t) inner *= size_t(dc[t]);
      const int ncx = dc[X], npx = 2 * lx[X] + 1;
      std::fill(dst, dst + nv, 0.0);
      for (size_t a = 0; a < outer; ++a)
        for (int p = 0; p < npx; ++p)
          for (int c = 0; c < ncx; ++c) {
            int e[3];
            cart_exp(lx[X], c, e);
            const double coef = solid_coeff(lx[X], p - lx[X], e[0], e[1], e[2]);
            if (coef == 0.0) continue;
            const double* src = &cart[(a * ncx + c) * inner];
            double* d = &dst[(a * npx + p) * inner];
            for (size_t b = 0; b < inner; ++b) d[b] += coef * src[b];
          }
    }
}

// deriv_order = 2 (Engine::compute2<coulomb, xx_xx, 2>): the 78 second-
// derivative shell sets, composed from first-derivative sets that the GPU
// computes in one batched launch.  With X' = shell X raised by one angular
// momentum quantum, Cartesian, every primitive coefficient times 2 alpha, and
// X_ = X lowered by one,
//   d/dY_j d/dX_i (..x..) = d/dY_j (..X'(x+1_i)..) - x_i d/dY_j (..X_(x-1_i)..)
// for every pair of centres (both factors act at the primitive level, so for
// Y = X the 2 alpha of X' multiplies the one the inner derivative brings).
// Sets in libint's order (CartesianDerivIterator<4>(2),
// include/libint2/deriv_iter.h: coordinate pairs c1 <= c2, row-major over
// A_x..D_z) and in the caller's shell order, so no derivative remap is
// needed; pure shells are transformed after the Cartesian composition.
// Shells up to LGX_MAX_L: the raised copies reach LGX_MAX_L + 1 (Cartesian
// class programs of kMaxLInternal).
lgx_status shellset_deriv2(lgx_context* ctx, const lgx_shell shells[4], double precision,
                           int screening, double* out, size_t out_capacity, int* nsets,
                           int* nvalues, int* is_null) {
  if (screening != LGX_SCREEN_ORIGINAL && screening != LGX_SCREEN_CONSERVATIVE)
    return fail(ctx, LGX_ERR_INVALID_ARG, "unsupported screening method");
  int lx[4], n[4];
  size_t nv = 1;
  for (int k = 0; k < 4; ++k) {
    if (!shells[k].alpha || !shells[k].coeff) return fail(ctx, LGX_ERR_INVALID_ARG, "null shell data");
    lx[k] = shells[k].l;
    if (lx[k] < 0 || lx[k] > kMaxL)
      return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "shell angular momentum exceeds LGX_MAX_L");
    n[k] = nfunc(lx[k], shells[k].pure ? 1 : 0);
    nv *= size_t(n[k]);
  }
  if (nv * 78 > out_capacity) return fail(ctx, LGX_ERR_TOO_LARGE, "output buffer too small");
  CK(cudaSetDevice(ctx->device));
  // small basis: 0-3 the shells, 4+X raised X, 8+X lowered X
  int l[12], pure[12], np[12], atom[12];
  double O[36];
  std::vector<double> al, co;
  auto push = [&](int k, int X, int dl, bool scale) {
    const lgx_shell& sh = shells[X];
    l[k] = sh.l + dl;
    pure[k] = dl == 0 ? (sh.pure ? 1 : 0) : 0;
    np[k] = sh.nprim;
    atom[k] = X;
    for (int x = 0; x < 3; ++x) O[3 * k + x] = sh.origin[x];
    for (int p = 0; p < sh.nprim; ++p) {
      al.push_back(sh.alpha[p]);
      co.push_back(scale ? 2.0 * sh.alpha[p] * sh.coeff[p] : sh.coeff[p]);
    }
  };
  // primitive data must follow the shell index order (upload_basis
  // derives the primitive offsets from it)
  for (int X = 0; X < 4; ++X) push(X, X, 0, false);
  for (int X = 0; X < 4; ++X) push(4 + X, X, +1, true);
  for (int X = 0; X < 4; ++X) push(8 + X, X, lx[X] > 0 ? -1 : 0, false);
  lgx_status s =
      upload_basis(ctx, ctx->small, 12, l, pure, np, atom, O, al.data(), co.data(), kMaxLInternal);
  if (s != LGX_OK) return s;
  const double ln_prec =
      precision > 0 ? std::log(precision) : -std::numeric_limits<double>::max();
  s = ensure_pairs(ctx, ctx->small, ln_prec, screening);
  if (s != LGX_OK) return s;
  // first-derivative sets of the raised / lowered quartets, one launch
  std::vector<int32_t> q;
  std::vector<int64_t> off;
  size_t su[4] = {0, 0, 0, 0}, sd[4] = {0, 0, 0, 0}, total = 0;
  int64_t offu[4] = {0, 0, 0, 0}, offd[4] = {-1, -1, -1, -1};
  for (int X = 0; X < 4; ++X)
    for (int dir = 0; dir < 2; ++dir) {
      if (dir == 1 && lx[X] == 0) continue;
      int qq[4] = {0, 1, 2, 3};
      qq[X] = (dir == 0 ? 4 : 8) + X;
      size_t sz = 12;
      for (int k = 0; k < 4; ++k) sz *= size_t(k == X ? ncart(l[qq[k]]) : n[k]);
      q.insert(q.end(), qq, qq + 4);
      off.push_back(int64_t(total));
      if (dir == 0) { offu[X] = int64_t(total); su[X] = sz / 12; }
      else { offd[X] = int64_t(total); sd[X] = sz / 12; }
      total += sz;
    }
  const long long nq = (long long)off.size();
  CK(ctx->out.ensure(std::max<size_t>(total, 1) * sizeof(double)));
  CK(ctx->isnull.ensure(size_t(nq) * sizeof(int)));
  CK(cudaMemsetAsync(ctx->out.p, 0, total * sizeof(double), ctx->stream));
  s = run_explicit(ctx, ctx->small, q.data(), nq, 1, kModeStore, 0.0, off.data(),
                   ctx->out.as<double>(), ctx->isnull.as<int>(), precision, screening, nullptr);
  if (s != LGX_OK) return s;
  std::vector<double> d1(total);
  std::vector<int> nul(nq);
  CK(cudaMemcpyAsync(d1.data(), ctx->out.p, total * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaMemcpyAsync(nul.data(), ctx->isnull.p, nq * sizeof(int), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  s = check_errflag(ctx);
  if (s != LGX_OK) return s;
  *nsets = 78;
  *nvalues = int(nv);
  bool all_null = true;
  for (int v : nul) all_null = all_null && v != 0;
  *is_null = all_null ? 1 : 0;
  if (all_null) return LGX_OK;
  int pure4[4];
  for (int k = 0; k < 4; ++k) pure4[k] = shells[k].pure ? 1 : 0;
  compose_deriv2(lx, n, pure4, d1.data(), offu, offd, su, sd, nv, out);
  return LGX_OK;
}


// Caller position of canonical shell k for shells of angular momenta l[]
// (la >= lb, lc >= ld, la + lb <= lc + ld; the same rule as canonicalize).
void canonical_perm(const int l[4], int perm[4], bool* stb, bool* stk, bool* sbk) {
  *stb = l[0] < l[1];
  *stk = l[2] < l[3];
  *sbk = l[0] + l[1] > l[2] + l[3];
  perm[0] = *sbk ? (*stk ? 3 : 2) : (*stb ? 1 : 0);
  perm[1] = *sbk ? (*stk ? 2 : 3) : (*stb ? 0 : 1);
  perm[2] = *sbk ? (*stb ? 1 : 0) : (*stk ? 3 : 2);
  perm[3] = *sbk ? (*stb ? 0 : 1) : (*stk ? 2 : 3);
}

// Enqueues one prim_set_kernel launch for (l[0] l[1]|l[2] l[3]) on
// ctx->stream: packs the caller's primitive quartets into staging rows in
// the canonical orientation (bra pair swap: P - B = PA + AB and B - A;
// ket pair swap likewise; bra-ket swap exchanges PA/QC, WP/WQ, zeta/eta
// factors and AB/CD), every (00|00)^(m) times the 2 alpha of caller
// centre `scale_ctr` when >= 0, and writes the sets to the device buffer
// d_out.  Returns the program's set count through *nsets_out.
lgx_status prim_set_launch(lgx_context* ctx, const int l[4], int deriv,
                           const lgx_prim_quartet* prims, int nprim, const double AB[3],
                           const double CD[3], int scale_ctr, double* d_out) {
  int perm[4];
  bool stb, stk, sbk;
  canonical_perm(l, perm, &stb, &stk, &sbk);
  ProgDev* P = nullptr;
  lgx_status s = get_prog(ctx, l[perm[0]], l[perm[1]], l[perm[2]], l[perm[3]], deriv, &P);
  if (s != LGX_OK) return s;
  const int mmax = l[0] + l[1] + l[2] + l[3] + deriv;
  if (mmax > kStMaxM) return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "(00|00)^(m) beyond m = 15");
  double ab[3], cd[3];
  for (int x = 0; x < 3; ++x) {
    ab[x] = stb ? -AB[x] : AB[x];
    cd[x] = stk ? -CD[x] : CD[x];
  }
  std::vector<double> rows(size_t(nprim) * kStage, 0.0);
  for (int p = 0; p < nprim; ++p) {
    const lgx_prim_quartet& q = prims[p];
    double* st = &rows[size_t(p) * kStage];
    double pa[3], qc[3], wp[3], wq[3];
    for (int x = 0; x < 3; ++x) {
      pa[x] = stb ? q.PA[x] + AB[x] : q.PA[x];
      qc[x] = stk ? q.QC[x] + CD[x] : q.QC[x];
      wp[x] = q.WP[x];
      wq[x] = q.WQ[x];
    }
    double z = q.oo2z, e = q.oo2e, rz = q.roz, re = q.roe;
    if (sbk) {
      for (int x = 0; x < 3; ++x) {
        std::swap(pa[x], qc[x]);
        std::swap(wp[x], wq[x]);
      }
      std::swap(z, e);
      std::swap(rz, re);
    }
    const double w = scale_ctr >= 0 ? q.two_alpha[scale_ctr] : 1.0;
    for (int m = 0; m <= mmax; ++m) st[kStF + m] = w * q.ss[m];
    for (int x = 0; x < 3; ++x) {
      st[kStPA + x] = pa[x];
      st[kStWP + x] = wp[x];
      st[kStQC + x] = qc[x];
      st[kStWQ + x] = wq[x];
    }
    st[kStOo2z] = z;
    st[kStRoz] = rz;
    st[kStOo2e] = e;
    st[kStRoe] = re;
    st[kStOo2ze] = q.oo2ze;
    st[kStW + 0] = q.two_alpha[perm[0]];
    st[kStW + 1] = q.two_alpha[perm[1]];
    st[kStW + 2] = q.two_alpha[perm[3]];
  }
  if (sbk)
    for (int x = 0; x < 3; ++x) std::swap(ab[x], cd[x]);
  PrimSetArgs a{};
  a.prog = P->dev;
  a.nrows = nprim;
  a.stage_rows = 32;
  for (int x = 0; x < 3; ++x) {
    a.AB[x] = ab[x];
    a.CD[x] = cd[x];
  }
  for (int k = 0; k < 4; ++k) a.perm[k] = perm[k];
  a.out = d_out;
  CK(ctx->prim_rows.ensure(std::max<size_t>(rows.size(), 1) * sizeof(double)));
  // pageable source: the copy has read `rows` when cudaMemcpyAsync returns
  CK(cudaMemcpyAsync(ctx->prim_rows.p, rows.data(), rows.size() * sizeof(double),
                     cudaMemcpyHostToDevice, ctx->stream));
  a.rows = ctx->prim_rows.as<double>();
  a.slot_stride = (P->host.total_slots() + 1) & ~1;
  const size_t slot_bytes = size_t(a.slot_stride) * sizeof(double);
  const size_t smem_cap = std::min<size_t>(ctx->smem_optin, 200 * 1024);
  // many rows of a small class: whole rows per warp (8 staged rows each),
  // no block-wide barrier per recurrence level
  const size_t per_warp = stage_bytes_per_warp(false, 8) + slot_bytes;
  size_t smem;
  if (nprim >= 8 && (kBlockThreads / 32) * per_warp <= smem_cap) {
    a.warp_rows = 1;
    a.stage_rows = 8;
    smem = (kBlockThreads / 32) * per_warp;
  } else {
    a.warp_rows = 0;
    const size_t stage = stage_bytes_per_warp(false, a.stage_rows);
    smem = stage + slot_bytes;
    if (smem > smem_cap) {  // slots in global memory (L1/L2 resident)
      CK(ctx->prim_slots.ensure(slot_bytes));
      a.slots = ctx->prim_slots.as<double>();
      smem = stage;
    }
  }
  CK(launch_prim_set(a, smem, ctx->stream));
  return LGX_OK;
}

// lgx_compute_primitive_set: one launch (deriv 0/1), or the first-
// derivative sets of the raised / lowered quartets and the composition
// (deriv 2).
lgx_status primitive_set(lgx_context* ctx, const int l[4], int deriv,
                         const lgx_prim_quartet* prims, int nprim, const double AB[3],
                         const double CD[3], double* out, size_t out_capacity, int* nsets,
                         int* nvalues) {
  int n[4];
  size_t nv = 1;
  for (int k = 0; k < 4; ++k) {
    if (l[k] < 0 || l[k] > kMaxL)
      return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "shell angular momentum beyond the build's limit");
    n[k] = ncart(l[k]);
    nv *= size_t(n[k]);
  }
  const int ns = deriv == 0 ? 1 : (deriv == 1 ? 12 : 78);
  if (nv * ns > out_capacity) return fail(ctx, LGX_ERR_TOO_LARGE, "output buffer too small");
  *nsets = ns;
  *nvalues = int(nv);
  if (nprim == 0) {
    std::fill(out, out + nv * ns, 0.0);
    return LGX_OK;
  }
  CK(cudaSetDevice(ctx->device));
  if (deriv < 2) {
    CK(ctx->out.ensure(nv * ns * sizeof(double)));
    lgx_status s = prim_set_launch(ctx, l, deriv, prims, nprim, AB, CD, -1, ctx->out.as<double>());
    if (s != LGX_OK) return s;
    CK(cudaMemcpyAsync(out, ctx->out.p, nv * ns * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return LGX_OK;
  }
  // deriv 2: raised (weights 2 a_X) and lowered quartets, first derivatives
  int64_t offu[4] = {0, 0, 0, 0}, offd[4] = {0, 0, 0, 0};
  size_t su[4] = {0, 0, 0, 0}, sd[4] = {0, 0, 0, 0}, total = 0;
  for (int X = 0; X < 4; ++X) {
    su[X] = nv / size_t(n[X]) * size_t(ncart(l[X] + 1));
    offu[X] = int64_t(total);
    total += 12 * su[X];
    if (l[X] > 0) {
      sd[X] = nv / size_t(n[X]) * size_t(ncart(l[X] - 1));
      offd[X] = int64_t(total);
      total += 12 * sd[X];
    }
  }
  CK(ctx->out.ensure(total * sizeof(double)));
  double* d1 = ctx->out.as<double>();
  for (int X = 0; X < 4; ++X) {
    int lu[4] = {l[0], l[1], l[2], l[3]};
    ++lu[X];
    lgx_status s = prim_set_launch(ctx, lu, 1, prims, nprim, AB, CD, X, d1 + offu[X]);
    if (s != LGX_OK) return s;
    if (l[X] > 0) {
      int ld[4] = {l[0], l[1], l[2], l[3]};
      --ld[X];
      s = prim_set_launch(ctx, ld, 1, prims, nprim, AB, CD, -1, d1 + offd[X]);
      if (s != LGX_OK) return s;
    }
  }
  std::vector<double> h(total);
  CK(cudaMemcpyAsync(h.data(), d1, total * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const int pure[4] = {0, 0, 0, 0};
  compose_deriv2(l, n, pure, h.data(), offu, offd, su, sd, nv, out);
  return LGX_OK;
}

}  // namespace

// =================================================================== C ABI
extern "C" {

const char* lgx_version(void) { return kVersion; }

const char* lgx_last_error(const lgx_context* ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

lgx_status lgx_create(lgx_context** out, int device) {
  if (!out) return LGX_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev)
    return LGX_ERR_NO_DEVICE;
  auto ctx = std::make_unique<lgx_context>();
  lgx_context* c = ctx.get();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return LGX_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return LGX_ERR_NO_DEVICE;
  if (prop.major < 10) return LGX_ERR_NO_DEVICE;
  ctx->nsm = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  {
    lgx_context* ctx = c;  // for CK
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    CK(cudaEventCreate(&c->ev2));
    CK(cudaEventCreate(&c->ev3));
    for (int b = 0; b < lgx_context::kMaxBranches; ++b) {
      CK(cudaStreamCreateWithFlags(&c->s64[b], cudaStreamNonBlocking));
      CK(cudaStreamCreateWithFlags(&c->s32[b], cudaStreamNonBlocking));
    }
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    for (auto& e : c->ev_join) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const auto boys = make_boys_table();
    const auto sph = make_sph_table();
    CK(c->boys.ensure(boys.size() * sizeof(double)));
    CK(cudaMemcpy(c->boys.p, boys.data(), boys.size() * sizeof(double), cudaMemcpyHostToDevice));
    {
      // pre-divided Taylor coefficients F_{m+i}(T_k)/i!
      std::vector<double> tay(size_t(kBoysRows) * (kBoysMaxM + 1) * kBoysTaylorStride, 0.0);
      for (int k = 0; k < kBoysRows; ++k)
        for (int m = 0; m <= kBoysMaxM; ++m) {
          double f = 1;
          for (int i = 0; i < 7; ++i) {
            if (i > 0) f *= i;
            tay[(size_t(k) * (kBoysMaxM + 1) + m) * kBoysTaylorStride + i] =
                boys[size_t(k) * kBoysCols + m + i] / f;
          }
          if (m == 0)
            tay[size_t(k) * (kBoysMaxM + 1) * kBoysTaylorStride + 7] =
                double(expl(-(long double)k * kBoysDT));
        }
      CK(c->boys_tay.ensure(tay.size() * sizeof(double)));
      CK(cudaMemcpy(c->boys_tay.p, tay.data(), tay.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    {
      // sparse solid-harmonic rows
      std::vector<int> off(4 * 9, 0), cidx;
      std::vector<double> cd;
      std::vector<float> cf;
      for (int l = 0; l <= 3; ++l) {
        const int nc = ncart(l);
        for (int p = 0; p <= 2 * l; ++p) {
          off[l * 9 + p] = int(cidx.size());
          for (int c2 = 0; c2 < nc; ++c2) {
            const double v = sph[sph_off(l) + p * nc + c2];
            if (v != 0.0) {
              cidx.push_back(c2);
              cd.push_back(v);
              cf.push_back(float(v));
            }
          }
        }
        off[l * 9 + 2 * l + 1] = int(cidx.size());
      }
      CK(c->sph_off.ensure(off.size() * sizeof(int)));
      CK(c->sph_c.ensure(cidx.size() * sizeof(int)));
      CK(c->sph_cd.ensure(cd.size() * sizeof(double)));
      CK(c->sph_cf.ensure(cf.size() * sizeof(float)));
      CK(cudaMemcpy(c->sph_off.p, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(c->sph_c.p, cidx.data(), cidx.size() * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(c->sph_cd.p, cd.data(), cd.size() * sizeof(double), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(c->sph_cf.p, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    std::vector<float> boysf(boys.begin(), boys.end());
    CK(c->boys32.ensure(boysf.size() * sizeof(float)));
    CK(cudaMemcpy(c->boys32.p, boysf.data(), boysf.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (const char* e = getenv("LGX_DISABLE_RK")) c->use_rk = (e[0] == '0');
    if (const char* e = getenv("LGX_DISABLE_POST")) c->use_post = (e[0] == '0');
    if (const char* e = getenv("LGX_TUNE")) c->tune = (e[0] != '0');
    if (const char* e = getenv("LGX_GRAPHS")) c->use_graphs = (e[0] != '0');
    if (const char* e = getenv("LGX_OVERLAP")) c->overlap = (e[0] != '0');
    if (const char* e = getenv("LGX_FP64_BPS")) c->fp64_bps = std::max(0, atoi(e));
    if (const char* e = getenv("LGX_FP32_BPS")) c->fp32_bps = std::max(0, atoi(e));
    if (const char* e = getenv("LGX_BRANCHES")) c->branches = std::max(1, atoi(e));
    if (const char* e = getenv("LGX_BRANCH_POLICY")) c->branch_policy = std::min(2, std::max(0, atoi(e)));
    if (const char* e = getenv("LGX_TUNE_MIN")) c->tune_min = std::max(1LL, atoll(e));

    {
      double h[40];
      for (int m = 0; m < 40; ++m) h[m] = 1.0 / (2 * m + 1);
      CK(c->inv_odd.ensure(sizeof(h)));
      CK(cudaMemcpy(c->inv_odd.p, h, sizeof(h), cudaMemcpyHostToDevice));
    }
    CK(c->counter.ensure(64));
    CK(c->errflag.ensure(64));
    CK(c->primcount.ensure(64));
    CK(cudaMemset(c->errflag.p, 0, 64));
  }
  *out = ctx.release();
  return LGX_OK;
}

lgx_status lgx_destroy(lgx_context* ctx) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev2) cudaEventDestroy(ctx->ev2);
  if (ctx->ev3) cudaEventDestroy(ctx->ev3);
  if (ctx->jk_exec) cudaGraphExecDestroy(ctx->jk_exec);
  for (cudaEvent_t e : ctx->lev) cudaEventDestroy(e);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  for (cudaEvent_t e : ctx->ev_join)
    if (e) cudaEventDestroy(e);
  std::vector<cudaStream_t> side;
  for (int b = 0; b < lgx_context::kMaxBranches; ++b) {
    side.push_back(ctx->s64[b]);
    side.push_back(ctx->s32[b]);
  }
  cudaStream_t st = ctx->stream;
  delete ctx;
  if (st) cudaStreamDestroy(st);
  for (cudaStream_t x : side)
    if (x) cudaStreamDestroy(x);
  return LGX_OK;
}

}  // extern "C"

namespace {
// One shell set (deriv 0 / 1) of four caller shells; pair_ln: NULL, or the
// screening logarithms of the bra (shells 0, 1) and ket (shells 2, 3)
// primitive pairs (a caller's ShellPair data) in place of ln(precision).
lgx_status shellset_locked(lgx_context* ctx, const lgx_shell shells[4], int deriv,
                           double precision, int screening, const double* pair_ln, double* out,
                           size_t out_capacity, int* nsets, int* nvalues, int* is_null) {
  if (deriv < 0 || deriv > kMaxDeriv)
    return fail(ctx, LGX_ERR_INVALID_ARG, "deriv must be 0, 1 or 2");
  if (screening != LGX_SCREEN_ORIGINAL && screening != LGX_SCREEN_CONSERVATIVE)
    return fail(ctx, LGX_ERR_INVALID_ARG, "unsupported screening method");
  CK(cudaSetDevice(ctx->device));
  int l[4], pure[4], np[4], atom[4] = {0, 1, 2, 3};
  double O[12];
  std::vector<double> al, co;
  long long nv = 1;
  for (int k = 0; k < 4; ++k) {
    const lgx_shell& s = shells[k];
    if (!s.alpha || !s.coeff) return fail(ctx, LGX_ERR_INVALID_ARG, "null shell data");
    l[k] = s.l;
    pure[k] = s.pure ? 1 : 0;
    np[k] = s.nprim;
    for (int x = 0; x < 3; ++x) O[3 * k + x] = s.origin[x];
    al.insert(al.end(), s.alpha, s.alpha + s.nprim);
    co.insert(co.end(), s.coeff, s.coeff + s.nprim);
    if (s.l < 0 || s.l > kMaxL)
      return fail(ctx, LGX_ERR_LMAX_EXCEEDED, "shell angular momentum exceeds LGX_MAX_L");
    nv *= nfunc(s.l, pure[k]);
  }
  const int ns = deriv ? 12 : 1;
  if (size_t(nv * ns) > out_capacity)
    return fail(ctx, LGX_ERR_TOO_LARGE, "output buffer too small");
  lgx_status s = upload_basis(ctx, ctx->small, 4, l, pure, np, atom, O, al.data(), co.data());
  if (s != LGX_OK) return s;
  const double ln_prec =
      precision > 0 ? std::log(precision) : -std::numeric_limits<double>::max();
  if (!pair_ln) {
    s = ensure_pairs(ctx, ctx->small, ln_prec, screening);
    if (s != LGX_OK) return s;
  } else {
    // the table at the tighter of the two, then the other pair cut to its own
    // (the small basis holds shells 0..3: pairs (1, 0) and (3, 2))
    BasisDev& B = ctx->small;
    const double lb = pair_ln[0], lk = pair_ln[1];
    s = ensure_pairs(ctx, B, std::min(lb, lk), screening);
    if (s != LGX_OK) return s;
    const PairRec& pb = B.hpairs[pidx(1, 0)];
    const PairRec& pk = B.hpairs[pidx(3, 2)];
    PrimPairRec* pp = B.pprims.as<PrimPairRec>();
    if (lb > lk) CK(launch_drop_pairs(pp + pb.pp_off, pb.npp, lb, ctx->stream));
    if (lk > lb) CK(launch_drop_pairs(pp + pk.pp_off, pk.npp, lk, ctx->stream));
    B.pairs_ok = lb == lk;  // a cut table is not reused
  }
  CK(ctx->out.ensure(size_t(nv * ns) * sizeof(double)));
  CK(ctx->isnull.ensure(sizeof(int)));
  const int32_t q[4] = {0, 1, 2, 3};
  s = run_explicit(ctx, ctx->small, q, 1, deriv, kModeStore, 0.0, nullptr, ctx->out.as<double>(),
                   ctx->isnull.as<int>(), precision, screening, nullptr);
  if (s != LGX_OK) return s;
  int nul = 0;
  CK(cudaMemcpyAsync(&nul, ctx->isnull.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->out.p, size_t(nv * ns) * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  s = check_errflag(ctx);
  if (s != LGX_OK) return s;
  *nsets = ns;
  *nvalues = int(nv);
  *is_null = nul;
  return LGX_OK;
}
}  // namespace

extern "C" {

lgx_status lgx_compute_shellset(lgx_context* ctx, const lgx_shell shells[4], int deriv,
                                double precision, int screening, double* out,
                                size_t out_capacity, int* nsets, int* nvalues, int* is_null) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!shells || !out || !nsets || !nvalues || !is_null)
    return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (deriv == 2)
    return shellset_deriv2(ctx, shells, precision, screening, out, out_capacity, nsets, nvalues,
                           is_null);
  return shellset_locked(ctx, shells, deriv, precision, screening, nullptr, out, out_capacity,
                         nsets, nvalues, is_null);
}

lgx_status lgx_compute_shellset_pairs(lgx_context* ctx, const lgx_shell shells[4], int deriv,
                                      double precision, int screening,
                                      const double pair_ln_prec[2], double* out,
                                      size_t out_capacity, int* nsets, int* nvalues,
                                      int* is_null) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!shells || !out || !nsets || !nvalues || !is_null || !pair_ln_prec)
    return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (deriv != 0 && deriv != 1)
    return fail(ctx, LGX_ERR_INVALID_ARG, "caller pair data: deriv must be 0 or 1");
  if (std::isnan(pair_ln_prec[0]) || std::isnan(pair_ln_prec[1]))
    return fail(ctx, LGX_ERR_INVALID_ARG, "pair precision is NaN");
  return shellset_locked(ctx, shells, deriv, precision, screening, pair_ln_prec, out,
                         out_capacity, nsets, nvalues, is_null);
}

double lgx_solid_coeff(int l, int m, int lx, int ly, int lz) {
  if (l < 0 || lx < 0 || ly < 0 || lz < 0 || lx + ly + lz != l || m < -l || m > l) return 0.0;
  return solid_coeff(l, m, lx, ly, lz);
}

lgx_status lgx_compute_primitive_set(lgx_context* ctx, int l1, int l2, int l3, int l4,
                                     int deriv, const lgx_prim_quartet* prims, int nprim,
                                     const double AB[3], const double CD[3], double* out,
                                     size_t out_capacity, int* nsets, int* nvalues) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!AB || !CD || !out || !nsets || !nvalues || nprim < 0 || (nprim > 0 && !prims))
    return fail(ctx, LGX_ERR_INVALID_ARG, "null argument or negative primitive count");
  if (deriv < 0 || deriv > 2)
    return fail(ctx, LGX_ERR_INVALID_ARG, "deriv must be 0, 1 or 2");
  const int l[4] = {l1, l2, l3, l4};
  return primitive_set(ctx, l, deriv, prims, nprim, AB, CD, out, out_capacity, nsets, nvalues);
}

lgx_status lgx_set_basis(lgx_context* ctx, int nshell, const int32_t* l, const int32_t* pure,
                         const int32_t* nprim, const int32_t* atom, const double* origins,
                         const double* alpha, const double* coeff) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  ctx->bins.valid = false;
  ctx->tuned.clear();
  ctx->pair_subset.clear();  // pair indices refer to the previous basis
  ++ctx->subset_version;
  ++ctx->version;
  return upload_basis(ctx, ctx->basis, nshell, l, pure, nprim, atom, origins, alpha, coeff);
}

lgx_status lgx_set_pair_subset(lgx_context* ctx, const int32_t* pairs, int64_t n) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  const int ns = ctx->basis.nshell;
  if (ns == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  if (n < 0 || (n > 0 && !pairs)) return fail(ctx, LGX_ERR_INVALID_ARG, "bad pair list");
  std::vector<unsigned char> mask;
  if (n > 0) {
    mask.assign(size_t(ns) * (ns + 1) / 2, 0);
    for (int64_t i = 0; i < n; ++i) {
      const int a = pairs[2 * i], b = pairs[2 * i + 1];
      if (a < 0 || b < 0 || a >= ns || b >= ns)
        return fail(ctx, LGX_ERR_INVALID_ARG, "shell index out of range in the pair list");
      mask[pidx(std::max(a, b), std::min(a, b))] = 1;
    }
  }
  ctx->pair_subset.swap(mask);
  ++ctx->subset_version;
  ++ctx->version;
  return LGX_OK;
}

lgx_status lgx_basis_nbf(lgx_context* ctx, int* nbf) {
  if (!ctx || !nbf) return LGX_ERR_INVALID_ARG;
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  *nbf = ctx->basis.nbf;
  return LGX_OK;
}

lgx_status lgx_schwarz(lgx_context* ctx, double* K) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!K) return fail(ctx, LGX_ERR_INVALID_ARG, "null output");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  CK(cudaSetDevice(ctx->device));
  BasisDev& B = ctx->basis;
  lgx_status s = ensure_schwarz(ctx, B);
  if (s != LGX_OK) return s;
  const int n = B.nshell;
  for (int s1 = 0; s1 < n; ++s1)
    for (int s2 = 0; s2 <= s1; ++s2)
      K[(size_t)s1 * n + s2] = K[(size_t)s2 * n + s1] = B.Kpair[pidx(s1, s2)];
  return LGX_OK;
}

// lgx_compute_batch / lgx_compute_batch_device: `out` / `is_null` are host
// memory (copied from the context's buffers) or, for `device_out`, device
// memory the kernels write directly.
static lgx_status compute_batch(lgx_context* ctx, const int32_t* quartets, int64_t n,
                                int deriv, int mode, double mixed_thresh, const int64_t* offsets,
                                double* out, size_t out_capacity, int32_t* is_null,
                                bool device_out) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!quartets || n < 0 || !out) return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  if (deriv < 0 || deriv > kMaxDeriv) return fail(ctx, LGX_ERR_INVALID_ARG, "bad deriv");
  if (!valid_mode(mode)) return fail(ctx, LGX_ERR_INVALID_ARG, "bad mode");
  if (mixed_mode(mode) && deriv) return fail(ctx, LGX_ERR_INVALID_ARG, "mixed mode is deriv 0");
  CK(cudaSetDevice(ctx->device));
  BasisDev& B = ctx->basis;
  size_t need = 0;
  for (int64_t q = 0; q < n; ++q) {
    long long nv = 1;
    for (int k = 0; k < 4; ++k) {
      const int s = quartets[4 * q + k];
      if (s < 0 || s >= B.nshell) return fail(ctx, LGX_ERR_INVALID_ARG, "shell index out of range");
      nv *= nfunc(B.l[s], B.pure[s]);
    }
    nv *= deriv ? 12 : 1;
    const size_t end = size_t((offsets ? offsets[q] : (int64_t)need) + nv);
    need = offsets ? std::max(need, end) : end;
  }
  if (need > out_capacity) return fail(ctx, LGX_ERR_TOO_LARGE, "output buffer too small");
  lgx_status s;
  if (mixed_mode(mode)) {
    s = ensure_schwarz(ctx, B);
    if (s != LGX_OK) return s;
  }
  const double eps = std::numeric_limits<double>::epsilon();
  s = ensure_pairs(ctx, B, std::log(eps), 0);
  if (s != LGX_OK) return s;
  double* d_out = out;
  int* d_isnull = reinterpret_cast<int*>(is_null);
  if (!device_out) {
    CK(ctx->out.ensure(std::max<size_t>(need, 1) * sizeof(double)));
    d_out = ctx->out.as<double>();
  }
  if (!device_out || !is_null) {
    CK(ctx->isnull.ensure(std::max<int64_t>(n, 1) * sizeof(int)));
    d_isnull = ctx->isnull.as<int>();
  }
  CK(cudaMemsetAsync(d_out, 0, std::max<size_t>(need, 1) * sizeof(double), ctx->stream));
  s = run_explicit(ctx, B, quartets, n, deriv, kModeStore,
                   mixed_mode(mode) ? mixed_thresh : 0.0, offsets, d_out, d_isnull, eps, 0,
                   nullptr, mixed_mode(mode) ? fp32_kernel_mode(ctx, mode, kModeStore) : kModeStore);
  if (s != LGX_OK) return s;
  if (!device_out) {
    CK(cudaMemcpyAsync(out, d_out, need * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (is_null)
      CK(cudaMemcpyAsync(is_null, d_isnull, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return check_errflag(ctx);
}

lgx_status lgx_compute_batch(lgx_context* ctx, const int32_t* quartets, int64_t n, int deriv,
                             int mode, double mixed_thresh, const int64_t* offsets, double* out,
                             size_t out_capacity, int32_t* is_null) {
  return compute_batch(ctx, quartets, n, deriv, mode, mixed_thresh, offsets, out, out_capacity,
                       is_null, false);
}

lgx_status lgx_compute_batch_device(lgx_context* ctx, const int32_t* quartets, int64_t n,
                                    int deriv, int mode, double mixed_thresh,
                                    const int64_t* offsets, double* d_out, size_t out_capacity,
                                    int32_t* d_is_null) {
  return compute_batch(ctx, quartets, n, deriv, mode, mixed_thresh, offsets, d_out, out_capacity,
                       d_is_null, true);
}

}  // extern "C"

namespace {
// Body of lgx_jk_device; the caller holds ctx->mu.
lgx_status jk_device_locked(lgx_context* ctx, const double* dD, double* dJ, double* dK,
                            double thresh, int mode, double mixed, lgx_jk_stats* stats) {
  if (!dD || !dJ || !dK) return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  if (!valid_mode(mode)) return fail(ctx, LGX_ERR_INVALID_ARG, "bad mode");
  CK(cudaSetDevice(ctx->device));
  BasisDev& B = ctx->basis;
  lgx_status s = ensure_schwarz(ctx, B);
  if (s != LGX_OK) return s;
  // both mixed modes split the quartets alike; they differ in the kernels
  const bool mixedp = mixed_mode(mode);
  const int mode32 = fp32_kernel_mode(ctx, mode, kModeJK);
  s = build_bins(ctx, B, thresh, mixedp ? LGX_MIXED : LGX_FP64, mixedp ? mixed : 0.0);
  if (s != LGX_OK) return s;
  const double eps = std::numeric_limits<double>::epsilon();
  s = ensure_pairs(ctx, B, std::log(eps), 0);
  if (s != LGX_OK) return s;
  s = ensure_jk_records(ctx, B);
  if (s != LGX_OK) return s;
  const size_t nn = size_t(B.nbf) * B.nbf;
  CK(ctx->Jacc.ensure(nn * sizeof(double)));
  CK(ctx->Kacc.ensure(nn * sizeof(double)));
  if (mixedp) CK(ctx->Df.ensure(nn * sizeof(float)));
  const bool dscreen = ctx->fock_prec > 0.0;
  if (dscreen) CK(ctx->Dsh.ensure(size_t(B.nshell) * B.nshell * sizeof(double)));
  EriArgs a{};
  a.precision = eps;
  a.ln_prec = std::log(eps);
  a.screening = 0;
  a.D = dD;
  a.Df = ctx->Df.as<float>();
  a.Jacc = ctx->Jacc.as<double>();
  a.Kacc = ctx->Kacc.as<double>();
  a.nbf = B.nbf;
  if (dscreen) {
    a.dsh = ctx->Dsh.as<double>();
    a.kpair = B.Kd.as<double>();
    a.fock_prec = ctx->fock_prec;
  }
  if (mixedp) CK(launch_d2f(dD, ctx->Df.as<float>(), (long long)nn, ctx->stream));
  if (dscreen) CK(launch_shell_block_norm(B.dev, dD, B.nbf, ctx->Dsh.as<double>(), ctx->stream));
  s = tune_bins(ctx, B, kModeJK, 0, mode32, a);
  if (s != LGX_OK) return s;
  // the pass: zero the accumulators, FP32 copy of D, every class bin, J/K
  auto enqueue = [&](PassRecs& pr) -> lgx_status {
    CK(cudaMemsetAsync(ctx->Jacc.p, 0, nn * sizeof(double), ctx->stream));
    CK(cudaMemsetAsync(ctx->Kacc.p, 0, nn * sizeof(double), ctx->stream));
    if (mixedp) CK(launch_d2f(dD, ctx->Df.as<float>(), (long long)nn, ctx->stream));
    if (dscreen) CK(launch_shell_block_norm(B.dev, dD, B.nbf, ctx->Dsh.as<double>(), ctx->stream));
    lgx_status r = enqueue_bins(ctx, B, kModeJK, 0, mode32, a, pr);
    if (r != LGX_OK) return r;
    CK(launch_jk_finalize(ctx->Jacc.as<double>(), ctx->Kacc.as<double>(), dJ, dK, B.nbf,
                          ctx->stream));
    return LGX_OK;
  };
  // A pass whose key (pointers, settings, bins, tuning) matches the last
  // captured one replays its CUDA graph; otherwise it runs eagerly (which
  // also makes every allocation) and is then captured for the next call.
  PassKey key;
  const void* kp[] = {dD, dJ, dK, ctx->Df.p, ctx->Jacc.p, ctx->Kacc.p, ctx->gscratch.p,
                      ctx->primcount.p, ctx->scratch_sig()};
  for (int i = 0; i < 9; ++i) key.ptr[i] = kp[i];
  key.thresh = thresh;
  key.mixed = mixedp ? mixed : 0.0;
  key.mode = mode;
  key.version = ctx->version;
  const bool graphable = ctx->use_graphs;
  const bool replay = graphable && ctx->jk_exec && ctx->jk_key == key;
  CK(cudaEventRecord(ctx->ev2, ctx->stream));
  if (replay) {
    CK(cudaGraphLaunch(ctx->jk_exec, ctx->stream));
  } else {
    s = enqueue(ctx->jk_recs);
    if (s != LGX_OK) return s;
  }
  CK(cudaEventRecord(ctx->ev3, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  s = finish_bins(ctx, B, 0, mixedp, ctx->jk_recs, stats);
  if (s != LGX_OK) return s;
  float pass_ms = 0;
  CK(cudaEventElapsedTime(&pass_ms, ctx->ev2, ctx->ev3));
  s = check_errflag(ctx);
  if (s != LGX_OK) return s;
  if (!replay && graphable && key.ptr[6] == ctx->gscratch.p && key.ptr[7] == ctx->primcount.p &&
      key.ptr[8] == ctx->scratch_sig()) {
    if (ctx->jk_exec) {
      cudaGraphExecDestroy(ctx->jk_exec);
      ctx->jk_exec = nullptr;
    }
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    PassRecs tmp;
    const lgx_status cs = enqueue(tmp);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (cs != LGX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return cs;
    }
    if (ce != cudaSuccess) return fail(ctx, LGX_ERR_CUDA, cudaGetErrorString(ce));
    const cudaError_t ie = cudaGraphInstantiate(&ctx->jk_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      ctx->jk_exec = nullptr;
      return fail(ctx, LGX_ERR_CUDA, cudaGetErrorString(ie));
    }
    ctx->jk_key = key;
    ctx->jk_recs = tmp;  // replays follow the captured launch order
  }
  if (stats) {
    stats->pass_ms = pass_ms;
    stats->launches += 1;
  }
  return LGX_OK;
}
}  // namespace

extern "C" {

lgx_status lgx_jk_device(lgx_context* ctx, const double* dD, double* dJ, double* dK,
                         double thresh, int mode, double mixed, lgx_jk_stats* stats) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return jk_device_locked(ctx, dD, dJ, dK, thresh, mode, mixed, stats);
}

}  // extern "C"

namespace {
// Scratch of lgx_jk_device_noalloc: J and K accumulators (FP64) and the
// FP32 copy of D for nbf <= LGX_NOALLOC_MAX_NBF, one array per device that
// loads the library.  Host code only ever uses its device address, looked
// up once per device with cudaGetSymbolAddress.
constexpr size_t kNoAllocN = size_t(LGX_NOALLOC_MAX_NBF) * LGX_NOALLOC_MAX_NBF;
constexpr size_t kNoAllocBytes = 2 * kNoAllocN * sizeof(double) + kNoAllocN * sizeof(float);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
std::map<int, unsigned char*> g_noalloc_addr;  // device -> address of the array

lgx_status noalloc_scratch(lgx_context* ctx, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  auto it = g_noalloc_addr.find(ctx->device);
  if (it != g_noalloc_addr.end()) {
    *out = it->second;
    return LGX_OK;
  }
  void* p = nullptr;
  CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  g_noalloc_addr[ctx->device] = static_cast<unsigned char*>(p);
  *out = static_cast<unsigned char*>(p);
  return LGX_OK;
}

struct NoAllocGuard {
  lgx_context* c;
  explicit NoAllocGuard(lgx_context* ctx) : c(ctx) { c->noalloc = true; }
  ~NoAllocGuard() {
    c->noalloc = false;
    c->scratch = nullptr;
  }
};
}  // namespace

extern "C" {

lgx_status lgx_jk_device_noalloc(lgx_context* ctx, const double* dD, double* dJ, double* dK,
                                 double thresh, int mode, double mixed, lgx_jk_stats* stats) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!dD || !dJ || !dK) return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  if (!valid_mode(mode)) return fail(ctx, LGX_ERR_INVALID_ARG, "bad mode");
  BasisDev& B = ctx->basis;
  if (B.nbf > LGX_NOALLOC_MAX_NBF)
    return fail(ctx, LGX_ERR_TOO_LARGE,
                "lgx_jk_device_noalloc: nbf = " + std::to_string(B.nbf) +
                    " exceeds LGX_NOALLOC_MAX_NBF = " + std::to_string(LGX_NOALLOC_MAX_NBF));
  const double eps = std::numeric_limits<double>::epsilon();
  const BinCache& C = ctx->bins;
  const bool mixedp = mixed_mode(mode);
  const int mode32 = fp32_kernel_mode(ctx, mode, kModeJK);
  const double mixed_key = mixedp ? mixed : 0.0;
  if (!B.schwarz_ok || !B.pairs_ok || B.pairs_lnprec != std::log(eps) || B.pairs_method != 0 ||
      !C.valid || C.thresh != thresh || C.mode != (mixedp ? LGX_MIXED : LGX_FP64) ||
      C.mixed != mixed_key ||
      C.subset_version != ctx->subset_version)
    return fail(ctx, LGX_ERR_INVALID_ARG,
                "lgx_jk_device_noalloc: basis state not prepared for these settings; call "
                "lgx_jk_device (or lgx_jk) once with the same threshold and mode first");
  const bool dscreen = ctx->fock_prec > 0.0;
  if (dscreen && ctx->Dsh.n < size_t(B.nshell) * B.nshell * sizeof(double))
    return fail(ctx, LGX_ERR_INVALID_ARG,
                "lgx_jk_device_noalloc: density screening not prepared; call lgx_jk_device "
                "once with the same settings first");
  CK(cudaSetDevice(ctx->device));
  unsigned char* scratch = nullptr;
  lgx_status s = noalloc_scratch(ctx, &scratch);
  if (s != LGX_OK) return s;
  NoAllocGuard guard(ctx);
  s = ensure_jk_records(ctx, B);
  if (s != LGX_OK) return s;
  const size_t nn = size_t(B.nbf) * B.nbf;
  double* Jacc = reinterpret_cast<double*>(scratch);
  double* Kacc = Jacc + kNoAllocN;
  float* Df = reinterpret_cast<float*>(Kacc + kNoAllocN);
  // The prepared pass ran its program-kernel launches on parallel branches,
  // each growing its own slot scratch; this pass runs every launch on
  // ctx->stream one after another, so the largest of those buffers serves
  // all of them (plan_launch clamps each grid to it).
  DBuf* slot_scratch = &ctx->gscratch;
  for (DBuf& b : ctx->gscratch_br)
    if (b.n > slot_scratch->n) slot_scratch = &b;
  ctx->scratch = slot_scratch;
  CK(cudaEventRecord(ctx->ev2, ctx->stream));
  CK(cudaMemsetAsync(Jacc, 0, nn * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(Kacc, 0, nn * sizeof(double), ctx->stream));
  if (mixedp) CK(launch_d2f(dD, Df, (long long)nn, ctx->stream));
  EriArgs a{};
  a.precision = eps;
  a.ln_prec = std::log(eps);
  a.screening = 0;
  a.D = dD;
  a.Df = Df;
  a.Jacc = Jacc;
  a.Kacc = Kacc;
  a.nbf = B.nbf;
  if (dscreen) {
    a.dsh = ctx->Dsh.as<double>();
    a.kpair = B.Kd.as<double>();
    a.fock_prec = ctx->fock_prec;
    CK(launch_shell_block_norm(B.dev, dD, B.nbf, ctx->Dsh.as<double>(), ctx->stream));
  }
  s = run_bins(ctx, B, kModeJK, 0, mode32, a, stats);
  if (s != LGX_OK) return s;
  CK(launch_jk_finalize(Jacc, Kacc, dJ, dK, B.nbf, ctx->stream));
  CK(cudaEventRecord(ctx->ev3, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (stats) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev2, ctx->ev3));
    stats->pass_ms = ms;
    stats->launches += 1;
  }
  return check_errflag(ctx);
}

lgx_status lgx_jk(lgx_context* ctx, const double* D, double* J, double* K, double thresh,
                  int mode, double mixed, lgx_jk_stats* stats) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  // one lock over the copy in, the pass and the copy out, so that two
  // threads sharing a context cannot interleave their D, J and K
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!D || !J || !K) return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  const size_t nn = size_t(ctx->basis.nbf) * ctx->basis.nbf;
  CK(cudaSetDevice(ctx->device));
  CK(ctx->Dd.ensure(nn * sizeof(double)));
  CK(ctx->Jd.ensure(nn * sizeof(double)));
  CK(ctx->Kd.ensure(nn * sizeof(double)));
  CK(cudaMemcpyAsync(ctx->Dd.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  lgx_status s = jk_device_locked(ctx, ctx->Dd.as<double>(), ctx->Jd.as<double>(),
                                  ctx->Kd.as<double>(), thresh, mode, mixed, stats);
  if (s != LGX_OK) return s;
  CK(cudaMemcpyAsync(J, ctx->Jd.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(K, ctx->Kd.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LGX_OK;
}

lgx_status lgx_set_operator(lgx_context* ctx, int op, double omega) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (op != LGX_OP_COULOMB && op != LGX_OP_ERF_COULOMB && op != LGX_OP_ERFC_COULOMB)
    return fail(ctx, LGX_ERR_INVALID_ARG, "unknown operator");
  if (!(omega >= 0.0) || !std::isfinite(omega))
    return fail(ctx, LGX_ERR_INVALID_ARG, "omega must be finite and >= 0");
  if (op == LGX_OP_COULOMB) omega = 0.0;
  if (op == ctx->op && omega == ctx->omega) return LGX_OK;
  ctx->op = op;
  ctx->omega = omega;
  // Schwarz factors, quartet bins and the captured pass depend on the operator
  ctx->basis.schwarz_ok = false;
  ctx->bins.valid = false;
  ++ctx->version;
  return LGX_OK;
}

lgx_status lgx_boys(lgx_context* ctx, int variant, const double* T, int64_t n, int mmax,
                    double* F) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (variant < 0 || variant > 6) return fail(ctx, LGX_ERR_INVALID_ARG, "bad Boys variant");
  const int mmax_cap = (variant == 1 || variant == 3 || variant >= 5) ? 6 : kBoysMaxM;
  if (mmax < 0 || mmax > mmax_cap)
    return fail(ctx, LGX_ERR_INVALID_ARG, "mmax out of range for this evaluator");
  if (n < 0 || (n > 0 && (!T || !F))) return fail(ctx, LGX_ERR_INVALID_ARG, "bad arrays");
  if (n == 0) return LGX_OK;
  const int64_t nin = variant == 6 ? 8 * n : n;  // variant 6: pair data per argument
  if (variant == 6) {
    // |P| <= 1e4 bohr, 1e-10 <= zeta <= 1e10: the double-float records'
    // range (and a Boys argument that stays finite)
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 8; ++c) {
        const double v = T[8 * i + c];
        const bool ok = (c % 4 == 3) ? (v >= 1e-10 && v <= 1e10) : (std::fabs(v) <= 1e4);
        if (!ok) return fail(ctx, LGX_ERR_INVALID_ARG, "pair data out of range");
      }
  } else {
    for (int64_t i = 0; i < n; ++i)  // the table lookup needs 0 <= T (NaN rejected too)
      if (!(T[i] >= 0.0) || !std::isfinite(T[i]))
        return fail(ctx, LGX_ERR_INVALID_ARG, "Boys argument T must be finite and >= 0");
  }
  CK(cudaSetDevice(ctx->device));
  const size_t nf = size_t(n) * (mmax + 1);
  CK(ctx->boysT.ensure(size_t(nin) * sizeof(double)));
  CK(ctx->boysF.ensure(nf * sizeof(double)));
  CK(cudaMemcpyAsync(ctx->boysT.p, T, size_t(nin) * sizeof(double), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(launch_boys_eval(ctx->boys.as<double>(), ctx->boys_tay.as<double>(), ctx->boys32.as<float>(),
                      ctx->inv_odd.as<double>(), variant, ctx->boysT.as<double>(), n, mmax,
                      ctx->boysF.as<double>(), ctx->stream));
  CK(cudaMemcpyAsync(F, ctx->boysF.p, nf * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return LGX_OK;
}

lgx_status lgx_set_fock_precision(lgx_context* ctx, double precision) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!(precision >= 0.0) || !std::isfinite(precision))
    return fail(ctx, LGX_ERR_INVALID_ARG, "Fock precision must be finite and >= 0");
  if (precision == ctx->fock_prec) return LGX_OK;
  ctx->fock_prec = precision;
  ++ctx->version;  // a launch argument of the captured pass
  return LGX_OK;
}

lgx_status lgx_set_watchdog(lgx_context* ctx, int64_t max_chunks) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (max_chunks < 0) max_chunks = -1;
  if (max_chunks == ctx->watchdog_chunks) return LGX_OK;
  ctx->watchdog_chunks = max_chunks;
  ++ctx->version;  // the bound is a launch argument of the captured pass
  return LGX_OK;
}

lgx_status lgx_last_pass_launches(lgx_context* ctx, lgx_launch_stats* out, int max, int* n) {
  if (!ctx || !n || max < 0 || (max > 0 && !out)) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  const int cnt = int(ctx->last_launches.size());
  *n = cnt;
  for (int i = 0; i < cnt && i < max; ++i) out[i] = ctx->last_launches[i];
  return LGX_OK;
}

lgx_status lgx_jk_grad(lgx_context* ctx, const double* D, double* gJ, double* gK, int natoms,
                       double thresh, lgx_jk_stats* stats) {
  if (!ctx) return LGX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!D || !gJ || !gK) return fail(ctx, LGX_ERR_INVALID_ARG, "null argument");
  if (ctx->basis.nshell == 0) return fail(ctx, LGX_ERR_NO_BASIS, "no basis set");
  BasisDev& B = ctx->basis;
  if (natoms < B.natoms) return fail(ctx, LGX_ERR_INVALID_ARG, "natoms smaller than atom count");
  CK(cudaSetDevice(ctx->device));
  lgx_status s = ensure_schwarz(ctx, B);
  if (s != LGX_OK) return s;
  s = build_bins(ctx, B, thresh, LGX_FP64, 0.0);
  if (s != LGX_OK) return s;
  const double eps = std::numeric_limits<double>::epsilon();
  s = ensure_pairs(ctx, B, std::log(eps), 0);
  if (s != LGX_OK) return s;
  s = ensure_jk_records(ctx, B);
  if (s != LGX_OK) return s;
  const size_t nn = size_t(B.nbf) * B.nbf;
  CK(ctx->Dd.ensure(nn * sizeof(double)));
  CK(ctx->gJ.ensure(3 * natoms * sizeof(double)));
  CK(ctx->gK.ensure(3 * natoms * sizeof(double)));
  CK(cudaMemcpyAsync(ctx->Dd.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->gJ.p, 0, 3 * natoms * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->gK.p, 0, 3 * natoms * sizeof(double), ctx->stream));
  EriArgs a{};
  a.precision = eps;
  a.ln_prec = std::log(eps);
  a.D = ctx->Dd.as<double>();
  a.gJ = ctx->gJ.as<double>();
  a.gK = ctx->gK.as<double>();
  a.nbf = B.nbf;
  s = tune_bins(ctx, B, kModeGrad, 1, -1, a);
  if (s != LGX_OK) return s;
  s = run_bins(ctx, B, kModeGrad, 1, -1, a, stats);
  if (s != LGX_OK) return s;
  CK(cudaMemcpyAsync(gJ, ctx->gJ.p, 3 * natoms * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaMemcpyAsync(gK, ctx->gK.p, 3 * natoms * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_errflag(ctx);
}

}  // extern "C"
