// Kernel argument structures shared by the launchers (lgx_api.cu) and the
// kernels (lgx_kernels.cu).
#pragma once
#include "lgx_device.cuh"

namespace lgx {

enum KernelMode : int {
  kModeStore = 0,    // write shell sets in libint buffer order
  kModeSchwarz = 1,  // K(pair) = sqrt(max |(ab|ab)|)
  kModeJK = 2,       // digest into J/K accumulators (deriv 0)
  kModeGrad = 3      // digest first derivatives into gJ/gK (deriv 1)
};

// Explicit work item: one shell quartet in canonical orientation.
struct QuartetItem {
  int bra_pair, ket_pair;  // pair-table indices
  int flags;               // bit0 bra swapped, bit1 ket swapped,
                           // bits 2..4 (swap_braket, swap_tbra, swap_tket)
  int pad;
  long long out;           // output offset (doubles) or K index (Schwarz)
};

// Implicit work (one class bin of the screened J/K quartet space).
struct BinWork {
  const int* bra_pairs;     // pair ids of the bra class, sorted by K desc
  const int* ket_pairs;     // pair ids of the ket class, sorted by K desc
  const long long* row_start;  // [nbra+1] prefix sums of per-row counts
  const int* row_j0;        // first ket index of each row in this space
  int nbra;
  int pad;
  long long total;
};

struct EriArgs {
  DevBasis basis;
  const PairRec* pairs;
  const PrimPairRec* pprims;
  const unsigned char* pair_swap;  // per pair: 1 if its canonical bra1 is s2
  DevProg prog;
  const double* boys;
  const float* boys32;   // FP32 copy of the Boys table
  const double* sph;
  // screening
  double precision, ln_prec;
  int screening;  // 0 Original, 1 Conservative
  // work
  const QuartetItem* items;
  long long nitems;
  BinWork bin;
  int implicit;   // 1: use bin, 0: use items
  int chunk;
  int group;           // register kernels: lanes per quartet (power of 2)
  unsigned long long* counter;
  // slots
  int slot_stride;     // slots per warp (elements of T)
  int global_slots;    // 1: slots live in gscratch
  void* gscratch;      // [nwarps_total][slot_stride] of T
  // outputs
  double* out;         // kModeStore
  int* is_null;        // kModeStore, per item (may be null)
  double* kschwarz;    // kModeSchwarz
  const double* D;     // kModeJK / kModeGrad
  const float* Df;     // FP32 copy of D (FP32 register kernels)
  double* Jacc;
  double* Kacc;
  double* gJ;
  double* gK;
  int nbf;
  // watchdog: a bounded number of work chunks per warp
  long long max_chunks;
  int* error_flag;
  // statistics
  unsigned long long* prim_count;
};

}  // namespace lgx
