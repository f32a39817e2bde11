// Shared declarations of the register-resident (thread-per-quartet) kernels.
#pragma once
#include "lgx_kernels.cuh"

namespace lgx {
namespace rk {

// VRR geometric factors of one primitive quartet (engine.impl.h:1514-1701).
template <typename T>
struct Geo {
  T PAx, PAy, PAz, WPx, WPy, WPz, QCx, QCy, QCz, WQx, WQy, WQz;
  T oo2z, roz, oo2e, roe, oo2ze;
};

}  // namespace rk
}  // namespace lgx
