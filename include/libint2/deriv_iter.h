// libint2::FixedOrderedIntegerPartitionIterator and CartesianDerivIterator
// (the reference's include/libint2/util/intpart_iter.h and deriv_iter.h):
// the order in which libint lays out geometric-derivative shell sets, so
// that code digesting derivative integrals (gradients, Hessians) indexes
// them the same way against this library.
//
// The iterator enumerates the partitions of n into k non-negative ordered
// parts: it starts at (n, 0, ..., 0); to advance, when the parts after the
// first already hold their last arrangement (everything in the final part)
// one unit moves from the first part to the second and the rest restart at
// their first arrangement, otherwise the parts after the first advance.
// For CartesianDerivIterator<NCenters>(d) the parts are the 3 NCenters
// Cartesian coordinates of the centres and n = d, so d = 1 gives A_x, A_y,
// ..., D_z and d = 2 the coordinate pairs c1 <= c2 row-major.  Names and
// semantics (operator*, next, last, operator bool = last, range_size, rank)
// follow the reference so that caller code compiles unchanged.
#ifndef LGX_LIBINT2_DERIV_ITER_H
#define LGX_LIBINT2_DERIV_ITER_H

#include <array>
#include <cstddef>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace libint2 {

namespace detail {
template <class T>
struct static_size : std::false_type {};
template <class T, std::size_t N>
struct static_size<std::array<T, N>> : std::true_type {};
}  // namespace detail

template <typename Sequence>
class FixedOrderedIntegerPartitionIterator {
 public:
  typedef const Sequence& value_type;
  typedef typename Sequence::value_type integer_type;
  typedef typename Sequence::size_type size_type;
  static_assert(std::is_integral<integer_type>::value, "partitions of integers");

  /// fixed-size sequences (std::array): k = the array size
  template <typename S = Sequence,
            typename std::enable_if<detail::static_size<S>::value, int>::type = 0>
  explicit FixedOrderedIntegerPartitionIterator(std::size_t n) : n_(n) {
    part_.fill(integer_type(0));
    part_[0] = integer_type(n);
  }
  /// resizable sequences: k parts
  template <typename S = Sequence,
            typename std::enable_if<!detail::static_size<S>::value, int>::type = 0>
  FixedOrderedIntegerPartitionIterator(std::size_t n, size_type k) : n_(n) {
    if (k == 0) throw std::invalid_argument("FixedOrderedIntegerPartitionIterator: k > 0");
    part_.assign(k, integer_type(0));
    part_[0] = integer_type(n);
  }

  value_type operator*() const { return part_; }
  const Sequence* operator->() const { return &part_; }
  /// as in the reference: true at the last partition
  operator bool() const { return last(); }
  bool last() const { return is_last(part_.data(), part_.size()); }
  void next() { advance(part_.data(), part_.size()); }

  /// number of partitions: C(n + k - 1, n)
  intmax_t range_size() const {
    return count(intmax_t(n_), intmax_t(part_.size()));
  }

  /// position of `p` in the enumeration (0 for (n, 0, ..., 0))
  template <typename Seq>
  static intmax_t rank(const Seq& p) {
    const intmax_t k = intmax_t(p.size());
    intmax_t rest = 0;
    for (intmax_t i = 0; i < k; ++i) rest += intmax_t(p[size_type(i)]);
    intmax_t r = 0;
    for (intmax_t i = 0; i + 1 < k; ++i) {
      const intmax_t v = intmax_t(p[size_type(i)]);
      // partitions of `rest` whose part i exceeds v come first
      for (intmax_t w = rest; w > v; --w) r += count(rest - w, k - i - 1);
      rest -= v;
    }
    return r;
  }

 private:
  std::size_t n_;
  Sequence part_;

  // partitions of m into j ordered non-negative parts: C(m + j - 1, m)
  static intmax_t count(intmax_t m, intmax_t j) {
    if (j <= 0) return m == 0 ? 1 : 0;
    intmax_t c = 1;
    for (intmax_t d = 1; d <= m; ++d) c = c * (j + d - 1) / d;
    return c;
  }
  static bool is_last(const integer_type* p, size_type k) {
    const auto total = std::accumulate(p, p + k, std::uintmax_t(0));
    return std::uintmax_t(p[k - 1]) == total;
  }
  static void advance(integer_type* p, size_type k) {
    if (k <= 1) return;
    if (is_last(p + 1, k - 1)) {
      const auto tail = std::accumulate(p + 1, p + k, integer_type(0));
      --p[0];
      for (size_type i = 1; i < k; ++i) p[i] = integer_type(0);
      p[1] = integer_type(tail + 1);
    } else {
      advance(p + 1, k - 1);
    }
  }
};

/// geometric derivatives of order d over NCenters centres, in libint's order
template <unsigned int NCenters>
using CartesianDerivIterator =
    FixedOrderedIntegerPartitionIterator<std::array<unsigned int, NCenters * 3>>;

}  // namespace libint2

#endif
