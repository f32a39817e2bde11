/* Minimal stand-in for libint2/initialize.h: only the solid-harmonics
 * ordering switch and the verbosity accessors that Shell/solidharmonics use.
 * Test-only shim. */
#ifndef LGX_REF_SHIM_INITIALIZE_H
#define LGX_REF_SHIM_INITIALIZE_H
#include <libint2/shgshell_ordering.h>
#include <atomic>
#include <iostream>
namespace libint2 {
inline SHGShellOrdering solid_harmonics_ordering() {
  return SHGShellOrdering_Standard;
}
inline bool verbose() { return false; }
inline std::ostream& verbose_stream() { return std::clog; }
inline bool initialized() { return true; }
inline void initialize(bool = false) {}
}  // namespace libint2
#endif
