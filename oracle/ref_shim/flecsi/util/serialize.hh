// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include <cstddef>
namespace flecsi::util::serial { template<class T, class = void> struct traits; template<class T, class P> void put(P&, const T&...); template<class T> T get(const std::byte*&); }
