// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include <cstddef>
namespace flecsi {
using PrivilegeCount = unsigned short; using privilege = unsigned; using Privileges = unsigned;
inline constexpr privilege na = 0, ro = 1, wo = 2, rw = 3;
template<Privileges A, Privileges B> inline constexpr Privileges privilege_cat = 0;
template<privilege P, PrivilegeCount N> inline constexpr Privileges privilege_repeat = 0;
namespace data { enum class layout { dense, single };
  template<class T, layout L, class Topo, typename Topo::index_space S> struct field_reference;
  template<class T, Privileges P> struct topology_accessor; }
template<class T, data::layout L = data::layout::dense> struct field;
template<class T> struct topology;
}
namespace flecsi::topo { template<auto S> using id = std::size_t; }
