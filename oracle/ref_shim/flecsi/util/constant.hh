// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include <array>
#include <cstddef>
namespace flecsi::util { template<auto V> struct constant { static constexpr auto value = V; };
template<auto... V> struct constants { static constexpr std::size_t size = sizeof...(V); };
// an array indexed by the (unscoped enum) keys of a constants<> list
template<class T, class Keys> struct key_array : std::array<T, Keys::size> {}; }
