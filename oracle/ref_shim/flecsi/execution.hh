// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include "flecsi/data.hh"
#include "flecsi/flog.hh"
#include "flecsi/util/array_ref.hh"
namespace flecsi {
struct scheduler { static scheduler* instance; template<class... A> void execute(A&&...); template<class... A> int reduce(A&&...); };
struct mpi_t{}; inline constexpr mpi_t mpi{};
// a task launch (only named by code that is not run here)
template<auto F, auto... A, class... Args> void execute(Args&&...) {}
#ifndef FLECSI_INLINE_TARGET
#define FLECSI_INLINE_TARGET inline
#endif
namespace exec { struct on_t{}; inline constexpr on_t on{}; namespace fold { struct sum{}; struct min{}; struct max{}; }
  struct executor_t { template<class R> executor_t forall_(R&&); executor_t named(const char*); };
  struct launch_t { int index; }; struct accelerator { executor_t executor(); launch_t launch(); }; struct cpu { }; }
namespace run { struct context { static context& instance(); int process(); }; }
}
#define forall(it, R) forall_(R) ->* [&](auto it)
#define reduceall(it, up, R, F, T) forall_(R) ->* [&](auto it, auto up)
