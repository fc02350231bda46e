// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
