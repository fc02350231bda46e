// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  flog writes to stderr; flog_assert
// throws so the driver can report the failed assertion instead of aborting.
#pragma once
#include <iostream>
#include <stdexcept>
#define flog(lvl) std::cerr << "[" #lvl "] "
#define flog_assert(c, m) do { if(!(c)) { throw std::runtime_error(m); } } while(0)
#define flog_warn(m) (std::cerr << "[warn] " << (m) << std::endl)
#define flog_error(m) (std::cerr << "[error] " << (m) << std::endl)
