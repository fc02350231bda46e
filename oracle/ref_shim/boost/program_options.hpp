// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include "boost/program_options/options_description.hpp"
namespace boost::program_options {
struct variables_map {}; struct option { std::vector<std::string> original_tokens; };
struct parsed_options { std::vector<option> options; };
enum collect_unrecognized_mode { include_positional, exclude_positional };
inline parsed_options parse_config_file(const char*, const options_description&, bool) { return {}; }
inline void store(const parsed_options&, variables_map&) {} inline void notify(variables_map&) {}
inline std::vector<std::string> collect_unrecognized(const std::vector<option>&, collect_unrecognized_mode) { return {}; }
}
