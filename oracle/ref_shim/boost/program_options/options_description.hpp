// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include <string>
#include <vector>
#include <functional>
namespace boost::program_options {
struct value_semantic { virtual ~value_semantic() = default; };
template<class T> struct typed_value : value_semantic { T* t; explicit typed_value(T* t):t(t){}
  typed_value* required() { return this; }
  typed_value* default_value(const T& v) { *t = v; return this; }
  typed_value* default_value(const T& v, const std::string&) { *t = v; return this; }
  typed_value* notifier(std::function<void(const T&)>) { return this; }
  typed_value* multitoken() { return this; } };
template<class T> typed_value<T>* value(T* t = nullptr) { return new typed_value<T>(t); }
struct options_description;
struct options_init { options_description* d;
  options_init& operator()(const char*, value_semantic*, const char*) { return *this; } };
struct options_description { options_init add_options() { return {this}; } options_description& add(const options_description&) { return *this; } };
}
