// Minimal stand-in for the {fmt} header, just enough for the reference's
// geometry headers and the few reference sources oracle/ref_harness.cpp
// compiles.  It formats nothing: format() returns the format string itself.
// Used only to build oracle/_ref (test infrastructure).
#ifndef XDG_ORACLE_FMT_SHIM_H
#define XDG_ORACLE_FMT_SHIM_H

#include <string>

namespace fmt {

struct format_context {
  int out() { return 0; }
};

template <typename T, typename Char = char, typename Enable = void>
struct formatter {
  template <typename Ctx>
  int format(const T&, Ctx&) const { return 0; }
};

template <typename... Args>
std::string format(const std::string& s, const Args&...) { return s; }

template <typename Out, typename... Args>
Out format_to(Out o, const std::string&, const Args&...) { return o; }

} // namespace fmt

#endif
