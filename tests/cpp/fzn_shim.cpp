// Test helper: the FlatZinc front end (include/pirgpu_fzn.hpp) behind a C
// function, so that the Python tests can compile a model without a GPU and
// run it on the oracle.  Output text: "nvars nprops", one "lb ub name" line
// per variable ("-" for generated ones), one "op x y z" line per propagator.
#include <cstdio>
#include <cstring>
#include <string>

#include "pirgpu_fzn.hpp"

extern "C" int fzn_compile(const char *text, char *out, int cap) {
  lala_gpu::fzn::Model m;
  lala_gpu::IDiagnostics d;
  std::string s;
  if (!lala_gpu::fzn::compile(text, m, d)) {
    for (const auto &e : d.errors) s += e + "\n";
    std::snprintf(out, (size_t)cap, "%s", s.c_str());
    return 1;
  }
  s = std::to_string(m.dom.size()) + " " + std::to_string(m.props.size()) + "\n";
  for (size_t v = 0; v < m.dom.size(); ++v)
    s += std::to_string(m.dom[v].lb) + " " + std::to_string(m.dom[v].ub) + " " +
         (m.name[v].empty() ? std::string("-") : m.name[v]) + "\n";
  for (const auto &p : m.props)
    s += std::to_string((int)p.op) + " " + std::to_string(p.x) + " " + std::to_string(p.y) + " " +
         std::to_string(p.z) + "\n";
  if ((int)s.size() + 1 > cap) return 2;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return 0;
}
