// Test helper: the FlatZinc front end for PC (include/pirgpu_fzn_pc.hpp)
// behind C functions, so that the Python tests compile the models of lala-pc's
// PC tests without a GPU and run them on the oracle or on the engine.  A
// handle holds one model; each pcfzn_compile adds to it and reports what it
// added as text:
//   "nvars0 nvars nmeets nnodes nprops"
//   one "lb ub name" line per new variable,
//   one "var lb ub" line per store meet on an older variable,
//   one "kind a b c" line per tape node (indices local to this call),
//   one root index per new propagator.
#include <cstdio>
#include <cstring>
#include <string>

#include "pirgpu_fzn_pc.hpp"

extern "C" void *pcfzn_new() { return new lala_gpu::fzn::PcModel(); }
extern "C" void pcfzn_free(void *h) { delete static_cast<lala_gpu::fzn::PcModel *>(h); }

extern "C" int pcfzn_compile(void *h, const char *text, char *out, int cap) {
  auto &m = *static_cast<lala_gpu::fzn::PcModel *>(h);
  lala_gpu::IDiagnostics d;
  std::string s;
  if (!lala_gpu::fzn::compile_pc(text, m, d)) {
    for (const auto &e : d.errors) s += e + "\n";
    std::snprintf(out, (size_t)cap, "%s", s.c_str());
    return 1;
  }
  lala_gpu::pc::TapeWriter w;
  for (size_t i = m.nprops0; i < m.props.size(); ++i) w.prop(m.props[i]);
  s = std::to_string(m.nvars0) + " " + std::to_string(m.dom.size()) + " " + std::to_string(m.meets.size()) + " " +
      std::to_string(w.kind.size()) + " " + std::to_string(w.roots.size()) + "\n";
  for (size_t v = m.nvars0; v < m.dom.size(); ++v)
    s += std::to_string(m.dom[v].lb) + " " + std::to_string(m.dom[v].ub) + " " + m.name[v] + "\n";
  for (const auto &mt : m.meets)
    s += std::to_string(mt.first) + " " + std::to_string(mt.second.lb) + " " + std::to_string(mt.second.ub) + "\n";
  for (size_t i = 0; i < w.kind.size(); ++i)
    s += std::to_string(w.kind[i]) + " " + std::to_string(w.a[i]) + " " + std::to_string(w.b[i]) + " " +
         std::to_string(w.c[i]) + "\n";
  for (int32_t r : w.roots) s += std::to_string(r) + "\n";
  if ((int)s.size() + 1 > cap) return 2;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return 0;
}
