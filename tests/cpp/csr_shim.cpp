// Host test shim: the event schedules' adjacency builder (pir_csr.h) behind a
// C entry point, for tests/test_csr.py.
#include "../../lala-pc_gb300/csrc/pir_csr.h"

extern "C" void csr_build(long long n, int nv, const int *x, const int *y, const int *z, int *ptr, int *adj,
                          int nthreads) {
  pirgpu::build_adjacency(n, nv, x, y, z, ptr, adj, nthreads);
}

extern "C" int csr_threads(long long n, int requested) { return pirgpu::adjacency_threads(n, requested); }

extern "C" int pc_adjacency(int np, const int *roots, const int *tape, int nv, int *ptr, int *adj, int cap,
                            int nthreads) {
  std::vector<int32_t> a;
  pirgpu::build_formula_adjacency(np, roots, tape, nv, ptr, a, nthreads);
  if ((int)a.size() > cap) return -1;
  std::copy(a.begin(), a.end(), adj);
  return (int)a.size();
}
