// Host test shim: the event schedules' adjacency builder (pir_csr.h) behind a
// C entry point, for tests/test_csr.py.
#include "../../lala-pc_gb300/csrc/pir_csr.h"

extern "C" void csr_build(long long n, int nv, const int *x, const int *y, const int *z, int *ptr, int *adj,
                          int nthreads) {
  pirgpu::build_adjacency(n, nv, x, y, z, ptr, adj, nthreads);
}

extern "C" int csr_threads(long long n, int requested, long long nvars) {
  return pirgpu::adjacency_threads(n, requested, nvars);
}

extern "C" int pc_adjacency(int np, const int *roots, const int *tape, int nv, int *ptr, int *adj, int cap,
                            int nthreads) {
  std::vector<int32_t> a;
  pirgpu::build_formula_adjacency(np, roots, tape, nv, ptr, a, nthreads);
  if ((int)a.size() > cap) return -1;
  std::copy(a.begin(), a.end(), adj);
  return (int)a.size();
}

#include <numeric>

#include "../../lala-pc_gb300/csrc/pir_sort.h"

// The install order: a permutation of 0 .. n-1 stably sorted by (op, y, x, z).
extern "C" void install_order(int n, const int *op, const int *x, const int *y, const int *z, int *perm,
                              int nthreads) {
  std::vector<int> p((size_t)n);
  std::iota(p.begin(), p.end(), 0);
  pirgpu::parallel_stable_sort(p, [&](int a, int b) {
    if (op[a] != op[b]) return op[a] < op[b];
    if (y[a] != y[b]) return y[a] < y[b];
    if (x[a] != x[b]) return x[a] < x[b];
    return z[a] < z[b];
  }, nthreads);
  std::copy(p.begin(), p.end(), perm);
}
