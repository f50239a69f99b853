// Host test shim: the event schedules' adjacency builder (pir_csr.h) behind a
// C entry point, for tests/test_csr.py.
#include "../../lala-pc_gb300/csrc/pir_csr.h"

extern "C" void csr_build(long long n, int nv, const int *x, const int *y, const int *z, int *ptr, int *adj,
                          int nthreads) {
  pirgpu::build_adjacency(n, nv, x, y, z, ptr, adj, nthreads);
}

extern "C" int csr_threads(long long n, int requested) { return pirgpu::adjacency_threads(n, requested); }
