// Host test shim: the event schedules' adjacency builder (pir_csr.h) behind a
// C entry point, for tests/test_csr.py.
#include "../../lala-pc_gb300/csrc/pir_csr.h"

extern "C" int csr_build(long long n, int nv, const int *x, const int *y, const int *z, int *ptr, int *adj,
                         int nthreads) {
  return pirgpu::build_adjacency(n, nv, x, y, z, ptr, adj, nthreads) ? 1 : 0;
}

extern "C" int csr_threads(long long n, int requested, long long nvars) {
  return pirgpu::adjacency_threads(n, requested, nvars);
}

extern "C" int pc_adjacency(int np, const int *roots, const int *tape, int nv, int *ptr, int *adj, int cap,
                            int nthreads) {
  std::vector<int32_t> a;
  if (!pirgpu::build_formula_adjacency(np, roots, tape, nv, ptr, a, nthreads)) return -2;
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

#include "../../lala-pc_gb300/csrc/pir_segments.h"

// The path segments of a bytecode (pir_segments.h): seg_build keeps the result
// and reports the sizes of its arrays; seg_get copies one array out.
static pirgpu::Segments g_seg;

extern "C" int seg_build(long long n, int nv, const int *op, const int *x, const int *y, const int *z, int nthreads,
                         long long *sizes) {
  std::vector<int> ptr((size_t)nv + 1), adj((size_t)(3 * n));
  if (!pirgpu::build_adjacency(n, nv, x, y, z, ptr.data(), adj.data(), nthreads)) return -1;
  if (!pirgpu::build_segments(n, nv, op, x, y, z, ptr.data(), adj.data(), nthreads, g_seg)) return -1;
  sizes[0] = (long long)g_seg.seg_of.size();
  sizes[1] = (long long)g_seg.pptr.size();
  sizes[2] = (long long)g_seg.code.size();
  sizes[3] = (long long)g_seg.prop.size();
  sizes[4] = (long long)g_seg.vptr.size();
  sizes[5] = (long long)g_seg.var.size();
  sizes[6] = (long long)g_seg.umask.size();
  sizes[7] = (long long)g_seg.uptr.size();
  sizes[8] = (long long)g_seg.uadj.size();
  sizes[9] = (long long)g_seg.in_seg.size();
  return g_seg.nseg;
}

extern "C" void seg_get(int which, void *out) {
  const pirgpu::Segments &S = g_seg;
  switch (which) {
    case 0: std::copy(S.seg_of.begin(), S.seg_of.end(), (int32_t *)out); break;
    case 1: std::copy(S.pptr.begin(), S.pptr.end(), (int32_t *)out); break;
    case 2: std::copy(S.code.begin(), S.code.end(), (int32_t *)out); break;
    case 3: std::copy(S.prop.begin(), S.prop.end(), (int32_t *)out); break;
    case 4: std::copy(S.vptr.begin(), S.vptr.end(), (int32_t *)out); break;
    case 5: std::copy(S.var.begin(), S.var.end(), (uint32_t *)out); break;
    case 6: std::copy(S.umask.begin(), S.umask.end(), (uint64_t *)out); break;
    case 7: std::copy(S.uptr.begin(), S.uptr.end(), (int32_t *)out); break;
    case 8: std::copy(S.uadj.begin(), S.uadj.end(), (int32_t *)out); break;
    default: std::copy(S.in_seg.begin(), S.in_seg.end(), (uint32_t *)out); break;
  }
}
