// Variable -> propagator adjacency of a ternary bytecode (CSR), built on the
// host's threads for the event schedules: adj[ptr[v] .. ptr[v + 1]) lists,
// in increasing propagator order, every propagator p with v among x[p],
// y[p], z[p] (once per occurrence, x before y before z).  The arrays are
// those of a sequential counting sort whatever the thread count: each
// thread counts its contiguous chunk of propagators per variable, the counts
// become per-thread write cursors (the chunks' order is the propagators'
// order), and each thread then fills its chunk's entries.  Plain C++ (no
// CUDA), so the host tests build it alone.
#ifndef PIR_CSR_H
#define PIR_CSR_H

#include <algorithm>
#include <climits>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/pirgpu.h"  // enum pc_kind

namespace pirgpu {

// Runs fn(t) for t = 0 .. nthreads - 1, one std::thread each (t = 0 on the
// calling thread).
template <class F>
inline void run_threads(int nthreads, F fn) {
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(fn, t);
  fn(0);
  for (std::thread &th : pool) th.join();
}

// Threads worth using for n work items (0 requested: the host's).  With
// nvars > 0, each thread's per-variable counts (nvars words) stay within the
// 3 n entries they count.
inline int adjacency_threads(long long n, int requested = 0, long long nvars = 0) {
  int t = requested > 0 ? requested : (int)std::thread::hardware_concurrency();
  t = std::max(1, std::min(t, 16));
  if (n < (1ll << 16)) t = 1;
  if (nvars > 0) t = (int)std::max(1ll, std::min((long long)t, 3 * n / nvars));
  return t;
}

// The adjacency indexes its entries with int32 (ptr, the kernels' cursors):
// at most INT32_MAX of them.
inline bool adjacency_fits(long long entries) { return entries >= 0 && entries <= (long long)INT32_MAX; }

// ptr: nv + 1 entries; adj: 3 n entries.  Variables must lie in [0, nv).
// Returns false, writing nothing, when the 3 n entries do not fit int32
// offsets (n > 715,827,882 propagators).
inline bool build_adjacency(long long n, int nv, const int32_t *x, const int32_t *y, const int32_t *z,
                            int32_t *ptr, int32_t *adj, int nthreads) {
  if (n < 0 || !adjacency_fits(3 * n)) return false;
  const int T = std::max(1, nthreads);
  std::vector<long long> lo(T + 1);
  for (int t = 0; t <= T; ++t) lo[t] = n * t / T;
  // per thread and variable: entries of the thread's chunk, then its cursor
  std::vector<std::vector<int32_t>> cnt((size_t)T);
  run_threads(T, [&](int t) {
    std::vector<int32_t> &c = cnt[(size_t)t];
    c.assign((size_t)nv, 0);
    for (long long p = lo[t]; p < lo[t + 1]; ++p) {
      ++c[(size_t)x[p]];
      ++c[(size_t)y[p]];
      ++c[(size_t)z[p]];
    }
  });
  // degrees and their prefix sum over variable ranges
  std::vector<long long> vlo(T + 1), part(T + 1, 0);
  for (int t = 0; t <= T; ++t) vlo[t] = (long long)nv * t / T;
  run_threads(T, [&](int t) {
    long long s = 0;
    for (long long v = vlo[t]; v < vlo[t + 1]; ++v)
      for (int u = 0; u < T; ++u) s += cnt[(size_t)u][(size_t)v];
    part[t + 1] = s;
  });
  for (int t = 0; t < T; ++t) part[t + 1] += part[t];
  ptr[0] = 0;
  run_threads(T, [&](int t) {
    long long s = part[t];
    for (long long v = vlo[t]; v < vlo[t + 1]; ++v) {
      // thread u writes variable v's entries from s + (entries of threads before u)
      for (int u = 0; u < T; ++u) {
        const int32_t k = cnt[(size_t)u][(size_t)v];
        cnt[(size_t)u][(size_t)v] = (int32_t)s;
        s += k;
      }
      ptr[v + 1] = (int32_t)s;
    }
  });
  run_threads(T, [&](int t) {
    std::vector<int32_t> &c = cnt[(size_t)t];
    for (long long p = lo[t]; p < lo[t + 1]; ++p) {
      adj[c[(size_t)x[p]]++] = (int32_t)p;
      adj[c[(size_t)y[p]]++] = (int32_t)p;
      adj[c[(size_t)z[p]]++] = (int32_t)p;
    }
  });
  return true;
}

// The PC event schedule's variable -> formula adjacency: adj[ptr[v] ..
// ptr[v + 1]) lists, in increasing order, the formulas i (roots[i] in a tape
// of 4-int nodes {kind, a, b, c}, the kinds of enum pc_kind) with variable v
// among their leaves (variable terms, variable literals, store items), each
// formula once.  ptr: nv + 1 entries; adj is resized to the entry count.
// Each thread walks a contiguous chunk of formulas (their distinct variables
// sorted, which the adjacency does not see), then counts, cursors and fills
// as build_adjacency does: the arrays equal a sequential build's.  Returns
// false, writing nothing, when the entries do not fit int32 offsets.
inline bool build_formula_adjacency(int np, const int32_t *roots, const int32_t *tape, int nv, int32_t *ptr,
                                    std::vector<int32_t> &adj, int nthreads) {
  const int T = std::max(1, nthreads);
  std::vector<long long> lo(T + 1);
  for (int t = 0; t <= T; ++t) lo[t] = (long long)np * t / T;
  std::vector<std::vector<int32_t>> vars((size_t)T), start((size_t)T), cnt((size_t)T);
  run_threads(T, [&](int t) {
    std::vector<int32_t> &vs = vars[(size_t)t], &st = start[(size_t)t], &c = cnt[(size_t)t];
    c.assign((size_t)nv, 0);
    st.reserve((size_t)(lo[t + 1] - lo[t]) + 1);
    vs.reserve((size_t)(lo[t + 1] - lo[t]) * 4);
    std::vector<int32_t> todo;
    todo.reserve(64);
    for (long long i = lo[t]; i < lo[t + 1]; ++i) {
      st.push_back((int32_t)vs.size());
      const size_t first = vs.size();
      todo.assign(1, roots[i]);
      while (!todo.empty()) {
        const int32_t *d = tape + 4 * (size_t)todo.back();
        todo.pop_back();
        const int k = d[0];
        if (k == PC_VAR || k == PC_PVAR || k == PC_NVAR || (k >= PC_TELL && k <= PC_NASK_OUT)) {
          vs.push_back(d[1]);
        } else if (k == PC_AE || k == PC_NADD || k == PC_NMUL) {
          for (int j = 0; j < d[2]; ++j) todo.push_back(d[1] + j);
        } else if (k == PC_FORMULA || k == PC_NEG || k == PC_ABS || k == PC_ARG) {
          todo.push_back(d[1]);
        } else if ((k >= PC_ADD && k <= PC_MAX) || (k >= PC_LEQ && k <= PC_XOR)) {
          todo.push_back(d[1]);
          todo.push_back(d[2]);
        }
      }
      std::sort(vs.begin() + (long)first, vs.end());
      vs.erase(std::unique(vs.begin() + (long)first, vs.end()), vs.end());
      for (size_t q = first; q < vs.size(); ++q) ++c[(size_t)vs[q]];
    }
    st.push_back((int32_t)vs.size());
  });
  std::vector<long long> vlo(T + 1), part(T + 1, 0);
  for (int t = 0; t <= T; ++t) vlo[t] = (long long)nv * t / T;
  run_threads(T, [&](int t) {
    long long s = 0;
    for (long long v = vlo[t]; v < vlo[t + 1]; ++v)
      for (int u = 0; u < T; ++u) s += cnt[(size_t)u][(size_t)v];
    part[t + 1] = s;
  });
  for (int t = 0; t < T; ++t) part[t + 1] += part[t];
  if (!adjacency_fits(part[T])) return false;
  ptr[0] = 0;
  run_threads(T, [&](int t) {
    long long s = part[t];
    for (long long v = vlo[t]; v < vlo[t + 1]; ++v) {
      for (int u = 0; u < T; ++u) {
        const int32_t k = cnt[(size_t)u][(size_t)v];
        cnt[(size_t)u][(size_t)v] = (int32_t)s;
        s += k;
      }
      ptr[v + 1] = (int32_t)s;
    }
  });
  adj.resize((size_t)part[T]);
  run_threads(T, [&](int t) {
    const std::vector<int32_t> &vs = vars[(size_t)t], &st = start[(size_t)t];
    std::vector<int32_t> &c = cnt[(size_t)t];
    for (long long i = lo[t]; i < lo[t + 1]; ++i) {
      const size_t r = (size_t)(i - lo[t]);
      for (int32_t q = st[r]; q < st[r + 1]; ++q) adj[(size_t)c[(size_t)vs[(size_t)q]]++] = (int32_t)i;
    }
  });
  return true;
}

}  // namespace pirgpu

#endif
