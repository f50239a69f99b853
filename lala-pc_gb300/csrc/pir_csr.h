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
#include <cstdint>
#include <thread>
#include <vector>

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

// Threads worth using for n propagators (0: the host's).
inline int adjacency_threads(long long n, int requested = 0) {
  int t = requested > 0 ? requested : (int)std::thread::hardware_concurrency();
  t = std::max(1, std::min(t, 16));
  // each thread's per-variable counts cost nvars words: not for small inputs
  if (n < (1ll << 16)) t = 1;
  return t;
}

// ptr: nv + 1 entries; adj: 3 n entries.  Variables must lie in [0, nv).
inline void build_adjacency(long long n, int nv, const int32_t *x, const int32_t *y, const int32_t *z,
                            int32_t *ptr, int32_t *adj, int nthreads) {
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
}

}  // namespace pirgpu

#endif
