// Stable sort of an index permutation on the host's threads, for the install
// order of the bytecode (pir.hpp:343-347 sorts it by (op, y, x, z), stably).
// Contiguous chunks are sorted stably, one per thread, then neighbouring runs
// are merged pairwise, each round's merges in parallel; std::merge takes
// equal elements from the left run first, so the permutation is exactly the
// one std::stable_sort gives.  Plain C++ (no CUDA), so the host tests build
// it alone.
#ifndef PIR_SORT_H
#define PIR_SORT_H

#include <algorithm>
#include <vector>

#include "pir_csr.h"  // run_threads

namespace pirgpu {

template <class T, class Less>
inline void parallel_stable_sort(std::vector<T> &v, Less less, int nthreads) {
  const size_t n = v.size();
  int parts = std::max(1, nthreads);
  if (n < 4096) parts = 1;
  std::vector<size_t> cut((size_t)parts + 1);
  for (int t = 0; t <= parts; ++t) cut[(size_t)t] = n * (size_t)t / (size_t)parts;
  run_threads(parts, [&](int t) {
    std::stable_sort(v.begin() + (long)cut[(size_t)t], v.begin() + (long)cut[(size_t)t + 1], less);
  });
  std::vector<T> buf(parts > 1 ? n : 0);
  std::vector<T> *src = &v, *dst = &buf;
  for (int width = 1; width < parts; width *= 2) {
    const int pairs = (parts + 2 * width - 1) / (2 * width);
    const int workers = std::max(1, std::min(pairs, nthreads));
    run_threads(workers, [&](int t) {
      for (int p = t; p < pairs; p += workers) {
        const size_t a = cut[(size_t)std::min(parts, 2 * width * p)];
        const size_t m = cut[(size_t)std::min(parts, 2 * width * p + width)];
        const size_t b = cut[(size_t)std::min(parts, 2 * width * p + 2 * width)];
        std::merge(src->begin() + (long)a, src->begin() + (long)m, src->begin() + (long)m, src->begin() + (long)b,
                   dst->begin() + (long)a, less);
      }
    });
    std::swap(src, dst);
  }
  if (src != &v) v.swap(*src);
}

}  // namespace pirgpu

#endif
