// Path segments of a ternary bytecode, for the single-instance event schedule.
//
// A link variable is a variable with exactly two occurrences, in two distinct
// propagators: whatever narrows it can only matter to the other one.  The
// propagators whose link variables lead to one or two other such propagators
// form paths (a chain x_{i+1} = x_i + c_i is one long path).  Here the paths
// are cut into segments of at most SEG_MAX consecutive propagators; the event
// kernel runs a segment as one unit: a warp stages its variables in shared
// memory and one lane sweeps its propagators forward and backward until none
// of them narrows anything, then the warp joins the changes into the store.
// A link of the path then costs a few shared-memory accesses instead of a few
// dependent L2 round trips.
//
// Every propagator outside the segments stays a unit of its own.  The units'
// variable -> unit adjacency (CSR) lists, for each variable, every distinct
// unit using it: propagator p as p, segment s as ~s (negative).
//
// Plain C++ (no CUDA), so the host tests build it alone.
#ifndef PIR_SEGMENTS_H
#define PIR_SEGMENTS_H

#include <algorithm>
#include <cstdint>
#include <vector>

#include "pir_csr.h"

namespace pirgpu {

constexpr int SEG_MAX = 64;  // propagators per segment (the dirty set is one 64-bit word)
constexpr int SEG_MIN = 4;   // shorter pieces of a path stay single propagators
constexpr int SEG_VARS = 3 * SEG_MAX;  // local variables of a segment, at most
constexpr uint32_t SEG_BOUNDARY = 0x80000000u;  // seg_var flag: the variable has occurrences outside the segment

struct Segments {
  int nseg = 0;
  std::vector<int32_t> seg_of;       // per propagator: its segment, -1 if none
  std::vector<int32_t> pptr;         // nseg + 1 offsets into code (propagators of a segment, path order)
  std::vector<int32_t> code;         // op | slot_x << 8 | slot_y << 16 | slot_z << 24 (local variable slots)
  std::vector<int32_t> prop;         // the propagator of each code word (engine order index)
  std::vector<int32_t> vptr;         // nseg + 1 offsets into var / umask
  std::vector<uint32_t> var;         // global variable of each local slot | SEG_BOUNDARY
  std::vector<uint64_t> umask;       // per local slot: the segment's propagators (bits, path order) using it
  std::vector<int32_t> uptr, uadj;   // variable -> unit adjacency
  std::vector<uint32_t> in_seg;      // bit p: propagator p belongs to a segment
};

// Builds the segments and the unit adjacency from the bytecode (n
// propagators over nv variables, engine order) and its propagator adjacency
// (ptr, adj as build_adjacency makes them).  Returns false, writing nothing
// useful, when the unit adjacency would not fit int32 offsets.
inline bool build_segments(long long n, int nv, const int32_t *op, const int32_t *x, const int32_t *y,
                           const int32_t *z, const int32_t *ptr, const int32_t *adj, int nthreads, Segments &S) {
  S = Segments();
  if (n < 0 || !adjacency_fits(3 * n)) return false;
  const int32_t *slot[3] = {x, y, z};
  // the other propagator across variable v, when v is a link variable, else -1
  auto across = [&](int32_t v, int32_t p) -> int32_t {
    if (ptr[v + 1] - ptr[v] != 2) return -1;
    const int32_t a = adj[ptr[v]], b = adj[ptr[v] + 1];
    if (a == b) return -1;
    return a == p ? b : a;
  };
  // link degree: propagators with one or two link neighbours form the paths
  std::vector<uint8_t> ld((size_t)n, 0);
  const int T = std::max(1, nthreads);
  run_threads(T, [&](int t) {
    for (long long p = n * t / T; p < n * (t + 1) / T; ++p) {
      int d = 0;
      for (int k = 0; k < 3; ++k)
        if (across(slot[k][p], (int32_t)p) >= 0) ++d;
      ld[(size_t)p] = (uint8_t)d;
    }
  });
  auto eligible = [&](int32_t p) { return ld[(size_t)p] == 1 || ld[(size_t)p] == 2; };
  // path neighbours of an eligible propagator (at most two; a pair joined by
  // two link variables appears twice and the walk stops at the visited one)
  auto neighbours = [&](int32_t p, int32_t out[3]) {
    int m = 0;
    for (int k = 0; k < 3; ++k) {
      const int32_t q = across(slot[k][p], p);
      if (q >= 0 && eligible(q)) out[m++] = q;
    }
    return m;
  };
  S.seg_of.assign((size_t)n, -1);
  std::vector<uint8_t> seen((size_t)n, 0);
  std::vector<int32_t> path;
  S.pptr.push_back(0);
  S.vptr.push_back(0);
  auto emit = [&](const int32_t *props, int len) {
    const int s = S.nseg++;
    // local slots in order of first use; occurrences within the segment
    std::vector<int32_t> lvar;
    std::vector<int32_t> occ;
    auto local = [&](int32_t v) {
      for (size_t j = 0; j < lvar.size(); ++j)
        if (lvar[j] == v) return (int)j;
      lvar.push_back(v);
      occ.push_back(0);
      return (int)lvar.size() - 1;
    };
    const size_t u0 = S.umask.size();
    for (int k = 0; k < len; ++k) {
      const int32_t p = props[k];
      int sl[3];
      for (int j = 0; j < 3; ++j) {
        sl[j] = local(slot[j][p]);
        ++occ[(size_t)sl[j]];
      }
      S.seg_of[(size_t)p] = s;
      S.code.push_back((int32_t)((uint32_t)op[p] | (uint32_t)sl[0] << 8 | (uint32_t)sl[1] << 16 |
                                 (uint32_t)sl[2] << 24));
      S.prop.push_back(p);
      S.umask.resize(u0 + lvar.size(), 0ull);
      for (int j = 0; j < 3; ++j) S.umask[u0 + (size_t)sl[j]] |= 1ull << k;
    }
    for (size_t j = 0; j < lvar.size(); ++j) {
      const int32_t v = lvar[j];
      const bool boundary = ptr[v + 1] - ptr[v] > occ[j];
      S.var.push_back((uint32_t)v | (boundary ? SEG_BOUNDARY : 0u));
    }
    S.pptr.push_back((int32_t)S.code.size());
    S.vptr.push_back((int32_t)S.var.size());
  };
  // a path of len propagators: segments of nearly equal size, at most SEG_MAX
  auto cut = [&](const std::vector<int32_t> &pth) {
    const int len = (int)pth.size();
    if (len < SEG_MIN) return;
    const int parts = (len + SEG_MAX - 1) / SEG_MAX;
    for (int i = 0; i < parts; ++i) {
      const int b = (int)((long long)len * i / parts), e = (int)((long long)len * (i + 1) / parts);
      if (e - b >= SEG_MIN) emit(pth.data() + b, e - b);
    }
  };
  auto walk = [&](int32_t start) {
    path.clear();
    int32_t cur = start;
    while (cur >= 0) {
      seen[(size_t)cur] = 1;
      path.push_back(cur);
      int32_t nb[3];
      const int m = neighbours(cur, nb);
      int32_t next = -1;
      for (int j = 0; j < m && next < 0; ++j)
        if (!seen[(size_t)nb[j]]) next = nb[j];
      cur = next;
    }
    cut(path);
  };
  // paths from their ends, then what is left (cycles), each cut once
  for (long long p = 0; p < n; ++p) {
    if (seen[(size_t)p] || !eligible((int32_t)p)) continue;
    int32_t nb[3];
    if (neighbours((int32_t)p, nb) <= 1) walk((int32_t)p);
  }
  for (long long p = 0; p < n; ++p)
    if (!seen[(size_t)p] && eligible((int32_t)p)) walk((int32_t)p);
  // membership bits
  S.in_seg.assign((size_t)((n + 31) / 32), 0u);
  for (long long p = 0; p < n; ++p)
    if (S.seg_of[(size_t)p] >= 0) S.in_seg[(size_t)(p >> 5)] |= 1u << (p & 31);
  // unit adjacency: each variable's propagators as units, each unit once
  S.uptr.assign((size_t)nv + 1, 0);
  std::vector<int32_t> cnt((size_t)nv, 0);
  auto unit = [&](int32_t p) { return S.seg_of[(size_t)p] >= 0 ? ~S.seg_of[(size_t)p] : p; };
  // mark[s] = the last variable whose list took segment s (one array per thread)
  auto units_of = [&](int32_t v, int32_t *out, std::vector<int32_t> &mark) {
    int m = 0;
    for (int32_t k = ptr[v]; k < ptr[v + 1]; ++k) {
      const int32_t u = unit(adj[k]);
      bool dup;
      if (u < 0) {
        dup = mark[(size_t)~u] == v;
        mark[(size_t)~u] = v;
      } else {
        dup = m > 0 && out[m - 1] == u;  // a propagator's occurrences of v are adjacent in adj
      }
      if (!dup) out[m++] = u;
    }
    return m;
  };
  run_threads(T, [&](int t) {
    std::vector<int32_t> buf, mark((size_t)S.nseg, -1);
    for (long long v = (long long)nv * t / T; v < (long long)nv * (t + 1) / T; ++v) {
      buf.resize((size_t)(ptr[v + 1] - ptr[v]) + 1);
      cnt[(size_t)v] = units_of((int32_t)v, buf.data(), mark);
    }
  });
  long long tot = 0;
  for (int v = 0; v < nv; ++v) {
    S.uptr[(size_t)v] = (int32_t)tot;
    tot += cnt[(size_t)v];
  }
  S.uptr[(size_t)nv] = (int32_t)tot;
  S.uadj.resize((size_t)tot);
  run_threads(T, [&](int t) {
    std::vector<int32_t> mark((size_t)S.nseg, -1);
    for (long long v = (long long)nv * t / T; v < (long long)nv * (t + 1) / T; ++v)
      units_of((int32_t)v, S.uadj.data() + S.uptr[(size_t)v], mark);
  });
  return true;
}

}  // namespace pirgpu

#endif
