// CPU oracle for the PIR propagator fixpoint — TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this code (as the checker, or as the timed CPU baseline).  The product never
// links it.
//
// Restates lala-pc include/lala/pir.hpp:395-817 (propagators), :326-352
// (install), :417-438 (ask) and the Gauss-Seidel loop used by
// tests/pir_test.cpp:60-62.  The lattice it runs on, Interval<ZLB<int>> in a
// VStore, lives in lala-core v1.2.8 (CMakeLists.txt:31-43, not vendored); its
// semantics are restated here from their mathematical meaning:
//   * a bound pair (lb, ub) of int32; lb = INT32_MIN is "no lower bound"
//     (ZLB top, pir.hpp:403-404,738), ub = INT32_MAX is "no upper bound";
//   * an interval is empty (bot) when lb > ub, or a bound sits at its own
//     bottom sentinel (lb = INT32_MAX or ub = INT32_MIN);
//   * embed = meet (max of lbs, min of ubs), "changed" iff a bound narrowed;
//   * join / fjoin = interval hull, with bot as the neutral element;
//   * tdiv/fdiv/cdiv/ediv (cuda-battery, not vendored): truncating, floor,
//     ceiling and Euclidean integer division, by their definitions.
// The reference computes in plain int and overflows (undefined behaviour) near
// +-2^31.  Here every intermediate is exact in int64 and clamped to int32 when
// it becomes a bound; g_overflows counts intermediates outside int32, so a run
// with a zero count is one where the reference's arithmetic is defined and the
// two agree exactly.
#include "pir_oracle.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

using i32 = int32_t;
using i64 = int64_t;
constexpr i32 INF = INT32_MAX;   // pir.hpp:403
constexpr i32 MINF = INT32_MIN;  // pir.hpp:404

thread_local i64 g_overflows = 0;

// An intermediate the reference evaluates in int: exact here, counted if the
// reference would have overflowed.
inline i64 ov(i64 v) {
  if (v > INF || v < MINF) ++g_overflows;
  return v;
}
// A value becoming an int32 bound.
inline i32 cl(i64 v) { return v > INF ? INF : (v < MINF ? MINF : (i32)v); }
inline i64 mn(i64 a, i64 b) { return a < b ? a : b; }
inline i64 mx(i64 a, i64 b) { return a > b ? a : b; }

struct Itv {
  i32 l, u;
  static Itv top() { return {MINF, INF}; }
  static Itv bot() { return {INF, MINF}; }
  static Itv of(i64 l, i64 u) { return {cl(l), cl(u)}; }
  bool is_bot() const { return l > u || l == INF || u == MINF; }
  bool operator==(const Itv &o) const { return l == o.l && u == o.u; }
  // Interval meet, local (no change report).
  void meet(const Itv &o) {
    if (o.l > l) l = o.l;
    if (o.u < u) u = o.u;
  }
  // Interval hull with bot neutral.
  void join(const Itv &o) {
    if (o.is_bot()) return;
    if (is_bot()) { *this = o; return; }
    if (o.l < l) l = o.l;
    if (o.u > u) u = o.u;
  }
};
inline Itv fjoin(Itv a, const Itv &b) { a.join(b); return a; }

const Itv ONE{1, 1};   // pir.hpp:160-161
const Itv ZERO{0, 0};

// cuda-battery integer divisions (b != 0), exact in int64.
inline i64 tdiv(i64 a, i64 b) { return a / b; }
inline i64 fdiv(i64 a, i64 b) {
  i64 q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}
inline i64 cdiv(i64 a, i64 b) {
  i64 q = a / b;
  return (a % b != 0 && ((a < 0) == (b < 0))) ? q + 1 : q;
}
inline i64 ediv(i64 a, i64 b) {
  i64 q = a / b, r = a % b;
  if (r < 0) q = (b > 0) ? q - 1 : q + 1;
  return q;
}

// pir.hpp:407-415
inline i64 div_op(i64 a, i32 op, i64 b) {
  switch (op) {
    case ORC_TDIV: return ov(tdiv(a, b));
    case ORC_CDIV: return ov(cdiv(a, b));
    case ORC_FDIV: return ov(fdiv(a, b));
    default: return ov(ediv(a, b));
  }
}

// The macro names of pir.hpp:396-401.
#define xl ((i64)r1.l)
#define xu ((i64)r1.u)
#define yl ((i64)r2.l)
#define yu ((i64)r2.u)
#define zl ((i64)r3.l)
#define zu ((i64)r3.u)

// r1 = r2 / r3, pir.hpp:449-467
void itv_div(i32 op, Itv &r1, Itv &r2, Itv &r3) {
  if (zl < 0 && zu > 0) {
    r1.l = cl(mx(xl, mn(yl, yu == MINF ? (i64)INF : ov(-yu))));
    r1.u = cl(mn(xu, mx(yl == INF ? (i64)MINF : ov(-yl), yu)));
  } else {
    if (zl == 0) r3.l = 1;
    if (zu == 0) r3.u = -1;
    if (yl == MINF || yu == INF || zl == MINF || zu == INF) return;
    if (r3.is_bot()) return;
    i64 t1 = div_op(yl, op, zl), t2 = div_op(yl, op, zu);
    i64 t3 = div_op(yu, op, zl), t4 = div_op(yu, op, zu);
    r1.l = cl(mx(xl, mn(mn(t1, t2), mn(t3, t4))));
    r1.u = cl(mn(xu, mx(mx(t1, t2), mx(t3, t4))));
  }
}

// pir.hpp:469-479 (r1 = quotient, r3 = divisor)
Itv num_fdiv(const Itv &r1, const Itv &r3) {
  if (zl < 0 && zu > 0) {
    return Itv::of(mn(mn(xl, ov(-xu)), mn(ov(xl * zu), ov(ov(ov(xu + 1) * zl) + 1))),
                   mx(mx(ov(-xl), xu), mx(ov(xl * zl), ov(ov(ov(xu + 1) * zu) - 1))));
  } else if (zl > 0 || zu < 0) {
    return Itv::of(mn(mn(ov(xl * zl), ov(xl * zu)), mn(ov(ov(ov(xu + 1) * zl) + 1), ov(ov(ov(xu + 1) * zu) + 1))),
                   mx(mx(ov(xl * zl), ov(xl * zu)), mx(ov(ov(ov(xu + 1) * zl) - 1), ov(ov(ov(xu + 1) * zu) - 1))));
  }
  return Itv::top();
}

// pir.hpp:481-491
Itv num_cdiv(const Itv &r1, const Itv &r3) {
  if (zl < 0 && zu > 0) {
    return Itv::of(mn(mn(xl, ov(-xu)), mn(ov(xu * zl), ov(ov(ov(xl - 1) * zu) + 1))),
                   mx(mx(ov(-xl), xu), mx(ov(xu * zu), ov(ov(ov(xl - 1) * zl) - 1))));
  } else if (zl > 0 || zu < 0) {
    return Itv::of(mn(mn(ov(xu * zl), ov(xu * zu)), mn(ov(ov(ov(xl - 1) * zl) + 1), ov(ov(ov(xl - 1) * zu) + 1))),
                   mx(mx(ov(xu * zl), ov(xu * zu)), mx(ov(ov(ov(xl - 1) * zl) - 1), ov(ov(ov(xl - 1) * zu) - 1))));
  }
  return Itv::top();
}

// pir.hpp:493-507
Itv num_tdiv(const Itv &r1, const Itv &r3) {
  if (xl > 0) return num_fdiv(r1, r3);
  else if (xu < 0) return num_cdiv(r1, r3);
  else if (xl <= 0 && 0 <= xu) {
    Itv r = Itv::of(ov(mn(zl, ov(-zu)) + 1), ov(mx(ov(-zl), zu) - 1));
    if (xl != 0) r.join(num_cdiv(Itv{r1.l, -1}, r3));
    if (xu != 0) r.join(num_fdiv(Itv{1, r1.u}, r3));
    return r;
  }
  return Itv::top();
}

// pir.hpp:510-517
Itv num_ediv(const Itv &r1, const Itv &r3) {
  if (zl > 0) return num_fdiv(r1, r3);
  else if (zu < 0) return num_cdiv(r1, r3);
  else if (zl < 0 && zu > 0) return fjoin(num_cdiv(r1, Itv{r3.l, -1}), num_fdiv(r1, Itv{1, r3.u}));
  return Itv::top();
}

// pir.hpp:520-574 (r1 = quotient, r2 = numerator; result bounds the divisor)
Itv den_fdiv(const Itv &r1, const Itv &r2) {
  if (xl > 0 || ov(xu + 1) < 0) {
    if (yl > 0) {
      return Itv::of(ov(mn(fdiv(yl, ov(xu + 1)), fdiv(yu, ov(xu + 1))) + 1),
                     mx(fdiv(yl, xl), fdiv(yu, xl)));
    } else if (yu < 0) {
      return Itv::of(mn(cdiv(yl, xl), cdiv(yu, xl)),
                     ov(mx(cdiv(yl, ov(xu + 1)), cdiv(yu, ov(xu + 1))) - 1));
    } else if (0 == yl && yl < yu) {
      return den_fdiv(r1, Itv{1, r2.u});
    } else if (yl < yu && yu == 0) {
      return den_fdiv(r1, Itv{r2.l, -1});
    } else if (yl < 0 && 0 < yu) {
      return fjoin(den_fdiv(r1, Itv{r2.l, -1}), den_fdiv(r1, Itv{1, r2.u}));
    } else if (yl == 0 && yu == 0) {
      return Itv::bot();
    }
  } else if (xl == 0 && xu == 0) {
    if (yl > 0) return Itv::of(ov(yl + 1), INF);
    else if (yu < 0) return Itv::of(MINF, ov(yu - 1));
  } else if (xl == -1 && xu == -1) {
    if (yl > 0) return Itv::of(MINF, ov(-yl));
    else if (yu < 0) return Itv::of(ov(-yu), INF);
    else if (0 == yl && yl < yu) return Itv{MINF, -1};
    else if (yl < yu && yu == 0) return Itv{1, INF};
    else if (yl == 0 && yu == 0) return Itv::bot();
  } else if (xl == 0 && 0 < xu) {
    return fjoin(den_fdiv(Itv{0, 0}, r2), den_fdiv(Itv{1, r1.u}, r2));
  } else if (xl < -1 && xu == -1) {
    return fjoin(den_fdiv(Itv{r1.l, -2}, r2), den_fdiv(Itv{-1, -1}, r2));
  } else if (xl <= -1 && xu >= 0) {
    Itv r = den_fdiv(Itv{-1, -1}, r2);
    r.join(den_fdiv(Itv{0, 0}, r2));
    if (xl != -1) r.join(den_fdiv(Itv{r1.l, -2}, r2));
    if (xu != 0) r.join(den_fdiv(Itv{1, r1.u}, r2));
    return r;
  }
  return Itv::top();
}

// pir.hpp:577-630
Itv den_cdiv(const Itv &r1, const Itv &r2) {
  if (ov(xl - 1) > 0 || xu < 0) {
    if (yl > 0) {
      return Itv::of(mn(cdiv(yl, xu), cdiv(yu, xu)),
                     ov(mx(cdiv(yl, ov(xl - 1)), cdiv(yu, ov(xl - 1))) - 1));
    } else if (yu < 0) {
      return Itv::of(ov(mn(fdiv(yl, ov(xl - 1)), fdiv(yu, ov(xl - 1))) + 1),
                     mx(fdiv(yl, xu), fdiv(yu, xu)));
    } else if (0 == yl && yl < yu) {
      return den_cdiv(r1, Itv{1, r2.u});
    } else if (yl < yu && yu == 0) {
      return den_cdiv(r1, Itv{r2.l, -1});
    } else if (yl < 0 && 0 < yu) {
      return fjoin(den_cdiv(r1, Itv{r2.l, -1}), den_cdiv(r1, Itv{1, r2.u}));
    } else if (yl == 0 && yu == 0) {
      return Itv::bot();
    }
  } else if (xl == 0 && xu == 0) {
    if (yl > 0) return Itv::of(MINF, ov(ov(-yl) - 1));
    else if (yu < 0) return Itv::of(ov(ov(-yu) + 1), INF);
  } else if (xl == 1 && xu == 1) {
    if (yl > 0) return Itv{r2.l, INF};
    else if (yu < 0) return Itv{MINF, r2.u};
    else if (0 == yl && yl < yu) return Itv{1, INF};
    else if (yl < yu && yu == 0) return Itv{MINF, -1};
    else if (yl == 0 && yu == 0) return Itv::bot();
  } else if (xl < 0 && xu == 0) {
    return fjoin(den_cdiv(Itv{r1.l, -1}, r2), den_cdiv(Itv{0, 0}, r2));
  } else if (xl == 1 && 1 < xu) {
    return fjoin(den_cdiv(Itv{1, 1}, r2), den_cdiv(Itv{2, r1.u}, r2));
  } else if (xl <= 0 && xu >= 1) {
    Itv r = den_cdiv(Itv{1, 1}, r2);
    r.join(den_cdiv(Itv{0, 0}, r2));
    if (xl != 0) r.join(den_cdiv(Itv{r1.l, -1}, r2));
    if (xu != 1) r.join(den_cdiv(Itv{2, r1.u}, r2));
    return r;
  }
  return Itv::top();
}

// pir.hpp:633-649
Itv den_tdiv(const Itv &r1, const Itv &r2, const Itv &r3) {
  if (xl > 0) return den_fdiv(r1, r2);
  else if (xu < 0) return den_cdiv(r1, r2);
  else if (xl == 0 && xu == 0) {
    if (yl > 0 && zl > 0) return Itv::of(ov(yl + 1), INF);
    if (yl > 0 && zu < 0) return Itv::of(MINF, ov(ov(-yl) - 1));
    if (yu < 0 && zl > 0) return Itv::of(ov(ov(-yu) + 1), INF);
    if (yu < 0 && zu < 0) return Itv::of(MINF, ov(yu - 1));
  } else if (xl <= 0 && 0 <= xu) {
    Itv r = den_tdiv(Itv{0, 0}, r2, r3);
    if (xl != 0) r.join(den_cdiv(Itv{r1.l, -1}, r2));
    if (xu != 0) r.join(den_fdiv(Itv{1, r1.u}, r2));
    return r;
  }
  return Itv::top();
}

// pir.hpp:651-658
Itv den_ediv(const Itv &r1, const Itv &r2, const Itv &r3) {
  if (zl > 0) return den_fdiv(r1, r2);
  else if (zu < 0) return den_cdiv(r1, r2);
  else if (zl < 0 && 0 < zu) return fjoin(den_fdiv(r1, r2), den_cdiv(r1, r2));
  return Itv::top();
}

// pir.hpp:660-679
void itv_div_num(i32 op, Itv &r1, Itv &r2, Itv &r3) {
  switch (op) {
    case ORC_FDIV: r2.meet(num_fdiv(r1, r3)); break;
    case ORC_CDIV: r2.meet(num_cdiv(r1, r3)); break;
    case ORC_TDIV: r2.meet(num_tdiv(r1, r3)); break;
    case ORC_EDIV: r2.meet(num_ediv(r1, r3)); break;
  }
}

// pir.hpp:681-700
void itv_div_den(i32 op, Itv &r1, Itv &r2, Itv &r3) {
  switch (op) {
    case ORC_FDIV: r3.meet(den_fdiv(r1, r2)); break;
    case ORC_CDIV: r3.meet(den_cdiv(r1, r2)); break;
    case ORC_TDIV: r3.meet(den_tdiv(r1, r2, r3)); break;
    case ORC_EDIV: r3.meet(den_ediv(r1, r2, r3)); break;
  }
}

// y = x / z for x = y * z, pir.hpp:702-718
void mul_inv(const Itv &r1, Itv &r2, Itv &r3) {
  if (xl > 0 || xu < 0) {
    if (zl == 0) r3.l = 1;
    if (zu == 0) r3.u = -1;
  }
  if ((xl > 0 || xu < 0) && zl < 0 && zu > 0) {
    r2.l = cl(mx(yl, mn(xl, xu == MINF ? (i64)INF : ov(-xu))));
    r2.u = cl(mn(yu, mx(xl == INF ? (i64)MINF : ov(-xl), xu)));
  } else if (xl > 0 || xu < 0 || zl > 0 || zu < 0) {
    if (xl == MINF || xu == INF || zl == MINF || zu == INF) return;
    if (r3.is_bot()) return;
    r2.l = cl(mx(yl, mn(mn(ov(cdiv(xl, zl)), ov(cdiv(xl, zu))), mn(ov(cdiv(xu, zl)), ov(cdiv(xu, zu))))));
    r2.u = cl(mn(yu, mx(mx(ov(fdiv(xl, zl)), ov(fdiv(xl, zu))), mx(ov(fdiv(xu, zl)), ov(fdiv(xu, zu))))));
  }
}

// VStore::embed: meet into the store; returns the number of bounds narrowed.
inline int embed(i32 *s, i32 v, const Itv &d, int *failed) {
  int n = 0;
  if (d.l > s[2 * v]) { s[2 * v] = d.l; ++n; }
  if (d.u < s[2 * v + 1]) { s[2 * v + 1] = d.u; ++n; }
  if (n) {
    Itv now{s[2 * v], s[2 * v + 1]};
    if (now.is_bot()) *failed = 1;
  }
  return n;
}

// PIR::deduce(bytecode_type), pir.hpp:721-817.  Returns bounds narrowed.
int deduce(i32 op, i32 X, i32 Y, i32 Z, i32 *s, int *failed) {
  int ch = 0;
  Itv r1{s[2 * X], s[2 * X + 1]};
  Itv r2{s[2 * Y], s[2 * Y + 1]};
  Itv r3{s[2 * Z], s[2 * Z + 1]};
  switch (op) {
    case ORC_EQ: {  // pir.hpp:730-744
      if (r1 == ONE) {
        ch += embed(s, Y, r3, failed);
        ch += embed(s, Z, r2, failed);
      } else if (r1 == ZERO && (yl == yu || zl == zu)) {
        ch += embed(s, zl == zu ? Y : Z,
                    Itv{yl == zl ? cl(ov(yl + 1)) : MINF, yu == zu ? cl(ov(yu - 1)) : INF}, failed);
      } else if (yu == zl && yl == zu) {
        ch += embed(s, X, ONE, failed);
      } else if (yl > zu || yu < zl) {
        ch += embed(s, X, ZERO, failed);
      }
      return ch;
    }
    case ORC_LEQ: {  // pir.hpp:745-757
      if (r1 == ONE) {
        ch += embed(s, Y, Itv{r2.l, r3.u}, failed);
        ch += embed(s, Z, Itv{r2.l, r3.u}, failed);
      } else if (r1 == ZERO) {
        ch += embed(s, Y, Itv{cl(ov(zl + 1)), r2.u}, failed);
        ch += embed(s, Z, Itv{r3.l, cl(ov(yu - 1))}, failed);
      } else if (yu <= zl) {
        ch += embed(s, X, ONE, failed);
      } else if (yl > zu) {
        ch += embed(s, X, ZERO, failed);
      }
      return ch;
    }
    case ORC_ADD: {  // pir.hpp:758-766
      r1.l = (yl == MINF || zl == MINF) ? r1.l : cl(mx(xl, ov(yl + zl)));
      r1.u = (yu == INF || zu == INF) ? r1.u : cl(mn(xu, ov(yu + zu)));
      r2.l = (xl == MINF || zu == INF) ? r2.l : cl(mx(yl, ov(xl - zu)));
      r2.u = (xu == INF || zl == MINF) ? r2.u : cl(mn(yu, ov(xu - zl)));
      r3.l = (xl == MINF || yu == INF) ? r3.l : cl(mx(zl, ov(xl - yu)));
      r3.u = (xu == INF || yl == MINF) ? r3.u : cl(mn(zu, ov(xu - yl)));
      break;
    }
    case ORC_MUL: {  // pir.hpp:767-779
      if (yl != MINF && yu != INF && zl != MINF && zu != INF) {
        i64 t1 = ov(yl * zl), t2 = ov(yl * zu), t3 = ov(yu * zl), t4 = ov(yu * zu);
        r1.l = cl(mx(xl, mn(mn(t1, t2), mn(t3, t4))));
        r1.u = cl(mn(xu, mx(mx(t1, t2), mx(t3, t4))));
      }
      mul_inv(r1, r2, r3);
      mul_inv(r1, r3, r2);
      break;
    }
    case ORC_TDIV:
    case ORC_CDIV:
    case ORC_FDIV:
    case ORC_EDIV: {  // pir.hpp:780-792
      itv_div(op, r1, r2, r3);
      if (!r1.is_bot() && !r3.is_bot()) {
        itv_div_num(op, r1, r2, r3);
        if (!r2.is_bot()) itv_div_den(op, r1, r2, r3);
      }
      break;
    }
    case ORC_MIN: {  // pir.hpp:793-801
      r1.l = cl(mx(xl, mn(yl, zl)));
      r1.u = cl(mn(xu, mn(yu, zu)));
      r2.l = cl(mx(yl, xl));
      if (xu < zl) r2.u = cl(mn(yu, xu));
      r3.l = cl(mx(zl, xl));
      if (xu < yl) r3.u = cl(mn(zu, xu));
      break;
    }
    case ORC_MAX: {  // pir.hpp:802-810
      r1.l = cl(mx(xl, mx(yl, zl)));
      r1.u = cl(mn(xu, mx(yu, zu)));
      r2.u = cl(mn(yu, xu));
      if (xl > zu) r2.l = cl(mx(yl, xl));
      r3.u = cl(mn(zu, xu));
      if (xl > yu) r3.l = cl(mx(zl, xl));
      break;
    }
    default: return 0;
  }
  ch += embed(s, X, r1, failed);  // pir.hpp:813-815
  ch += embed(s, Y, r2, failed);
  ch += embed(s, Z, r3, failed);
  return ch;
}

// PIR::ask(bytecode_type), pir.hpp:417-438
int ask(i32 op, i32 X, i32 Y, i32 Z, const i32 *s) {
  Itv r1{s[2 * X], s[2 * X + 1]};
  Itv r2{s[2 * Y], s[2 * Y + 1]};
  Itv r3{s[2 * Z], s[2 * Z + 1]};
  switch (op) {
    case ORC_EQ: return (xl == 1 && yu == zl && yl == zu) || (xu == 0 && (yu < zl || yl > zu));
    case ORC_LEQ: return (xl == 1 && yu <= zl) || (xu == 0 && yl > zu);
    case ORC_ADD: return xl == xu && yl == yu && zl == zu && xl == ov(yl + zl);
    case ORC_MUL:
      return xl == xu && ((yl == yu && zl == zu && xl == ov(yl * zl)) ||
                          (xl == 0 && (r2 == ZERO || r3 == ZERO)));
    case ORC_TDIV:
    case ORC_CDIV:
    case ORC_FDIV:
    case ORC_EDIV:
      return (xl == xu && yl == yu && zl == zu && zl != 0 && xl == div_op(yl, op, zl)) ||
             (xl == yu && xu == yl && xl == 0 && (zl > 0 || zu < 0));
    case ORC_MIN: return (xl == yu && xu == yl && yu <= zl) || (xl == zu && xu == zl && zu <= yl);
    case ORC_MAX: return (xl == yu && xu == yl && yl >= zu) || (xl == zu && xu == zl && zl >= yu);
    default: return 0;
  }
}

#undef xl
#undef xu
#undef yl
#undef yu
#undef zl
#undef zu

bool store_bot(i32 nvars, const i32 *s) {
  for (i32 v = 0; v < nvars; ++v) {
    Itv d{s[2 * v], s[2 * v + 1]};
    if (d.is_bot()) return true;
  }
  return false;
}

// Gauss-Seidel loop over an explicit order (tests/pir_test.cpp:60-62), stopping
// after the first sweep that empties the store.
int gs_fixpoint(i32 n, const i32 *op, const i32 *x, const i32 *y, const i32 *z, i32 nvars,
                i32 *s, i64 max_sweeps, i64 *out) {
  g_overflows = 0;
  i64 sweeps = 0, execs = 0, narrowed = 0;
  int status = ORC_OK;
  if (store_bot(nvars, s)) {
    status = ORC_FAILED;
  } else {
    for (;;) {
      if (sweeps >= max_sweeps) { status = ORC_TIMEOUT; break; }
      int failed = 0;
      i64 ch = 0;
      for (i32 i = 0; i < n; ++i) ch += deduce(op[i], x[i], y[i], z[i], s, &failed);
      ++sweeps;
      execs += n;
      narrowed += ch;
      if (failed) { status = ORC_FAILED; break; }
      if (ch == 0) break;
    }
  }
  if (out) {
    out[0] = sweeps;
    out[1] = execs;
    out[2] = narrowed;
    out[3] = g_overflows;
  }
  return status;
}

template <class F>
void parallel_for(i64 count, int threads, F f) {
  if (threads <= 1 || count <= 1) {
    for (i64 j = 0; j < count; ++j) f(j);
    return;
  }
  std::atomic<i64> next{0};
  std::vector<std::thread> pool;
  int t = (int)std::min<i64>(threads, count);
  for (int k = 0; k < t; ++k)
    pool.emplace_back([&]() {
      for (;;) {
        i64 j = next.fetch_add(1);
        if (j >= count) break;
        f(j);
      }
    });
  for (auto &th : pool) th.join();
}

int resolve_threads(int threads) {
  if (threads > 0) return threads;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

// ---- exhaustive property checks (tests/bound_consistency_test.hpp) ----------

i64 mod_op(i32 kind, i64 a, i64 b) {
  // kind: 0 emod, 1 tmod, 2 cmod, 3 fmod; a - b * div(a, b)
  switch (kind) {
    case 0: return a - b * ediv(a, b);
    case 1: return a - b * tdiv(a, b);
    case 2: return a - b * cdiv(a, b);
    default: return a - b * fdiv(a, b);
  }
}

// The relation x = f(y, z) of each predicate of tests/pir_test.cpp:122-171.
bool pred_holds(i32 pred, i64 a, i64 b, i64 c) {
  switch (pred) {
    case 0: return (a == 0 || a == 1) && a == (b == c ? 1 : 0);
    case 1: return (a == 0 || a == 1) && a == (b <= c ? 1 : 0);
    case 2: return a == b + c;
    case 3: return a == std::min(b, c);
    case 4: return a == std::max(b, c);
    case 5: return a == b * c;
    case 6: return c != 0 && a == ediv(b, c);
    case 7: return c != 0 && a == tdiv(b, c);
    case 8: return c != 0 && a == cdiv(b, c);
    case 9: return c != 0 && a == fdiv(b, c);
    case 10: return c != 0 && a == mod_op(0, b, c);
    case 11: return c != 0 && a == mod_op(1, b, c);
    case 12: return c != 0 && a == mod_op(2, b, c);
    case 13: return c != 0 && a == mod_op(3, b, c);
  }
  return false;
}

struct Instance {
  i32 n = 0, nvars = 0;
  i32 op[4], x[4], y[4], z[4];
};

Instance build_pred(i32 pred) {
  Instance I;
  I.nvars = 3;
  auto push = [&](i32 o, i32 a, i32 b, i32 c) {
    I.op[I.n] = o; I.x[I.n] = a; I.y[I.n] = b; I.z[I.n] = c; ++I.n;
  };
  static const i32 direct[10] = {ORC_EQ, ORC_LEQ, ORC_ADD, ORC_MIN, ORC_MAX,
                                 ORC_MUL, ORC_EDIV, ORC_TDIV, ORC_CDIV, ORC_FDIV};
  if (pred < 10) {
    push(direct[pred], 0, 1, 2);  // constraint pred(y, z, x): x = y op z
  } else {
    // x = y mod z as q = y div z, m = q * z, y = m + x (fresh q = 3, m = 4).
    static const i32 divs[4] = {ORC_EDIV, ORC_TDIV, ORC_CDIV, ORC_FDIV};
    push(divs[pred - 10], 3, 1, 2);
    push(ORC_MUL, 4, 3, 2);
    push(ORC_ADD, 1, 4, 0);
    I.nvars = 5;
  }
  return I;
}

// create_and_interpret_and_tell: vars x,y,z with the given intervals, fresh
// vars top, then install (meet reified x with [0,1]) and the CPU sort.
struct Prepared {
  Instance I;
  i32 store[10];
  bool bot = false;
};

Prepared prepare(i32 pred, Itv x, Itv y, Itv z) {
  Prepared P;
  P.I = build_pred(pred);
  Itv init[5] = {x, y, z, Itv::top(), Itv::top()};
  for (i32 v = 0; v < P.I.nvars; ++v) {
    P.store[2 * v] = init[v].l;
    P.store[2 * v + 1] = init[v].u;
  }
  i32 perm[4];
  int st = orc_install(P.I.n, P.I.op, P.I.x, P.I.y, P.I.z, P.I.nvars, P.store, perm);
  Instance sorted = P.I;
  for (i32 i = 0; i < P.I.n; ++i) {
    sorted.op[i] = P.I.op[perm[i]];
    sorted.x[i] = P.I.x[perm[i]];
    sorted.y[i] = P.I.y[perm[i]];
    sorted.z[i] = P.I.z[perm[i]];
  }
  P.I = sorted;
  P.bot = (st == ORC_FAILED) || store_bot(P.I.nvars, P.store);
  return P;
}

// Hull of the relation's projection over the box (tests/bound_consistency_test.hpp:70-84).
void brute_hull(i32 pred, Itv x, Itv y, Itv z, Itv h[3]) {
  h[0] = h[1] = h[2] = Itv::bot();
  for (i64 a = x.l; a <= x.u; ++a)
    for (i64 b = y.l; b <= y.u; ++b)
      for (i64 c = z.l; c <= z.u; ++c)
        if (pred_holds(pred, a, b, c)) {
          h[0].join(Itv{(i32)a, (i32)a});
          h[1].join(Itv{(i32)b, (i32)b});
          h[2].join(Itv{(i32)c, (i32)c});
        }
}

// deduce_and_test2 (tests/bound_consistency_test.hpp:18-53) followed by the
// entailment checks (:89-109).  Returns the number of violated expectations.
i64 check_case(i32 pred, Prepared &P, const Itv before[3], const Itv after[3],
               bool test_completeness, bool disable_before_test) {
  i64 bad = 0;
  bool has_bot = after[0].is_bot() || after[1].is_bot() || after[2].is_bot();
  i32 *s = P.store;
  if (P.bot) return has_bot ? 0 : 1;
  if (!disable_before_test)
    for (int i = 0; i < 3; ++i)
      if (!(Itv{s[2 * i], s[2 * i + 1]} == before[i])) ++bad;
  bool all_single = true;
  for (int i = 0; i < 3; ++i) all_single &= (before[i].l == before[i].u);
  if (all_single) test_completeness = true;
  i64 out[4];
  int st = gs_fixpoint(P.I.n, P.I.op, P.I.x, P.I.y, P.I.z, P.I.nvars, s, 1 << 20, out);
  if (st == ORC_TIMEOUT) return bad + 1;
  if (st == ORC_FAILED) {
    if (!has_bot) ++bad;
  } else {
    for (int i = 0; i < 3; ++i) {
      Itv got{s[2 * i], s[2 * i + 1]};
      if (test_completeness) {
        if (!(got == after[i])) ++bad;
      } else if (!after[i].is_bot()) {
        // got >= after[i] in the lattice: got contains after[i]
        if (!(got.l <= after[i].l && got.u >= after[i].u)) ++bad;
      }
    }
    bool entailed = true;
    for (i32 i = 0; i < P.I.n; ++i) entailed &= ask(P.I.op[i], P.I.x[i], P.I.y[i], P.I.z[i], s) != 0;
    if (has_bot) {
      if (entailed) ++bad;
    } else if (entailed) {
      for (i64 a = after[0].l; a <= after[0].u; ++a)
        for (i64 b = after[1].l; b <= after[1].u; ++b)
          for (i64 c = after[2].l; c <= after[2].u; ++c)
            if (!pred_holds(pred, a, b, c)) ++bad;
    }
  }
  return bad;
}

}  // namespace

extern "C" {

int orc_deduce(int32_t op, int32_t x, int32_t y, int32_t z, int32_t *store, int *failed) {
  int f = 0;
  int ch = deduce(op, x, y, z, store, &f);
  if (failed && f) *failed = 1;
  return ch ? 1 : 0;
}

int orc_ask(int32_t op, int32_t x, int32_t y, int32_t z, const int32_t *store) {
  return ask(op, x, y, z, store);
}

// ask(bytecode) (pir.hpp:417-438) of op[k] over the private intervals in_lb/in_ub[k][0..2].
void orc_ask_batch(int64_t count, const int32_t *op, const int32_t *in_lb, const int32_t *in_ub, uint8_t *out) {
  const i64 chunk = 1 << 16;
  parallel_for((count + chunk - 1) / chunk, resolve_threads(0), [&](i64 c) {
    for (i64 k = c * chunk; k < std::min(count, (c + 1) * chunk); ++k) {
      i32 s[6];
      for (int j = 0; j < 3; ++j) {
        s[2 * j] = in_lb[3 * k + j];
        s[2 * j + 1] = in_ub[3 * k + j];
      }
      out[k] = orc_ask(op[k], 0, 1, 2, s) ? 1 : 0;
    }
  });
}

void orc_deduce_batch(int64_t count, const int32_t *op, const int32_t *in_lb, const int32_t *in_ub,
                      int32_t *out_lb, int32_t *out_ub, uint8_t *out_changed, uint8_t *out_failed,
                      int64_t *overflows) {
  std::atomic<i64> ovf{0};
  const i64 chunk = 1 << 16;
  parallel_for((count + chunk - 1) / chunk, resolve_threads(0), [&](i64 c) {
    g_overflows = 0;
    for (i64 k = c * chunk; k < std::min(count, (c + 1) * chunk); ++k) {
      i32 s[6];
      for (int j = 0; j < 3; ++j) {
        s[2 * j] = in_lb[3 * k + j];
        s[2 * j + 1] = in_ub[3 * k + j];
      }
      int failed = 0;
      int ch = deduce(op[k], 0, 1, 2, s, &failed);
      for (int j = 0; j < 3; ++j) {
        out_lb[3 * k + j] = s[2 * j];
        out_ub[3 * k + j] = s[2 * j + 1];
      }
      out_changed[k] = ch ? 1 : 0;
      out_failed[k] = (uint8_t)failed;
    }
    ovf += g_overflows;
  });
  if (overflows) *overflows = ovf.load();
}

int orc_store_is_bot(int32_t nvars, const int32_t *store) { return store_bot(nvars, store) ? 1 : 0; }

int orc_install(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                const int32_t *z, int32_t nvars, int32_t *store, int32_t *perm) {
  for (i32 i = 0; i < n; ++i) {
    if (op[i] < 0 || op[i] >= ORC_NUM_OPS) return ORC_EINVAL;
    if (x[i] < 0 || x[i] >= nvars || y[i] < 0 || y[i] >= nvars || z[i] < 0 || z[i] >= nvars)
      return ORC_EINVAL;
  }
  int failed = 0;
  for (i32 i = 0; i < n; ++i)
    if (op[i] == ORC_EQ || op[i] == ORC_LEQ) embed(store, x[i], Itv{0, 1}, &failed);  // pir.hpp:333-335
  if (perm) {
    std::iota(perm, perm + n, 0);
    std::stable_sort(perm, perm + n, [&](i32 a, i32 b) {  // pir.hpp:343-347
      if (op[a] != op[b]) return op[a] < op[b];
      if (y[a] != y[b]) return y[a] < y[b];
      if (x[a] != x[b]) return x[a] < x[b];
      return z[a] < z[b];
    });
  }
  return (failed || store_bot(nvars, store)) ? ORC_FAILED : ORC_OK;
}

int orc_fixpoint(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                 const int32_t *z, int32_t nvars, int32_t *store, int64_t max_sweeps,
                 int64_t *out) {
  return gs_fixpoint(n, op, x, y, z, nvars, store, max_sweeps, out);
}

// Depth-first search (the CPU reference of the search driver): every node is
// the store of its parent with one bisection, brought to its Gauss-Seidel
// fixpoint; a node with all decision variables fixed is a solution; otherwise
// the first unfixed decision variable (order 0) or the one with the smallest
// domain (order 1) is bisected at l + (u - l) / 2, lower half first.
// out_stats: nodes, failures, solutions.  Solutions (decision values) go to
// out_solutions while max_solutions allows (0: count only).
int orc_search(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y, const int32_t *z,
               int32_t nvars, const int32_t *store, int32_t ndec, const int32_t *dec, int32_t order,
               int64_t max_solutions, int64_t max_nodes, int32_t *out_solutions, int64_t *out_stats) {
  std::vector<std::vector<i32>> stack;
  stack.emplace_back(store, store + 2 * (size_t)nvars);
  i64 nodes = 0, fails = 0, sols = 0;
  int status = ORC_OK;
  while (!stack.empty()) {
    if (max_nodes > 0 && nodes >= max_nodes) {
      status = ORC_TIMEOUT;
      break;
    }
    std::vector<i32> s = std::move(stack.back());
    stack.pop_back();
    ++nodes;
    if (gs_fixpoint(n, op, x, y, z, nvars, s.data(), (i64)1 << 40, nullptr) == ORC_FAILED) {
      ++fails;
      continue;
    }
    int best = -1;
    i64 best_w = 0;
    for (int k = 0; k < ndec; ++k) {
      const i64 l = s[2 * (size_t)dec[k]], u = s[2 * (size_t)dec[k] + 1];
      if (l >= u) continue;
      if (order == 0) {
        best = k;
        break;
      }
      if (best < 0 || u - l < best_w) {
        best = k;
        best_w = u - l;
      }
    }
    if (best < 0) {
      if (max_solutions > 0)
        for (int k = 0; k < ndec; ++k) out_solutions[(size_t)sols * ndec + k] = s[2 * (size_t)dec[k]];
      ++sols;
      if (max_solutions > 0 && sols >= max_solutions) break;
      continue;
    }
    const size_t v = (size_t)dec[best];
    const i64 lo = s[2 * v], hi = s[2 * v + 1], mid = lo + (hi - lo) / 2;
    std::vector<i32> right = s;
    right[2 * v] = (i32)(mid + 1);
    s[2 * v + 1] = (i32)mid;
    stack.push_back(std::move(right));
    stack.push_back(std::move(s));
  }
  if (out_stats) {
    out_stats[0] = nodes;
    out_stats[1] = fails;
    out_stats[2] = sols;
  }
  return status;
}

int orc_sweeps(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
               const int32_t *z, int32_t *store, int64_t sweeps, int64_t *out) {
  g_overflows = 0;
  i64 narrowed = 0;
  int failed = 0;
  for (i64 k = 0; k < sweeps; ++k)
    for (i32 i = 0; i < n; ++i) narrowed += deduce(op[i], x[i], y[i], z[i], store, &failed);
  if (out) {
    out[0] = sweeps;
    out[1] = sweeps * (i64)n;
    out[2] = narrowed;
    out[3] = g_overflows;
  }
  return failed ? ORC_FAILED : ORC_OK;
}

int orc_fixpoint_nodes(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                       const int32_t *z, int32_t nvars, const int32_t *base_store,
                       int32_t nnodes, const int32_t *off, const int32_t *var,
                       const int32_t *lb, const int32_t *ub, int64_t max_sweeps,
                       int32_t threads, int32_t *out_store, int32_t *out_status,
                       int64_t *out_stats) {
  parallel_for(nnodes, resolve_threads(threads), [&](i64 j) {
    i32 *s = out_store + (i64)j * 2 * nvars;
    std::memcpy(s, base_store, sizeof(i32) * 2 * (size_t)nvars);
    int failed = 0;
    for (i32 k = off[j]; k < off[j + 1]; ++k) embed(s, var[k], Itv{lb[k], ub[k]}, &failed);
    out_status[j] = gs_fixpoint(n, op, x, y, z, nvars, s, max_sweeps, out_stats + 4 * j);
  });
  return ORC_OK;
}

int orc_fixpoint_instances(int32_t ninst, const int64_t *prop_off, const int64_t *var_off,
                           const int32_t *op, const int32_t *x, const int32_t *y,
                           const int32_t *z, int32_t *store, int64_t max_sweeps,
                           int32_t threads, int32_t install, int32_t *out_status,
                           int64_t *out_stats) {
  parallel_for(ninst, resolve_threads(threads), [&](i64 j) {
    i64 p0 = prop_off[j], p1 = prop_off[j + 1];
    i64 v0 = var_off[j], v1 = var_off[j + 1];
    const i32 n = (i32)(p1 - p0), nv = (i32)(v1 - v0);
    i32 *s = store + 2 * v0;
    if (!install) {
      out_status[j] = gs_fixpoint(n, op + p0, x + p0, y + p0, z + p0, nv, s, max_sweeps, out_stats + 4 * j);
      return;
    }
    // install (pir.hpp:326-352): reified meets and the CPU sort, then Gauss-Seidel
    std::vector<i32> perm((size_t)n), o((size_t)n), a((size_t)n), b((size_t)n), c((size_t)n);
    int st = orc_install(n, op + p0, x + p0, y + p0, z + p0, nv, s, perm.data());
    if (st != ORC_OK) {
      out_status[j] = st;
      for (int k = 0; k < 4; ++k) out_stats[4 * j + k] = 0;
      return;
    }
    for (i32 i = 0; i < n; ++i) {
      o[i] = op[p0 + perm[i]];
      a[i] = x[p0 + perm[i]];
      b[i] = y[p0 + perm[i]];
      c[i] = z[p0 + perm[i]];
    }
    out_status[j] = gs_fixpoint(n, o.data(), a.data(), b.data(), c.data(), nv, s, max_sweeps, out_stats + 4 * j);
  });
  return ORC_OK;
}

int32_t orc_build_pred(int32_t pred, int32_t *op, int32_t *x, int32_t *y, int32_t *z,
                       int32_t *nvars) {
  Instance I = build_pred(pred);
  for (i32 i = 0; i < I.n; ++i) {
    op[i] = I.op[i]; x[i] = I.x[i]; y[i] = I.y[i]; z[i] = I.z[i];
  }
  *nvars = I.nvars;
  return I.n;
}

int64_t orc_div(int32_t op, int64_t a, int64_t b) {
  switch (op) {
    case ORC_TDIV: return tdiv(a, b);
    case ORC_CDIV: return cdiv(a, b);
    case ORC_FDIV: return fdiv(a, b);
    default: return ediv(a, b);
  }
}

int64_t orc_mod(int32_t kind, int64_t a, int64_t b) { return mod_op(kind, a, b); }

// test_bound_propagator_soundness_exhaustive, tests/bound_consistency_test.hpp:155-225:
// one instance over [minval, maxval]^3, snapshot, then for every sub-interval
// triple: restore, embed the triple, fixpoint, compare with the projection.
int64_t orc_check_exhaustive(int32_t pred, int32_t minval, int32_t maxval,
                             int32_t test_completeness, int64_t *out) {
  Prepared base = prepare(pred, Itv{minval, maxval}, Itv{minval, maxval}, Itv{minval, maxval});
  std::vector<Itv> itvs;
  for (i32 l = minval; l <= maxval; ++l)
    for (i32 u = l; u <= maxval; ++u) itvs.push_back(Itv{l, u});
  const i64 K = (i64)itvs.size();
  const i32 W = maxval - minval + 1;
  std::atomic<i64> bad{0}, cases{0}, first{-1};
  parallel_for(K, resolve_threads(0), [&](i64 iy) {
    std::vector<i32> exists(W), minb(W), maxb(W), minc(W), maxc(W);
    i64 local_bad = 0, local_cases = 0;
    for (i64 iz = 0; iz < K; ++iz) {
      Itv yv = itvs[iy], zv = itvs[iz];
      // Per x value: hull of (y, z) over the solutions with that x.
      std::fill(exists.begin(), exists.end(), 0);
      for (i64 b = yv.l; b <= yv.u; ++b)
        for (i64 c = zv.l; c <= zv.u; ++c)
          for (i64 a = minval; a <= maxval; ++a) {
            if (!pred_holds(pred, a, b, c)) continue;
            i32 k = (i32)(a - minval);
            if (!exists[k]) {
              exists[k] = 1;
              minb[k] = maxb[k] = (i32)b;
              minc[k] = maxc[k] = (i32)c;
            } else {
              minb[k] = std::min<i32>(minb[k], (i32)b); maxb[k] = std::max<i32>(maxb[k], (i32)b);
              minc[k] = std::min<i32>(minc[k], (i32)c); maxc[k] = std::max<i32>(maxc[k], (i32)c);
            }
          }
      for (i64 ix = 0; ix < K; ++ix) {
        Itv xv = itvs[ix];
        Itv h[3] = {Itv::bot(), Itv::bot(), Itv::bot()};
        for (i32 a = xv.l; a <= xv.u; ++a) {
          i32 k = a - minval;
          if (!exists[k]) continue;
          h[0].join(Itv{a, a});
          h[1].join(Itv{minb[k], maxb[k]});
          h[2].join(Itv{minc[k], maxc[k]});
        }
        Prepared P = base;
        int failed = 0;
        embed(P.store, 0, xv, &failed);
        embed(P.store, 1, yv, &failed);
        embed(P.store, 2, zv, &failed);
        P.bot = store_bot(P.I.nvars, P.store);
        Itv before[3] = {{P.store[0], P.store[1]}, {P.store[2], P.store[3]}, {P.store[4], P.store[5]}};
        i64 b = check_case(pred, P, before, h, test_completeness != 0, false);
        ++local_cases;
        if (b) {
          local_bad += b;
          i64 idx = (iy * K + iz) * K + ix;
          i64 expected = -1;
          first.compare_exchange_strong(expected, idx);
        }
      }
    }
    bad += local_bad;
    cases += local_cases;
  });
  if (out) {
    out[0] = cases.load();
    out[1] = first.load();
  }
  return bad.load();
}

// test_bound_propagator_soundness, tests/bound_consistency_test.hpp:55-113.
int64_t orc_check_listed(int32_t pred, int32_t test_completeness, int64_t *out) {
  const i32 minval = -20, maxval = 20;
  const Itv itvs[] = {{minval, minval}, {minval + 1, maxval - 1}, {minval, -3}, {minval, -2},
                      {minval, 0}, {minval, maxval}, {-2, -1}, {-1, 0}, {-2, 2}, {-1, -1},
                      {0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {0, maxval}, {2, maxval},
                      {3, maxval}, {maxval, maxval}, {1, 0}, {2, 10}, {-25, 25}, {-2, 3}};
  const i64 K = sizeof(itvs) / sizeof(itvs[0]);
  // eq_reif / le_reif disable the "before" check (tests/pir_test.cpp:140-141).
  const bool disable_before = (pred == 0 || pred == 1);
  std::atomic<i64> bad{0}, first{-1};
  parallel_for(K * K * K, resolve_threads(0), [&](i64 idx) {
    Itv x = itvs[idx / (K * K)], y = itvs[(idx / K) % K], z = itvs[idx % K];
    Itv h[3];
    brute_hull(pred, x, y, z, h);
    Prepared P = prepare(pred, x, y, z);
    Itv before[3] = {x, y, z};
    i64 b = check_case(pred, P, before, h, test_completeness != 0, disable_before);
    if (b) {
      bad += b;
      i64 expected = -1;
      first.compare_exchange_strong(expected, idx);
    }
  });
  if (out) {
    out[0] = K * K * K;
    out[1] = first.load();
  }
  return bad.load();
}

// test_bound_propagator_completeness, tests/bound_consistency_test.hpp:115-153.
int64_t orc_check_completeness(int32_t pred, int32_t with_fixpoint, int64_t *out) {
  const i32 minval = -5, maxval = 5;
  i64 bad = 0, cases = 0, first = -1;
  for (i32 i = minval; i < maxval; ++i)
    for (i32 j = minval; j < maxval; ++j)
      for (i32 k = minval; k < maxval; ++k) {
        Itv x{i, i}, y{j, j}, z{k, k};
        Prepared P = prepare(pred, x, y, z);
        i64 b = 0;
        if (with_fixpoint && !P.bot) {
          i64 o[4];
          int st = gs_fixpoint(P.I.n, P.I.op, P.I.x, P.I.y, P.I.z, P.I.nvars, P.store, 1 << 20, o);
          if (st == ORC_FAILED) P.bot = true;
        }
        bool entailed = true;
        if (P.bot) entailed = false;
        else
          for (i32 q = 0; q < P.I.n; ++q)
            entailed &= ask(P.I.op[q], P.I.x[q], P.I.y[q], P.I.z[q], P.store) != 0;
        Itv before[3] = {x, y, z};
        if (!pred_holds(pred, i, j, k)) {
          if (entailed) ++b;
          Itv bots[3] = {Itv::bot(), Itv::bot(), Itv::bot()};
          b += check_case(pred, P, before, bots, true, false);
        } else {
          if (!entailed) ++b;
          b += check_case(pred, P, before, before, true, false);
        }
        ++cases;
        if (b && first < 0) first = cases - 1;
        bad += b;
      }
  if (out) {
    out[0] = cases;
    out[1] = first;
  }
  return bad;
}

}  // extern "C"
