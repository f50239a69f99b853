// CPU restatement of lala-pc's PC tree propagators — TEST INFRASTRUCTURE ONLY.
// See pc_oracle.h for what it restates and who may call it.
//
// Interval arithmetic (lala-core's Interval<ZLB<int>>, not vendored), restated
// from its meaning:
//   * an interval is [l, u] of int32 with l = INT32_MIN meaning -inf and
//     u = INT32_MAX meaning +inf; it is empty (bot) when l > u, l = +inf or
//     u = -inf.  An operator with an empty operand gives the empty interval.
//   * NEG, ABS, ADD, SUB, MIN, MAX, MUL: the exact image, computed in int64 on
//     the extended integers (0 * inf = 0) and clamped to int32 when it becomes
//     a bound (the reference overflows there; parity with it is not claimed
//     beyond int32).
//   * TDIV, FDIV, CDIV, EDIV: the exact hull of { y op z : y in Y, z in Z,
//     z != 0 } (Z = [0, 0] gives the empty interval).  The quotient is
//     monotone in each argument on a sign-definite divisor range, so the hull
//     is taken over the corners of the negative and of the positive part of Z,
//     on the extended integers: inf / z is +-inf, y / inf is the rounded sign
//     of a vanishing quotient (0, or -1 / +1 for the floor / ceiling side),
//     and inf / inf counts as a large y over a larger z.
//   * additive_inverse (GroupAdd::rev_op, terms.hpp:190-194) negates each
//     bound without swapping them: all + inverse(t) = [all.l - t.l,
//     all.u - t.u], the sum of the other operands of an n-ary sum.
//   * LB::prev(k) = k + 1 and UB::prev(k) = k - 1 (the next bound inwards;
//     tests/pc_test.cpp:386-390 pins x != 10 on [1, 10] to [1, 9]); infinities
//     are their own prev.
// Every operator is monotone for inclusion, so a fixpoint of the propagators
// does not depend on the order they run in (NaryMul's early exit on a product
// of exactly [0, 0], terms.hpp:487, is the exception: it skips the narrowing
// that a larger product would do).
#include "pc_oracle.h"

#include <algorithm>
#include <climits>
#include <cstdint>
#include <vector>

namespace {

using i64 = long long;
constexpr int32_t MINF = INT32_MIN, INF = INT32_MAX;

struct I {
  int32_t l, u;
};

I top() { return I{MINF, INF}; }
I empty() { return I{INF, MINF}; }
bool is_bot(I a) { return a.l > a.u || a.l == INF || a.u == MINF; }
I meet(I a, I b) { return I{std::max(a.l, b.l), std::min(a.u, b.u)}; }
// fjoin: the convex hull, with bot as the unit
I fjoin(I a, I b) {
  if (is_bot(a)) return b;
  if (is_bot(b)) return a;
  return I{std::min(a.l, b.l), std::max(a.u, b.u)};
}
// a >= eq_zero(): [0, 0] is included in a
bool has0(I a) { return !is_bot(a) && a.l <= 0 && a.u >= 0; }
// a <= [v, v]: a is [v, v] or empty
bool below_point(I a, int32_t v) { return is_bot(a) || (a.l == v && a.u == v); }
bool is_point(I a, int32_t v) { return a.l == v && a.u == v; }
int32_t clamp(i64 v) { return (int32_t)(v > INF ? (i64)INF : (v < MINF ? (i64)MINF : v)); }
int32_t prev_lb(int32_t k) { return (k == MINF || k == INF) ? k : k + 1; }
int32_t prev_ub(int32_t k) { return (k == MINF || k == INF) ? k : k - 1; }

// -u as a lower bound, -l as an upper bound
int32_t neg_of_ub(int32_t u) { return u == INF ? MINF : clamp(-(i64)u); }
int32_t neg_of_lb(int32_t l) { return l == MINF ? INF : clamp(-(i64)l); }

I neg(I a) {
  if (is_bot(a)) return empty();
  return I{neg_of_ub(a.u), neg_of_lb(a.l)};
}
I add(I a, I b) {
  if (is_bot(a) || is_bot(b)) return empty();
  return I{(a.l == MINF || b.l == MINF) ? MINF : clamp((i64)a.l + b.l),
           (a.u == INF || b.u == INF) ? INF : clamp((i64)a.u + b.u)};
}
I sub(I a, I b) { return add(a, neg(b)); }
I imin(I a, I b) {
  if (is_bot(a) || is_bot(b)) return empty();
  return I{std::min(a.l, b.l), std::min(a.u, b.u)};
}
I imax(I a, I b) {
  if (is_bot(a) || is_bot(b)) return empty();
  return I{std::max(a.l, b.l), std::max(a.u, b.u)};
}
I iabs(I a) {
  if (is_bot(a)) return empty();
  if (a.l >= 0) return a;
  if (a.u <= 0) return neg(a);
  return I{0, std::max(neg_of_lb(a.l), a.u)};
}

// extended integers for the products
struct X {
  int inf;  // -1: -inf, +1: +inf, 0: finite v
  i64 v;
};
X lbx(int32_t l) { return l == MINF ? X{-1, 0} : X{0, l}; }
X ubx(int32_t u) { return u == INF ? X{1, 0} : X{0, u}; }
int sgn(X p) { return p.inf ? p.inf : (p.v > 0) - (p.v < 0); }
X mulx(X p, X q) {
  if (sgn(p) == 0 || sgn(q) == 0) return X{0, 0};
  if (p.inf || q.inf) return X{sgn(p) * sgn(q), 0};
  return X{0, p.v * q.v};
}
bool lessx(X p, X q) {
  if (p.inf != q.inf) return p.inf < q.inf;
  return p.inf == 0 && p.v < q.v;
}
I imul(I a, I b) {
  if (is_bot(a) || is_bot(b)) return empty();
  const X c[4] = {mulx(lbx(a.l), lbx(b.l)), mulx(lbx(a.l), ubx(b.u)), mulx(ubx(a.u), lbx(b.l)),
                  mulx(ubx(a.u), ubx(b.u))};
  X lo = c[0], hi = c[0];
  for (int k = 1; k < 4; ++k) {
    if (lessx(c[k], lo)) lo = c[k];
    if (lessx(hi, c[k])) hi = c[k];
  }
  const int32_t l = lo.inf < 0 ? MINF : (lo.inf > 0 ? INF : clamp(lo.v));
  const int32_t u = hi.inf > 0 ? INF : (hi.inf < 0 ? MINF : clamp(hi.v));
  return I{l, u};
}

// integer divisions by their definitions, b != 0
i64 qdiv(int op, i64 a, i64 b) {
  const i64 q = a / b, r = a % b;
  switch (op) {
    case ORC_PC_TDIV: return q;
    case ORC_PC_FDIV: return (r != 0 && ((r < 0) != (b < 0))) ? q - 1 : q;
    case ORC_PC_CDIV: return (r != 0 && ((r < 0) == (b < 0))) ? q + 1 : q;
    default: return r < 0 ? (b > 0 ? q - 1 : q + 1) : q;  // Euclidean
  }
}
// y / z on the extended integers, z != 0 (sign-definite)
X qx(int op, X y, X z) {
  if (!z.inf) {
    if (!y.inf) return X{0, qdiv(op, y.v, z.v)};
    return X{sgn(y) * sgn(z), 0};
  }
  const int sy = sgn(y), s = sy * z.inf;  // sign of the vanishing quotient
  switch (op) {
    case ORC_PC_TDIV: return X{0, 0};
    case ORC_PC_FDIV: return X{0, s < 0 ? -1 : 0};
    case ORC_PC_CDIV: return X{0, s > 0 ? 1 : 0};
    default: return X{0, z.inf > 0 ? (sy < 0 ? -1 : 0) : (sy < 0 ? 1 : 0)};  // floor for z > 0, ceiling for z < 0
  }
}
I idiv(int op, I a, I b) {
  if (is_bot(a) || is_bot(b) || is_point(b, 0)) return empty();
  bool any = false;
  X lo{0, 0}, hi{0, 0};
  auto part = [&](X zl, X zu) {
    const X c[4] = {qx(op, lbx(a.l), zl), qx(op, lbx(a.l), zu), qx(op, ubx(a.u), zl), qx(op, ubx(a.u), zu)};
    for (const X &q : c) {
      if (!any || lessx(q, lo)) lo = q;
      if (!any || lessx(hi, q)) hi = q;
      any = true;
    }
  };
  if (b.l <= -1) part(lbx(b.l), X{0, std::min<i64>(b.u, -1)});
  if (b.u >= 1) part(X{0, std::max<i64>(b.l, 1)}, ubx(b.u));
  return I{lo.inf < 0 ? MINF : (lo.inf > 0 ? INF : clamp(lo.v)), hi.inf > 0 ? INF : (hi.inf < 0 ? MINF : clamp(hi.v))};
}
// GroupAdd::rev_op: all + additive_inverse(t)
I rev_add(I all, I t) {
  if (is_bot(all) || is_bot(t)) return empty();
  return I{(all.l == MINF || t.l == MINF) ? MINF : clamp((i64)all.l - t.l),
           (all.u == INF || t.u == INF) ? INF : clamp((i64)all.u - t.u)};
}

I itv_op(int op, I a, I b) {
  switch (op) {
    case ORC_PC_NEG: return neg(a);
    case ORC_PC_ABS: return iabs(a);
    case ORC_PC_ADD: return add(a, b);
    case ORC_PC_SUB: return sub(a, b);
    case ORC_PC_MUL: return imul(a, b);
    case ORC_PC_TDIV:
    case ORC_PC_FDIV:
    case ORC_PC_CDIV:
    case ORC_PC_EDIV: return idiv(op, a, b);
    case ORC_PC_MIN: return imin(a, b);
    case ORC_PC_MAX: return imax(a, b);
    default: return top();
  }
}

bool is_term(int32_t k) { return k >= ORC_PC_VAR && k <= ORC_PC_NMUL; }
bool is_formula(int32_t k) { return (k >= ORC_PC_PVAR && k <= ORC_PC_XOR) || k == ORC_PC_AE; }
bool is_item(int32_t k) { return k >= ORC_PC_TELL && k <= ORC_PC_NASK_OUT; }
bool is_division(int32_t k) { return k >= ORC_PC_TDIV && k <= ORC_PC_EDIV; }

// ------------------------------------------------------------- evaluator --
// The store is read from `s` and joined into `w`.  With w == s this is the
// reference's sequential semantics (a deduction reads its own earlier
// joins); with w != s every read of a round sees the round's initial store
// (the Jacobi rounds of the GPU engine).
struct Eval {
  const int32_t *k, *a, *b, *c;
  int32_t *s;
  int32_t failed;
  i64 narrowed;
  int32_t *w = nullptr;

  I load(int v) const { return I{s[2 * v], s[2 * v + 1]}; }

  // VStore::embed: meet into the variable, true iff a bound moved; an empty
  // result makes the store bot
  bool store_embed(int v, I u) {
    int32_t *out = w ? w : s;
    const I cur = load(v);
    bool ch = false;
    if (u.l > cur.l) {
      out[2 * v] = std::max(out[2 * v], u.l);
      ch = true;
      ++narrowed;
    }
    if (u.u < cur.u) {
      out[2 * v + 1] = std::min(out[2 * v + 1], u.u);
      ch = true;
      ++narrowed;
    }
    if (ch && is_bot(meet(cur, u))) failed = 1;
    return ch;
  }

  // ---- terms (terms.hpp) ----
  I project(int n) {
    const int32_t kind = k[n];
    switch (kind) {
      case ORC_PC_VAR: return load(a[n]);                      // Variable::project, terms.hpp:69
      case ORC_PC_CONST: return I{a[n], b[n]};                 // Constant::project :35
      case ORC_PC_FORMULA: return f_project(a[n]);             // Formula::project, formula.hpp:1097
      case ORC_PC_NEG:
      case ORC_PC_ABS: return itv_op(kind, project(a[n]), top());  // Unary::project :155
      case ORC_PC_NADD:
      case ORC_PC_NMUL: {                                      // Nary::project :465
        I accu = project(a[a[n]]);
        for (int i = 1; i < b[n]; ++i)
          accu = itv_op(kind == ORC_PC_NADD ? ORC_PC_ADD : ORC_PC_MUL, accu, project(a[a[n] + i]));
        return accu;
      }
      default: return itv_op(kind, project(a[n]), project(b[n]));  // Binary::project :399
    }
  }

  // Group*::left_residual (terms.hpp:196-324): the operand x of x op y = u
  I left_residual(int32_t kind, I u, I y) {
    switch (kind) {
      case ORC_PC_ADD: return sub(u, y);
      case ORC_PC_SUB: return add(u, y);
      case ORC_PC_MUL: return (has0(u) && has0(y)) ? top() : idiv(ORC_PC_EDIV, u, y);
      case ORC_PC_MIN:
      case ORC_PC_MAX:
        if (is_bot(meet(u, y))) return u;
        return kind == ORC_PC_MIN ? I{u.l, INF} : I{MINF, u.u};
      default: {  // GroupDiv: u * y, then the upper bound joined with prev(y.ub)
        I r = imul(u, y);
        r.u = std::max(r.u, prev_ub(y.u));
        return r;
      }
    }
  }

  // Group*::right_residual: the operand y of x op y = u; `r` is top, or for
  // a division y's current interval (Binary::embed :389-393)
  I right_residual(int32_t kind, I u, I x, I r) {
    switch (kind) {
      case ORC_PC_SUB: return sub(x, u);
      case ORC_PC_ADD:
      case ORC_PC_MUL:
      case ORC_PC_MIN:
      case ORC_PC_MAX: return left_residual(kind, u, x);
      default:  // GroupDiv::right_residual :279
        if (r.l == 0) r.l = std::max(r.l, 1);
        if (r.u == 0) r.u = std::min(r.u, -1);
        if (!has0(x) && !is_point(u, 0)) r = meet(r, idiv(kind, x, u));
        return r;
    }
  }

  bool embed(int n, I u) {
    const int32_t kind = k[n];
    switch (kind) {
      case ORC_PC_VAR: return store_embed(a[n], u);  // Variable::embed :65
      case ORC_PC_CONST: return false;                // Constant::embed :34
      case ORC_PC_FORMULA: return f_embed(a[n], u);
      case ORC_PC_NEG: return embed(a[n], neg(u));    // NegOp::residual :95
      case ORC_PC_ABS: return embed(a[n], fjoin(u, neg(u)));  // AbsOp::residual :112
      case ORC_PC_NADD:
      case ORC_PC_NMUL: {  // Nary::embed :480
        const I all = project(n);
        bool ch = false;
        if (kind == ORC_PC_NMUL && is_point(all, 0)) return false;  // GroupMul::is_absorbing
        for (int i = 0; i < b[n]; ++i) {
          const int t = a[a[n] + i];
          const I tmp = project(t);
          I tmp2, res;
          if (kind == ORC_PC_NADD) {
            tmp2 = rev_add(all, tmp);  // GroupAdd::rev_op
            res = sub(u, tmp2);
          } else {
            tmp2 = idiv(ORC_PC_EDIV, all, tmp);  // GroupMul::rev_op
            res = left_residual(ORC_PC_MUL, u, tmp2);
          }
          ch |= embed(t, res);
        }
        return ch;
      }
      default: {  // Binary::embed :376
        const int x = a[n], y = b[n];
        bool ch = false;
        if (k[x] != ORC_PC_CONST) ch |= embed(x, left_residual(kind, u, project(y)));
        if (k[y] != ORC_PC_CONST) {
          const I xt = project(x);
          const I r = is_division(kind) ? project(y) : top();
          ch |= embed(y, right_residual(kind, u, xt, r));
        }
        return ch;
      }
    }
  }

  // ---- formulas (formula.hpp) ----
  I f_project(int n) {
    if (failed) return empty();
    I r = I{0, 1};
    if (ask(n)) r = meet(r, I{1, 1});
    if (nask(n)) r = meet(r, I{0, 0});
    return r;
  }
  bool f_embed(int n, I u) {  // Formula::embed, formula.hpp:1090
    if (below_point(u, 1)) return deduce(n);
    if (below_point(u, 0)) return contradeduce(n);
    return false;
  }

  bool cmp_ask(int32_t kind, int n) {
    const I l = project(a[n]), r = project(b[n]);
    switch (kind) {
      case ORC_PC_EQ: return l.l == r.l && l.u == r.u && l.l == l.u;  // Equality::ask_impl :620
      case ORC_PC_NEQ: return is_bot(meet(l, r));
      case ORC_PC_LEQ: return l.u <= r.l;                               // Inequality::ask_impl :758
      default: return l.l > r.u;                                        // GT
    }
  }
  static int32_t negated(int32_t kind) {
    switch (kind) {
      case ORC_PC_EQ: return ORC_PC_NEQ;
      case ORC_PC_NEQ: return ORC_PC_EQ;
      case ORC_PC_LEQ: return ORC_PC_GT;
      default: return ORC_PC_LEQ;
    }
  }
  bool cmp_deduce(int32_t kind, int n) {
    const int L = a[n], R = b[n];
    bool ch = false;
    switch (kind) {
      case ORC_PC_EQ:  // Equality::deduce_impl<false> :634
        if (k[R] != ORC_PC_CONST) ch = embed(R, project(L));
        if (k[L] != ORC_PC_CONST) ch |= embed(L, project(R));
        return ch;
      case ORC_PC_NEQ: {  // Equality::deduce_impl<true> :634
        if (k[R] != ORC_PC_CONST) {
          const I l = project(L);
          if (l.l == l.u) {
            const I r = project(R);
            I lo = r, hi = r;
            lo.l = std::max(lo.l, prev_lb(l.l));
            hi.u = std::min(hi.u, prev_ub(l.u));
            return embed(R, fjoin(lo, hi));
          }
        }
        if (k[L] != ORC_PC_CONST) {
          const I r = project(R);
          if (r.l == r.u) {
            const I l = project(L);
            I lo = l, hi = l;
            lo.l = std::max(lo.l, prev_lb(r.l));
            hi.u = std::min(hi.u, prev_ub(r.u));
            return embed(L, fjoin(lo, hi));
          }
        }
        return false;
      }
      case ORC_PC_LEQ:  // Inequality::deduce_impl<false> :774
        if (k[L] != ORC_PC_CONST) ch |= embed(L, I{MINF, project(R).u});
        if (k[R] != ORC_PC_CONST) ch = embed(R, I{project(L).l, INF});  // '=' as in the reference
        return ch;
      default: {  // GT, Inequality::deduce_impl<true> :774
        if (k[L] != ORC_PC_CONST) {
          I r = project(R);
          r.l = std::max(r.l, prev_lb(r.l));
          ch = embed(L, I{r.l, INF});
        }
        if (k[R] != ORC_PC_CONST) {
          I l = project(L);
          l.u = std::min(l.u, prev_ub(l.u));
          ch |= embed(R, I{MINF, l.u});
        }
        return ch;
      }
    }
  }

  // AbstractElement (formula.hpp:14-78): the store's own ask (every item's
  // variable inside the item's interval) and deduce (meet every item), over
  // the items of one kind
  // item: ORC_PC_ASK or ORC_PC_NASK; the _OUT items of the same list ask
  // that the variable misses the interval
  bool ae_ask(int n, int32_t item) {
    const int32_t out = item + 2;
    for (int i = a[n]; i < a[n] + b[n]; ++i) {
      if (k[i] != item && k[i] != out) continue;
      const I x = load(a[i]);
      if (is_bot(x)) continue;
      if (k[i] == item ? !(x.l >= b[i] && x.u <= c[i]) : !is_bot(meet(x, I{b[i], c[i]}))) return false;
    }
    return true;
  }
  bool ae_tell(int n, int32_t item) {
    bool ch = false;
    for (int i = a[n]; i < a[n] + b[n]; ++i)
      if (k[i] == item) ch |= store_embed(a[i], I{b[i], c[i]});
    return ch;
  }

  bool ask(int n) {
    const int32_t kind = k[n];
    switch (kind) {
      case ORC_PC_AE: return ae_ask(n, ORC_PC_ASK);
      case ORC_PC_PVAR: return !has0(load(a[n]));           // VariableLiteral::ask_impl :101
      case ORC_PC_NVAR: return below_point(load(a[n]), 0);
      case ORC_PC_TRUE: return true;
      case ORC_PC_FALSE: return failed != 0;
      case ORC_PC_AND: return ask(a[n]) && ask(b[n]);
      case ORC_PC_OR: return ask(a[n]) || ask(b[n]);
      case ORC_PC_EQUIV: return (ask(a[n]) && ask(b[n])) || (nask(a[n]) && nask(b[n]));
      case ORC_PC_IMPLY: return nask(a[n]) || ask(b[n]);
      case ORC_PC_XOR: return (ask(a[n]) && nask(b[n])) || (nask(a[n]) && ask(b[n]));
      default: return cmp_ask(kind, n);
    }
  }
  bool nask(int n) {
    const int32_t kind = k[n];
    switch (kind) {
      case ORC_PC_AE: return ae_ask(n, ORC_PC_NASK);
      case ORC_PC_PVAR: return below_point(load(a[n]), 0);
      case ORC_PC_NVAR: return !has0(load(a[n]));
      case ORC_PC_TRUE: return failed != 0;
      case ORC_PC_FALSE: return true;
      case ORC_PC_AND: return nask(a[n]) || nask(b[n]);
      case ORC_PC_OR: return nask(a[n]) && nask(b[n]);
      case ORC_PC_EQUIV: return (ask(a[n]) && nask(b[n])) || (nask(a[n]) && ask(b[n]));
      case ORC_PC_IMPLY: return ask(a[n]) && nask(b[n]);
      case ORC_PC_XOR: return (ask(a[n]) && ask(b[n])) || (ask(a[n]) && nask(b[n]));  // as written, formula.hpp:552-556
      default: return cmp_ask(negated(kind), n);
    }
  }
  bool deduce(int n) {
    const int32_t kind = k[n];
    const int f = a[n], g = b[n];
    switch (kind) {
      case ORC_PC_AE: return ae_tell(n, ORC_PC_TELL);
      case ORC_PC_PVAR: return store_embed(a[n], I{1, 1});
      case ORC_PC_NVAR: return store_embed(a[n], I{0, 0});
      case ORC_PC_TRUE: return false;
      case ORC_PC_FALSE:
        if (!failed) {
          failed = 1;
          return true;
        }
        return false;
      case ORC_PC_AND: {
        bool ch = deduce(f);
        ch |= deduce(g);
        return ch;
      }
      case ORC_PC_OR:
        if (nask(f)) return deduce(g);
        if (nask(g)) return deduce(f);
        return false;
      case ORC_PC_EQUIV:
        if (ask(f)) return deduce(g);
        if (nask(f)) return contradeduce(g);
        if (ask(g)) return deduce(f);
        if (nask(g)) return contradeduce(f);
        return false;
      case ORC_PC_IMPLY:
        if (ask(f)) return deduce(g);
        if (nask(g)) return contradeduce(f);
        return false;
      case ORC_PC_XOR:
        if (ask(f)) return contradeduce(g);
        if (nask(f)) return deduce(g);
        if (ask(g)) return contradeduce(f);
        if (nask(g)) return deduce(f);
        return false;
      default: return cmp_deduce(kind, n);
    }
  }
  bool contradeduce(int n) {
    const int32_t kind = k[n];
    const int f = a[n], g = b[n];
    switch (kind) {
      case ORC_PC_AE: return ae_tell(n, ORC_PC_NTELL);
      case ORC_PC_PVAR: return store_embed(a[n], I{0, 0});
      case ORC_PC_NVAR: return store_embed(a[n], I{1, 1});
      case ORC_PC_TRUE:
        if (!failed) {
          failed = 1;
          return true;
        }
        return false;
      case ORC_PC_FALSE: return false;
      case ORC_PC_AND:
        if (ask(f)) return contradeduce(g);
        if (ask(g)) return contradeduce(f);
        return false;
      case ORC_PC_OR: {
        bool ch = contradeduce(f);
        ch |= contradeduce(g);
        return ch;
      }
      case ORC_PC_EQUIV:
        if (ask(f)) return contradeduce(g);
        if (nask(f)) return deduce(g);
        if (ask(g)) return contradeduce(f);
        if (nask(g)) return deduce(f);
        return false;
      case ORC_PC_IMPLY:
        if (ask(f)) return contradeduce(g);
        if (nask(g)) return deduce(f);
        return false;
      case ORC_PC_XOR:
        if (ask(f)) return deduce(g);
        if (nask(f)) return contradeduce(g);
        if (ask(g)) return deduce(f);
        if (nask(g)) return contradeduce(f);
        return false;
      default: return cmp_deduce(negated(kind), n);
    }
  }
};

bool store_has_bot(int32_t nvars, const int32_t *s) {
  for (int32_t v = 0; v < nvars; ++v)
    if (is_bot(I{s[2 * v], s[2 * v + 1]})) return true;
  return false;
}

std::vector<i64> lengths(int32_t nnodes, const int32_t *k, const int32_t *a, const int32_t *b) {
  std::vector<i64> len((size_t)nnodes, 1);
  auto cap = [](i64 v) { return std::min<i64>(v, (i64)1 << 40); };
  for (int32_t i = 0; i < nnodes; ++i) {
    const int32_t kind = k[i];
    if (kind == ORC_PC_FORMULA || kind == ORC_PC_ARG) len[(size_t)i] = len[(size_t)a[i]];
    else if (kind == ORC_PC_NEG || kind == ORC_PC_ABS) len[(size_t)i] = cap(1 + len[(size_t)a[i]]);
    else if (kind == ORC_PC_NADD || kind == ORC_PC_NMUL) {
      i64 s = 1;
      for (int j = 0; j < b[i]; ++j) s = cap(s + len[(size_t)(a[i] + j)]);
      len[(size_t)i] = s;
    } else if ((kind >= ORC_PC_ADD && kind <= ORC_PC_MAX) || (kind >= ORC_PC_LEQ && kind <= ORC_PC_XOR))
      len[(size_t)i] = cap(1 + len[(size_t)a[i]] + len[(size_t)b[i]]);
  }
  return len;
}

}  // namespace

extern "C" {

int32_t orc_pc_validate(int32_t nnodes, const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c,
                        int32_t nprops, const int32_t *roots, int32_t nvars) {
  std::vector<int32_t> depth((size_t)std::max(nnodes, 0), 1);
  auto child = [&](int32_t i, int32_t x, bool term) {
    return x >= 0 && x < i && (term ? is_term(k[x]) : is_formula(k[x]));
  };
  for (int32_t i = 0; i < nnodes; ++i) {
    const int32_t kind = k[i];
    bool ok = c[i] == 0 || is_item(kind);
    int32_t d = 1;
    switch (kind) {
      case ORC_PC_TELL:
      case ORC_PC_NTELL:
      case ORC_PC_ASK:
      case ORC_PC_NASK: ok = a[i] >= 0 && a[i] < nvars; break;
      case ORC_PC_AE:
        ok = ok && b[i] >= 0 && a[i] >= 0 && (int64_t)a[i] + b[i] <= i;
        for (int32_t j = 0; ok && j < b[i]; ++j) ok = is_item(k[a[i] + j]);
        break;
      case ORC_PC_VAR:
      case ORC_PC_PVAR:
      case ORC_PC_NVAR: ok = ok && a[i] >= 0 && a[i] < nvars; break;
      case ORC_PC_CONST:
      case ORC_PC_TRUE:
      case ORC_PC_FALSE: break;
      case ORC_PC_FORMULA: ok = ok && child(i, a[i], false); if (ok) d = 1 + depth[(size_t)a[i]]; break;
      case ORC_PC_NEG:
      case ORC_PC_ABS:
      case ORC_PC_ARG: ok = ok && child(i, a[i], true); if (ok) d = (kind == ORC_PC_ARG ? 0 : 1) + depth[(size_t)a[i]]; break;
      case ORC_PC_NADD:
      case ORC_PC_NMUL:
        ok = ok && b[i] >= 1 && a[i] >= 0 && (int64_t)a[i] + b[i] <= i;
        for (int32_t j = 0; ok && j < b[i]; ++j) {
          ok = k[a[i] + j] == ORC_PC_ARG;
          if (ok) d = std::max(d, 1 + depth[(size_t)(a[i] + j)]);
        }
        break;
      default:
        if ((kind >= ORC_PC_ADD && kind <= ORC_PC_MAX) || (kind >= ORC_PC_LEQ && kind <= ORC_PC_NEQ))
          ok = ok && child(i, a[i], true) && child(i, b[i], true);
        else if (kind >= ORC_PC_AND && kind <= ORC_PC_XOR)
          ok = ok && child(i, a[i], false) && child(i, b[i], false);
        else
          ok = false;
        if (ok) d = 1 + std::max(depth[(size_t)a[i]], depth[(size_t)b[i]]);
    }
    if (!ok) return -1 - i;
    depth[(size_t)i] = d;
  }
  int32_t best = 1;
  for (int32_t p = 0; p < nprops; ++p) {
    if (roots[p] < 0 || roots[p] >= nnodes || !is_formula(k[roots[p]])) return -1 - nnodes;
    best = std::max(best, depth[(size_t)roots[p]]);
  }
  return best;
}

void orc_pc_order(int32_t nnodes, const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *,
                  int32_t nprops, const int32_t *roots, int32_t *out) {
  const std::vector<i64> len = lengths(nnodes, k, a, b);
  std::vector<int32_t> r(roots, roots + nprops);
  std::stable_sort(r.begin(), r.end(), [&](int32_t x, int32_t y) {
    if (k[x] != k[y]) return k[x] < k[y];
    return len[(size_t)x] < len[(size_t)y];
  });
  std::copy(r.begin(), r.end(), out);
}

int32_t orc_pc_deduce(const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c, int32_t root,
                      int32_t *store, int32_t *failed, int64_t *narrowed) {
  Eval e{k, a, b, c, store, failed ? *failed : 0, 0};
  const bool ch = e.deduce(root);
  if (failed) *failed = e.failed;
  if (narrowed) *narrowed = e.narrowed;
  return ch ? 1 : 0;
}

int32_t orc_pc_ask(const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c, int32_t root,
                   const int32_t *store, int32_t failed) {
  Eval e{k, a, b, c, const_cast<int32_t *>(store), failed, 0};
  return e.ask(root) ? 1 : 0;
}

void orc_pc_project(const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c, int32_t node,
                    const int32_t *store, int32_t *out_lb, int32_t *out_ub) {
  Eval e{k, a, b, c, const_cast<int32_t *>(store), 0, 0};
  const I r = e.project(node);
  *out_lb = r.l;
  *out_ub = r.u;
}

int32_t orc_pc_embed(const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c, int32_t node,
                     int32_t lb, int32_t ub, int32_t *store, int32_t *failed) {
  Eval e{k, a, b, c, store, failed ? *failed : 0, 0};
  const bool ch = e.embed(node, I{lb, ub});
  if (failed) *failed = e.failed;
  return ch ? 1 : 0;
}

int32_t orc_pc_fixpoint(int32_t nnodes, const int32_t *k, const int32_t *a, const int32_t *b, const int32_t *c,
                        int32_t nprops, const int32_t *roots, int32_t nvars, int32_t *store, int64_t max_sweeps,
                        int64_t *out) {
  int64_t sweeps = 0, execs = 0, any_changed = 0;
  (void)nnodes;
  Eval e{k, a, b, c, store, store_has_bot(nvars, store) ? 1 : 0, 0};
  int32_t status = 0;
  if (e.failed) status = 1;
  while (!status) {
    const i64 before = e.narrowed;
    for (int32_t p = 0; p < nprops; ++p) {
      any_changed |= e.deduce(roots[p]) ? 1 : 0;
      ++execs;
      if (e.failed) break;
    }
    ++sweeps;
    if (e.failed) status = 1;
    else if (e.narrowed == before) break;
    else if (max_sweeps > 0 && sweeps >= max_sweeps) status = 2;
  }
  if (out) {
    out[0] = sweeps;
    out[1] = execs;
    out[2] = e.narrowed;
    out[3] = any_changed;
  }
  return status;
}

int32_t orc_pc_fixpoint_jacobi(int32_t nnodes, const int32_t *k, const int32_t *a, const int32_t *b,
                               const int32_t *c, int32_t nprops, const int32_t *roots, int32_t nvars,
                               int32_t *store, int64_t max_rounds, int64_t *out) {
  (void)nnodes;
  int64_t rounds = 0, narrowed = 0;
  int32_t status = store_has_bot(nvars, store) ? 1 : 0;
  std::vector<int32_t> next(store, store + 2 * (size_t)nvars);
  while (!status) {
    bool changed = false, failed = false;
    for (int32_t p = 0; p < nprops; ++p) {
      Eval e{k, a, b, c, store, 0, 0};
      e.w = next.data();
      e.deduce(roots[p]);
      changed |= e.narrowed != 0;
      failed |= e.failed != 0;
      narrowed += e.narrowed;
    }
    ++rounds;
    std::copy(next.begin(), next.end(), store);
    if (failed || store_has_bot(nvars, store)) status = 1;
    else if (!changed) break;
    else if (max_rounds > 0 && rounds >= max_rounds) status = 2;
  }
  if (out) {
    out[0] = rounds;
    out[1] = rounds * nprops;
    out[2] = narrowed;
    out[3] = 0;
  }
  return status;
}

void orc_pc_itv(int32_t op, int32_t al, int32_t au, int32_t bl, int32_t bu, int32_t *out_l, int32_t *out_u) {
  const I r = itv_op(op, I{al, au}, I{bl, bu});
  *out_l = r.l;
  *out_u = r.u;
}

}  // extern "C"
