// PC tree propagators on sm_103a: lala-pc's PC abstract domain
// (include/lala/pc.hpp) with the terms of terms.hpp and the formulas of
// formula.hpp, over the context's HBM store.
//
// Layout: the formulas of all propagators live in one tape of int4 nodes
// {kind, a, b, c} in HBM (children before parents, so a tape is acyclic by
// construction), read through the read-only path; the propagators are root
// indices sorted by (formula kind, tree length) as PC::deduce(tell) sorts them
// (pc.hpp:638-641), which also groups trees of one shape into the same warps.
//
// Execution: Jacobi rounds in one cooperative launch, a thread per propagator
// per step.  Every deduction of a round reads the store the round started
// from (A, never written during the round) and joins its narrowings into a
// second copy (B) with red.max / red.min; after a grid barrier B is copied
// back into A and checked for empty variables, and a second barrier starts
// the next round.  The result is therefore a deterministic function of the
// input, independent of thread timing.  PC's propagators are not monotone in
// general (Implication::contradeduce, formula.hpp:497-503, leaves an entailed
// implication alone when its premise is unknown, so a smaller store can be
// narrowed less), and for such sets even the reference's Gauss-Seidel result
// depends on the propagator order; for monotone sets every schedule reaches
// the same fixpoint.  A propagator is evaluated by a recursive descent that
// restates the reference's member functions one for one (project / embed of
// terms, ask / nask / deduce / contradeduce of formulas).  The recursion depth
// is the tree depth (at most PC_MAX_DEPTH); the per-thread call stack is
// sized from it before the launch.
//
// Interval arithmetic (lala-core's Interval<ZLB<int>>, not vendored in the
// reference) follows its mathematical meaning: exact images computed in int64
// on the extended integers (0 * inf = 0) and clamped to int32, division as the
// exact hull over the non-zero divisors, LB::prev(k) = k + 1,
// UB::prev(k) = k - 1.  Every operator is monotone for
// inclusion, so the fixpoint does not depend on the order of the propagators
// (NaryMul's early exit on a product of exactly [0, 0], terms.hpp:487, is the
// one exception, as in the reference).
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>
#include <vector>

#include "pir_csr.h"
#include "pir_engine.h"
#include "pir_sort.h"

namespace pirgpu {

struct PcState {
  std::vector<int4> tape;         // kind, a, b, c
  std::vector<long long> len;     // Formula::length / Term::length per node
  std::vector<int> depth;         // nodes on the longest path below a node
  std::vector<int> roots;         // engine order
  int max_var = -1;               // largest variable a node refers to
  int max_depth = 0;              // over the roots
  int4 *d_tape = nullptr;
  size_t cap_tape = 0;
  int *d_roots = nullptr;
  size_t cap_roots = 0;
  int2 *d_next = nullptr;         // the store's second copy (the joins of a Jacobi round)
  size_t cap_next = 0;
  std::vector<int> tree_base;     // per root node: first node of its tree, or -1 (recursive path)
  int *d_bases = nullptr;         // tree_base of each propagator, engine order
  size_t cap_bases = 0;
  std::vector<unsigned> stamp;    // scratch of the tree check
  unsigned stamp_gen = 0;
  size_t stack_bytes = 0;         // per-thread stack limit this context asked for
  // event schedule: variable -> formulas (engine indices), rebuilt after a
  // tell or a restore changed the propagators
  bool csr_valid = false;
  int csr_nvars = -1;             // store size the adjacency was built for
  int *d_adj_ptr = nullptr, *d_adj = nullptr, *d_list = nullptr;
  unsigned *d_pstamp = nullptr, *d_cnt = nullptr;
  size_t cap_adj_ptr = 0, cap_adj = 0, cap_list = 0, cap_pstamp = 0, cap_cnt = 0;
};

namespace {

constexpr int K_VAR = PC_VAR, K_CONST = PC_CONST, K_FORMULA = PC_FORMULA, K_NEG = PC_NEG, K_ABS = PC_ABS,
              K_ADD = PC_ADD, K_SUB = PC_SUB, K_MUL = PC_MUL, K_TDIV = PC_TDIV, K_FDIV = PC_FDIV,
              K_CDIV = PC_CDIV, K_EDIV = PC_EDIV, K_MIN = PC_MIN, K_MAX = PC_MAX, K_NADD = PC_NADD,
              K_NMUL = PC_NMUL, K_PVAR = PC_PVAR, K_NVAR = PC_NVAR, K_TRUE = PC_TRUE, K_FALSE = PC_FALSE,
              K_LEQ = PC_LEQ, K_GT = PC_GT, K_EQ = PC_EQ, K_NEQ = PC_NEQ, K_AND = PC_AND, K_OR = PC_OR,
              K_EQUIV = PC_EQUIV, K_IMPLY = PC_IMPLY, K_XOR = PC_XOR, K_ARG = PC_ARG, K_AE = PC_AE,
              K_TELL = PC_TELL, K_NTELL = PC_NTELL, K_ASK = PC_ASK, K_NASK = PC_NASK,
              K_ASK_OUT = PC_ASK_OUT, K_NASK_OUT = PC_NASK_OUT;

// ------------------------------------------------------ interval algebra --
__device__ __forceinline__ Itv itop() { return mk(MINF, INF); }
__device__ __forceinline__ Itv iempty() { return mk(INF, MINF); }
__device__ __forceinline__ Itv imeet(Itv a, Itv b) { return mk(max(a.l, b.l), min(a.u, b.u)); }
__device__ __forceinline__ Itv ifjoin(Itv a, Itv b) {
  if (is_bot(a)) return b;
  if (is_bot(b)) return a;
  return mk(min(a.l, b.l), max(a.u, b.u));
}
// a >= eq_zero(): 0 in a
__device__ __forceinline__ bool has0(Itv a) { return !is_bot(a) && a.l <= 0 && a.u >= 0; }
// a <= [v, v]: a is [v, v] or empty
__device__ __forceinline__ bool below_point(Itv a, int v) { return is_bot(a) || (a.l == v && a.u == v); }
__device__ __forceinline__ bool is_point(Itv a, int v) { return a.l == v && a.u == v; }
__device__ __forceinline__ int prev_lb(int k) { return (k == MINF || k == INF) ? k : k + 1; }
__device__ __forceinline__ int prev_ub(int k) { return (k == MINF || k == INF) ? k : k - 1; }
__device__ __forceinline__ int neg_of_ub(int u) { return u == INF ? MINF : cl(-(long long)u); }
__device__ __forceinline__ int neg_of_lb(int l) { return l == MINF ? INF : cl(-(long long)l); }

__device__ __forceinline__ Itv ineg(Itv a) { return is_bot(a) ? iempty() : mk(neg_of_ub(a.u), neg_of_lb(a.l)); }
__device__ __forceinline__ Itv iadd(Itv a, Itv b) {
  if (is_bot(a) || is_bot(b)) return iempty();
  return mk((a.l == MINF || b.l == MINF) ? MINF : cl((long long)a.l + b.l),
            (a.u == INF || b.u == INF) ? INF : cl((long long)a.u + b.u));
}
__device__ __forceinline__ Itv isub(Itv a, Itv b) { return iadd(a, ineg(b)); }
__device__ __forceinline__ Itv imin2(Itv a, Itv b) {
  return (is_bot(a) || is_bot(b)) ? iempty() : mk(min(a.l, b.l), min(a.u, b.u));
}
__device__ __forceinline__ Itv imax2(Itv a, Itv b) {
  return (is_bot(a) || is_bot(b)) ? iempty() : mk(max(a.l, b.l), max(a.u, b.u));
}
__device__ __forceinline__ Itv iabs(Itv a) {
  if (is_bot(a)) return iempty();
  if (a.l >= 0) return a;
  if (a.u <= 0) return ineg(a);
  return mk(0, max(neg_of_lb(a.l), a.u));
}

// Products on the extended integers: a bound is -inf (lb = MINF), +inf
// (ub = INF) or finite; 0 * inf = 0.  Encoded as int64 with +-2^62 for the
// infinities (finite products stay below 2^62 in magnitude).
constexpr long long XINF = 1ll << 62;
__device__ __forceinline__ long long xl(int l) { return l == MINF ? -XINF : (long long)l; }
__device__ __forceinline__ long long xu(int u) { return u == INF ? XINF : (long long)u; }
__device__ __forceinline__ long long xmul(long long p, long long q) {
  if (p == 0 || q == 0) return 0;
  if (p == XINF || p == -XINF || q == XINF || q == -XINF) return ((p < 0) != (q < 0)) ? -XINF : XINF;
  return p * q;
}
__device__ __forceinline__ Itv imul(Itv a, Itv b) {
  if (is_bot(a) || is_bot(b)) return iempty();
  if (b.l == b.u && b.l != MINF && b.l != INF) {  // a singleton factor: two corners suffice
    const Itv t = a;
    a = b;
    b = t;
  }
  if (a.l == a.u && a.l != MINF && a.l != INF) {
    const long long p0 = xmul(a.l, xl(b.l)), p1 = xmul(a.l, xu(b.u));
    const long long lo = mn(p0, p1), hi = mx(p0, p1);
    return mk(lo == -XINF ? MINF : cl(lo), hi == XINF ? INF : cl(hi));
  }
  const long long p0 = xmul(xl(a.l), xl(b.l)), p1 = xmul(xl(a.l), xu(b.u));
  const long long p2 = xmul(xu(a.u), xl(b.l)), p3 = xmul(xu(a.u), xu(b.u));
  const long long lo = mn(mn(p0, p1), mn(p2, p3)), hi = mx(mx(p0, p1), mx(p2, p3));
  return mk(lo == -XINF ? MINF : cl(lo), hi == XINF ? INF : cl(hi));
}

__device__ __forceinline__ int div_op(int kind) {
  return kind == K_TDIV ? OP_TDIV : (kind == K_FDIV ? OP_FDIV : (kind == K_CDIV ? OP_CDIV : OP_EDIV));
}
// y / z on the extended integers (XINF encoding), z != 0: inf / z is
// +-inf; y / inf is the rounded value of a vanishing quotient (0, or -1 / +1
// on the floor / ceiling side); inf / inf counts as a large y over a larger z
__device__ __forceinline__ long long xquo(int op, long long y, long long z) {
  const bool yi = y == XINF || y == -XINF, zi = z == XINF || z == -XINF;
  if (!zi) {
    if (!yi) return d_div(op, y, z);
    return ((y < 0) != (z < 0)) ? -XINF : XINF;
  }
  const int sy = (y > 0) - (y < 0), s = sy * (z > 0 ? 1 : -1);
  switch (op) {
    case OP_TDIV: return 0;
    case OP_FDIV: return s < 0 ? -1 : 0;
    case OP_CDIV: return s > 0 ? 1 : 0;
    default: return z > 0 ? (sy < 0 ? -1 : 0) : (sy < 0 ? 1 : 0);  // floor for z > 0, ceiling for z < 0
  }
}
// Exact hull of { y op z : y in a, z in b, z != 0 }: the quotient is monotone
// in each argument on a sign-definite divisor range, so the corners of b's
// negative and positive parts bound it.
static __device__ __noinline__ Itv idiv_hull(int op, Itv a, Itv b) {
  if (is_bot(a) || is_bot(b) || is_point(b, 0)) return iempty();
  const long long yl = xl(a.l), yu = xu(a.u);
  long long lo = LLONG_MAX, hi = LLONG_MIN;
  if (b.l <= -1) {
    const long long zl = xl(b.l), zu = min(b.u, -1);
    const long long q0 = xquo(op, yl, zl), q1 = xquo(op, yl, zu), q2 = xquo(op, yu, zl), q3 = xquo(op, yu, zu);
    lo = mn(lo, mn(mn(q0, q1), mn(q2, q3)));
    hi = mx(hi, mx(mx(q0, q1), mx(q2, q3)));
  }
  if (b.u >= 1) {
    const long long zl = max(b.l, 1), zu = xu(b.u);
    const long long q0 = xquo(op, yl, zl), q1 = xquo(op, yl, zu), q2 = xquo(op, yu, zl), q3 = xquo(op, yu, zu);
    lo = mn(lo, mn(mn(q0, q1), mn(q2, q3)));
    hi = mx(hi, mx(mx(q0, q1), mx(q2, q3)));
  }
  return mk(lo <= -XINF ? MINF : cl(lo), hi >= XINF ? INF : cl(hi));
}
// A singleton divisor c (the coefficient of a linear term): the quotient is
// monotone in the dividend, so the two dividend bounds give the hull -- the
// same values idiv_hull computes at its corners.
__device__ __forceinline__ Itv idiv(int op, Itv a, Itv b) {
  if (b.l == b.u && b.l != 0 && b.l != MINF && b.l != INF && !is_bot(a)) {
    const long long c = b.l;
    const long long ql = a.l == MINF ? (c > 0 ? -XINF : XINF) : d_div(op, a.l, c);
    const long long qu = a.u == INF ? (c > 0 ? XINF : -XINF) : d_div(op, a.u, c);
    const long long lo = mn(ql, qu), hi = mx(ql, qu);
    return mk(lo <= -XINF ? MINF : cl(lo), hi >= XINF ? INF : cl(hi));
  }
  return idiv_hull(op, a, b);
}
// GroupAdd::rev_op (terms.hpp:190-194): all + additive_inverse(t), the
// inverse negating each bound without swapping them, so that the result is
// the sum of the other operands
__device__ __forceinline__ Itv rev_add(Itv all, Itv t) {
  if (is_bot(all) || is_bot(t)) return iempty();
  return mk((all.l == MINF || t.l == MINF) ? MINF : cl((long long)all.l - t.l),
            (all.u == INF || t.u == INF) ? INF : cl((long long)all.u - t.u));
}

__device__ __forceinline__ Itv ibinary(int kind, Itv a, Itv b) {
  switch (kind) {
    case K_ADD: return iadd(a, b);
    case K_SUB: return isub(a, b);
    case K_MUL: return imul(a, b);
    case K_MIN: return imin2(a, b);
    case K_MAX: return imax2(a, b);
    default: return idiv(div_op(kind), a, b);
  }
}

// ------------------------------------------------------------- evaluator --
// Per-thread evaluation state (a local variable of the kernel; the recursive
// functions get its address).  Reads come from `rd`, joins go to `wr`: in a
// Jacobi round rd is the round's initial store and wr its copy; for a single
// deduce(i) both are the store.
struct PcEval {
  const int4 *tape;
  const int2 *rd;
  int2 *wr;
  int failed;          // this deduction emptied a variable (VStore's bot flag)
  unsigned narrowed;   // bounds moved
};

__device__ __forceinline__ int4 node(const PcEval *e, int n) { return __ldg(e->tape + n); }
__device__ __forceinline__ Itv load(const PcEval *e, int v) {
  const int2 t = __ldcg(e->rd + v);
  return mk(t.x, t.y);
}
// VStore::embed: meet u into variable v; true iff a bound moved
__device__ __forceinline__ bool store_embed(PcEval *e, int v, Itv u) {
  const Itv cur = load(e, v);
  bool ch = false;
  if (u.l > cur.l) {
    asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&e->wr[v].x), "r"(u.l) : "memory");
    ch = true;
    ++e->narrowed;
  }
  if (u.u < cur.u) {
    asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&e->wr[v].y), "r"(u.u) : "memory");
    ch = true;
    ++e->narrowed;
  }
  if (ch && is_bot(imeet(cur, u))) e->failed = 1;
  return ch;
}

// The recursive functions take the node already loaded; the inline wrappers
// below answer leaves (variables, constants, literals) in the caller, so a
// call, and its stack frame, is spent on inner nodes only.
__device__ Itv t_project_rec(PcEval *e, int n, int4 d);
__device__ bool t_embed_rec(PcEval *e, int n, int4 d, Itv u);
__device__ bool f_ask_rec(PcEval *e, int4 d);
__device__ bool f_nask_rec(PcEval *e, int4 d);
__device__ bool f_deduce_rec(PcEval *e, int4 d);
__device__ bool f_contra_rec(PcEval *e, int4 d);

__device__ __forceinline__ Itv t_project(PcEval *e, int n) {
  const int4 d = node(e, n);
  if (d.x == K_VAR) return load(e, d.y);
  if (d.x == K_CONST) return mk(d.y, d.z);
  return t_project_rec(e, n, d);
}
__device__ __forceinline__ bool t_embed(PcEval *e, int n, Itv u) {
  const int4 d = node(e, n);
  if (d.x == K_VAR) return store_embed(e, d.y, u);
  if (d.x == K_CONST) return false;
  return t_embed_rec(e, n, d, u);
}
__device__ __forceinline__ bool f_ask(PcEval *e, int n) {
  const int4 d = node(e, n);
  if (d.x == K_PVAR) return !has0(load(e, d.y));
  if (d.x == K_NVAR) return below_point(load(e, d.y), 0);
  return f_ask_rec(e, d);
}
__device__ __forceinline__ bool f_nask(PcEval *e, int n) {
  const int4 d = node(e, n);
  if (d.x == K_PVAR) return below_point(load(e, d.y), 0);
  if (d.x == K_NVAR) return !has0(load(e, d.y));
  return f_nask_rec(e, d);
}
__device__ __forceinline__ bool f_deduce(PcEval *e, int n) {
  const int4 d = node(e, n);
  if (d.x == K_PVAR) return store_embed(e, d.y, mk(1, 1));
  if (d.x == K_NVAR) return store_embed(e, d.y, mk(0, 0));
  return f_deduce_rec(e, d);
}
__device__ __forceinline__ bool f_contra(PcEval *e, int n) {
  const int4 d = node(e, n);
  if (d.x == K_PVAR) return store_embed(e, d.y, mk(0, 0));
  if (d.x == K_NVAR) return store_embed(e, d.y, mk(1, 1));
  return f_contra_rec(e, d);
}

// Formula::project (formula.hpp:1097-1102): the truth value in {0, 1}
static __device__ __noinline__ Itv f_project(PcEval *e, int n) {
  if (e->failed) return iempty();
  Itv r = mk(0, 1);
  if (f_ask(e, n)) r = imeet(r, mk(1, 1));
  if (f_nask(e, n)) r = imeet(r, mk(0, 0));
  return r;
}

// Term::project (terms.hpp:741): Variable :69, Constant :35, Unary :155,
// Binary :399, Nary :465
__device__ __noinline__ Itv t_project_rec(PcEval *e, int n, int4 d) {
  switch (d.x) {
    case K_VAR: return load(e, d.y);
    case K_CONST: return mk(d.y, d.z);
    case K_FORMULA: return f_project(e, d.y);
    case K_NEG: return ineg(t_project(e, d.y));
    case K_ABS: return iabs(t_project(e, d.y));
    case K_NADD:
    case K_NMUL: {
      Itv acc = t_project(e, node(e, d.y).y);
      for (int i = 1; i < d.z; ++i) {
        const Itv t = t_project(e, node(e, d.y + i).y);
        acc = d.x == K_NADD ? iadd(acc, t) : imul(acc, t);
      }
      return acc;
    }
    default: {
      const Itv x = t_project(e, d.y);
      return ibinary(d.x, x, t_project(e, d.z));
    }
  }
}

// Group*::left_residual (terms.hpp:196-324): x of `x op y = u`
__device__ __forceinline__ Itv left_residual(int kind, Itv u, Itv y) {
  switch (kind) {
    case K_ADD: return isub(u, y);
    case K_SUB: return iadd(u, y);
    case K_MUL: return (has0(u) && has0(y)) ? itop() : idiv(OP_EDIV, u, y);
    case K_MIN:
    case K_MAX:
      if (is_bot(imeet(u, y))) return u;
      return kind == K_MIN ? mk(u.l, INF) : mk(MINF, u.u);
    default: {  // GroupDiv :272-277
      Itv r = imul(u, y);
      r.u = max(r.u, prev_ub(y.u));
      return r;
    }
  }
}
// Group*::right_residual: y of `x op y = u`; r is y's interval for a division
__device__ __forceinline__ Itv right_residual(int kind, Itv u, Itv x, Itv r) {
  switch (kind) {
    case K_SUB: return isub(x, u);
    case K_ADD:
    case K_MUL:
    case K_MIN:
    case K_MAX: return left_residual(kind, u, x);
    default:  // GroupDiv :279-299
      if (r.l == 0) r.l = max(r.l, 1);
      if (r.u == 0) r.u = min(r.u, -1);
      if (!has0(x) && !is_point(u, 0)) r = imeet(r, idiv(div_op(kind), x, u));
      return r;
  }
}

// Formula::embed (formula.hpp:1090-1095)
static __device__ __noinline__ bool f_embed(PcEval *e, int n, Itv u) {
  if (below_point(u, 1)) return f_deduce(e, n);
  if (below_point(u, 0)) return f_contra(e, n);
  return false;
}

// Term::embed (terms.hpp:737): Variable :65, Constant :34, Unary :149,
// Binary :376, Nary :480
__device__ __noinline__ bool t_embed_rec(PcEval *e, int n, int4 d, Itv u) {
  switch (d.x) {
    case K_VAR: return store_embed(e, d.y, u);
    case K_CONST: return false;
    case K_FORMULA: return f_embed(e, d.y, u);
    case K_NEG: return t_embed(e, d.y, ineg(u));
    case K_ABS: return t_embed(e, d.y, ifjoin(u, ineg(u)));
    case K_NADD:
    case K_NMUL: {
      const Itv all = t_project(e, n);
      if (d.x == K_NMUL && is_point(all, 0)) return false;  // GroupMul::is_absorbing
      bool ch = false;
      for (int i = 0; i < d.z; ++i) {
        const int t = node(e, d.y + i).y;
        const Itv tmp = t_project(e, t);
        Itv res;
        if (d.x == K_NADD) res = isub(u, rev_add(all, tmp));  // GroupAdd rev_op / left_residual
        else res = left_residual(K_MUL, u, idiv(OP_EDIV, all, tmp));
        ch |= t_embed(e, t, res);
      }
      return ch;
    }
    default: {
      const int x = d.y, y = d.z;
      bool ch = false;
      if (node(e, x).x != K_CONST) ch |= t_embed(e, x, left_residual(d.x, u, t_project(e, y)));
      if (node(e, y).x != K_CONST) {
        const Itv xt = t_project(e, x);
        const Itv r = (d.x >= K_TDIV && d.x <= K_EDIV) ? t_project(e, y) : itop();
        ch |= t_embed(e, y, right_residual(d.x, u, xt, r));
      }
      return ch;
    }
  }
}

// Comparisons: Equality (formula.hpp:620-684), Inequality (:758-818)
static __device__ __noinline__ bool cmp_ask(PcEval *e, int kind, int L, int R) {
  const Itv l = t_project(e, L), r = t_project(e, R);
  switch (kind) {
    case K_EQ: return l.l == r.l && l.u == r.u && l.l == l.u;
    case K_NEQ: return is_bot(imeet(l, r));
    case K_LEQ: return l.u <= r.l;
    default: return l.l > r.u;
  }
}
__device__ __forceinline__ int negated(int kind) {
  return kind == K_EQ ? K_NEQ : (kind == K_NEQ ? K_EQ : (kind == K_LEQ ? K_GT : K_LEQ));
}
static __device__ __noinline__ bool cmp_deduce(PcEval *e, int kind, int L, int R) {
  const bool lc = node(e, L).x == K_CONST, rc = node(e, R).x == K_CONST;
  bool ch = false;
  switch (kind) {
    case K_EQ:
      if (!rc) ch = t_embed(e, R, t_project(e, L));
      if (!lc) ch |= t_embed(e, L, t_project(e, R));
      return ch;
    case K_NEQ:
      if (!rc) {
        const Itv l = t_project(e, L);
        if (l.l == l.u) {
          const Itv r = t_project(e, R);
          return t_embed(e, R, ifjoin(mk(max(r.l, prev_lb(l.l)), r.u), mk(r.l, min(r.u, prev_ub(l.u)))));
        }
      }
      if (!lc) {
        const Itv r = t_project(e, R);
        if (r.l == r.u) {
          const Itv l = t_project(e, L);
          return t_embed(e, L, ifjoin(mk(max(l.l, prev_lb(r.l)), l.u), mk(l.l, min(l.u, prev_ub(r.u)))));
        }
      }
      return false;
    case K_LEQ:
      if (!lc) ch |= t_embed(e, L, mk(MINF, t_project(e, R).u));
      if (!rc) ch = t_embed(e, R, mk(t_project(e, L).l, INF));  // '=' as in the reference (:815)
      return ch;
    default: {  // GT
      if (!lc) {
        const Itv r = t_project(e, R);
        ch = t_embed(e, L, mk(max(r.l, prev_lb(r.l)), INF));
      }
      if (!rc) {
        const Itv l = t_project(e, L);
        ch |= t_embed(e, R, mk(MINF, min(l.u, prev_ub(l.u))));
      }
      return ch;
    }
  }
}

// AbstractElement (formula.hpp:14-78): a formula of the store itself.  Its
// ask is the store's (every item's variable inside the item's interval), its
// deduce the store's tell (meet every item); nask / contradeduce use the
// negation's items.
// item: K_ASK or K_NASK; the _OUT items of the same list ask that the
// variable misses the interval (an ask of var != c)
static __device__ __noinline__ bool ae_ask(PcEval *e, int4 d, int item) {
  const int out = item + 2;
  for (int i = d.y; i < d.y + d.z; ++i) {
    const int4 t = node(e, i);
    if (t.x != item && t.x != out) continue;
    const Itv x = load(e, t.y);
    if (is_bot(x)) continue;
    if (t.x == item ? !(x.l >= t.z && x.u <= t.w) : !is_bot(imeet(x, mk(t.z, t.w)))) return false;
  }
  return true;
}
static __device__ __noinline__ bool ae_tell(PcEval *e, int4 d, int item) {
  bool ch = false;
  for (int i = d.y; i < d.y + d.z; ++i) {
    const int4 t = node(e, i);
    if (t.x == item) ch |= store_embed(e, t.y, mk(t.z, t.w));
  }
  return ch;
}

// ask / nask / deduce / contradeduce of every Formula alternative:
// VariableLiteral :101-160, False :184-195, True :220-230, Conjunction
// :268-288, Disjunction :338-358, Biconditional :408-438, Implication
// :482-503, ExclusiveDisjunction :546-574
__device__ __noinline__ bool f_ask_rec(PcEval *e, int4 d) {
  switch (d.x) {
    case K_AE: return ae_ask(e, d, K_ASK);
    case K_PVAR: return !has0(load(e, d.y));
    case K_NVAR: return below_point(load(e, d.y), 0);
    case K_TRUE: return true;
    case K_FALSE: return e->failed != 0;
    case K_AND: return f_ask(e, d.y) && f_ask(e, d.z);
    case K_OR: return f_ask(e, d.y) || f_ask(e, d.z);
    case K_EQUIV: return (f_ask(e, d.y) && f_ask(e, d.z)) || (f_nask(e, d.y) && f_nask(e, d.z));
    case K_IMPLY: return f_nask(e, d.y) || f_ask(e, d.z);
    case K_XOR: return (f_ask(e, d.y) && f_nask(e, d.z)) || (f_nask(e, d.y) && f_ask(e, d.z));
    default: return cmp_ask(e, d.x, d.y, d.z);
  }
}
__device__ __noinline__ bool f_nask_rec(PcEval *e, int4 d) {
  switch (d.x) {
    case K_AE: return ae_ask(e, d, K_NASK);
    case K_PVAR: return below_point(load(e, d.y), 0);
    case K_NVAR: return !has0(load(e, d.y));
    case K_TRUE: return e->failed != 0;
    case K_FALSE: return true;
    case K_AND: return f_nask(e, d.y) || f_nask(e, d.z);
    case K_OR: return f_nask(e, d.y) && f_nask(e, d.z);
    case K_EQUIV: return (f_ask(e, d.y) && f_nask(e, d.z)) || (f_nask(e, d.y) && f_ask(e, d.z));
    case K_IMPLY: return f_ask(e, d.y) && f_nask(e, d.z);
    case K_XOR: return (f_ask(e, d.y) && f_ask(e, d.z)) || (f_ask(e, d.y) && f_nask(e, d.z));  // as written (:552-556)
    default: return cmp_ask(e, negated(d.x), d.y, d.z);
  }
}
__device__ __noinline__ bool f_deduce_rec(PcEval *e, int4 d) {
  const int f = d.y, g = d.z;
  switch (d.x) {
    case K_AE: return ae_tell(e, d, K_TELL);
    case K_PVAR: return store_embed(e, d.y, mk(1, 1));
    case K_NVAR: return store_embed(e, d.y, mk(0, 0));
    case K_TRUE: return false;
    case K_FALSE:
      if (!e->failed) {
        e->failed = 1;
        return true;
      }
      return false;
    case K_AND: {
      bool ch = f_deduce(e, f);
      ch |= f_deduce(e, g);
      return ch;
    }
    case K_OR:
      if (f_nask(e, f)) return f_deduce(e, g);
      if (f_nask(e, g)) return f_deduce(e, f);
      return false;
    case K_EQUIV:
      if (f_ask(e, f)) return f_deduce(e, g);
      if (f_nask(e, f)) return f_contra(e, g);
      if (f_ask(e, g)) return f_deduce(e, f);
      if (f_nask(e, g)) return f_contra(e, f);
      return false;
    case K_IMPLY:
      if (f_ask(e, f)) return f_deduce(e, g);
      if (f_nask(e, g)) return f_contra(e, f);
      return false;
    case K_XOR:
      if (f_ask(e, f)) return f_contra(e, g);
      if (f_nask(e, f)) return f_deduce(e, g);
      if (f_ask(e, g)) return f_contra(e, f);
      if (f_nask(e, g)) return f_deduce(e, f);
      return false;
    default: return cmp_deduce(e, d.x, f, g);
  }
}
__device__ __noinline__ bool f_contra_rec(PcEval *e, int4 d) {
  const int f = d.y, g = d.z;
  switch (d.x) {
    case K_AE: return ae_tell(e, d, K_NTELL);
    case K_PVAR: return store_embed(e, d.y, mk(0, 0));
    case K_NVAR: return store_embed(e, d.y, mk(1, 1));
    case K_TRUE:
      if (!e->failed) {
        e->failed = 1;
        return true;
      }
      return false;
    case K_FALSE: return false;
    case K_AND:
      if (f_ask(e, f)) return f_contra(e, g);
      if (f_ask(e, g)) return f_contra(e, f);
      return false;
    case K_OR: {
      bool ch = f_contra(e, f);
      ch |= f_contra(e, g);
      return ch;
    }
    case K_EQUIV:
      if (f_ask(e, f)) return f_contra(e, g);
      if (f_nask(e, f)) return f_deduce(e, g);
      if (f_ask(e, g)) return f_contra(e, f);
      if (f_nask(e, g)) return f_deduce(e, f);
      return false;
    case K_IMPLY:
      if (f_ask(e, f)) return f_contra(e, g);
      if (f_nask(e, g)) return f_deduce(e, f);
      return false;
    case K_XOR:
      if (f_ask(e, f)) return f_deduce(e, g);
      if (f_nask(e, f)) return f_contra(e, g);
      if (f_ask(e, g)) return f_deduce(e, f);
      if (f_nask(e, g)) return f_contra(e, f);
      return false;
    default: return cmp_deduce(e, negated(d.x), f, g);
  }
}

// ---------------------------------------------------------------- kernels --
constexpr int PC_BLOCK = 128;

// ------------------------------------------- trees without the call stack --
// In a Jacobi round every read of a propagator sees the round's initial
// store, so what the recursive descent computes on the way down is a pure
// function of that store: every term's projection and every formula's ask /
// nask.  For a tree (each node reached once from the root) whose nodes are
// the contiguous tape range [base, root] (children before parents), both
// passes run without recursion over per-thread arrays in shared memory:
//   pass 1, base -> root: each node's interval, or its ask (bit 0) and nask
//     (bit 1), from its children's;
//   pass 2, root -> base: the requests the reference's member functions
//     would issue (deduce / contradeduce of a formula, embed of an interval
//     into a term), each node receiving at most one.
// The joins, and with them the round's result and its narrowing count, are
// those of the recursive descent.  (They can differ only after a deduction
// of the same propagator emptied a variable -- the recursive path then reads
// the store as bot in Formula::project -- and then the round fails either
// way.)  Other propagators take the recursive path.
constexpr int PC_TREE_MAX = 24;  // nodes per tree on this path
constexpr size_t PC_TREE_SMEM = (size_t)PC_TREE_MAX * PC_BLOCK * 3 * sizeof(int2);
enum : int { RQ_NONE = 0, RQ_DEDUCE = 1, RQ_CONTRA = 2, RQ_EMBED = 3 };

// ask / nask of a comparison from its operands' intervals (Equality :620,
// Inequality :758)
__device__ __forceinline__ bool cmp_holds(int kind, Itv l, Itv r) {
  switch (kind) {
    case K_EQ: return l.l == r.l && l.u == r.u && l.l == l.u;
    case K_NEQ: return is_bot(imeet(l, r));
    case K_LEQ: return l.u <= r.l;
    default: return l.l > r.u;
  }
}

// Per-thread slices of the node-major shared arrays: node j of this thread
// is element j * PC_BLOCK, so the threads of a warp touch consecutive words.
// The tree is staged first with independent loads -- its nodes, packed to 8
// bytes, then the store intervals of its variable leaves -- so that a tree
// costs two memory latencies instead of a chain of one per node.
//   node[j].x: kind | request << 5 | first operand << 8 | second operand (or
//              operand count) << 16, operands as indices into the tree;
//   node[j].y: the variable of a VAR / PVAR / NVAR leaf;
//   val[j]:    the node's interval (a CONST's value, a variable's interval,
//              a term's projection), or ask | nask << 1 of a formula;
//   req[j]:    the interval of an embed request, or the store interval of a
//              literal leaf.
struct TreeScratch {
  int2 *node, *val, *req;
  __device__ __forceinline__ Itv v(int j) const {
    const int2 t = val[j * PC_BLOCK];
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int bits(int j) const { return val[j * PC_BLOCK].x; }
  __device__ __forceinline__ void set(int j, Itv a) { val[j * PC_BLOCK] = make_int2(a.l, a.u); }
  __device__ __forceinline__ int word(int j) const { return node[j * PC_BLOCK].x; }
  __device__ __forceinline__ void send(int j, int k) { node[j * PC_BLOCK].x |= k << 5; }
  __device__ __forceinline__ void send(int j, Itv u) {
    node[j * PC_BLOCK].x |= RQ_EMBED << 5;
    req[j * PC_BLOCK] = make_int2(u.l, u.u);
  }
};

// VStore::embed with the variable's interval already read (cur)
__device__ __forceinline__ void join(PcEval *e, int v, Itv cur, Itv u) {
  bool ch = false;
  if (u.l > cur.l) {
    asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&e->wr[v].x), "r"(u.l) : "memory");
    ch = true;
    ++e->narrowed;
  }
  if (u.u < cur.u) {
    asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&e->wr[v].y), "r"(u.u) : "memory");
    ch = true;
    ++e->narrowed;
  }
  if (ch && is_bot(imeet(cur, u))) e->failed = 1;
}

__device__ __forceinline__ int pack_node(int4 d, int base) {
  const int k = d.x;
  if (k == K_VAR || k == K_PVAR || k == K_NVAR || k == K_CONST || k == K_TRUE || k == K_FALSE) return k;
  if (k == K_FORMULA || k == K_NEG || k == K_ABS || k == K_ARG) return k | (d.y - base) << 8;
  if (k == K_NADD || k == K_NMUL) return k | (d.y - base) << 8 | d.z << 16;
  return k | (d.y - base) << 8 | (d.z - base) << 16;
}

constexpr int STAGE = 8;  // loads in flight while a tree is staged

static __device__ __noinline__ void tree_deduce(PcEval *e, int root, int base, TreeScratch sc) {
  const int4 *tape = e->tape;
  const int n = root - base + 1;
  // stage the nodes, STAGE independent loads in flight at a time
  for (int j = 0; j < n; j += STAGE) {
    int4 t[STAGE];
#pragma unroll
    for (int k = 0; k < STAGE; ++k)
      if (j + k < n) t[k] = __ldg(tape + base + j + k);
#pragma unroll
    for (int k = 0; k < STAGE; ++k)
      if (j + k < n) {
        sc.node[(j + k) * PC_BLOCK] = make_int2(pack_node(t[k], base), t[k].y);
        if (t[k].x == K_CONST) sc.set(j + k, mk(t[k].y, t[k].z));
      }
  }
  // then the intervals of the variable leaves
  for (int j = 0; j < n; j += STAGE) {
    int2 v[STAGE];
    bool is_var[STAGE];
#pragma unroll
    for (int k = 0; k < STAGE; ++k) {
      is_var[k] = false;
      if (j + k < n) {
        const int2 w = sc.node[(j + k) * PC_BLOCK];
        const int kind = w.x & 31;
        is_var[k] = kind == K_VAR || kind == K_PVAR || kind == K_NVAR;
        if (is_var[k]) v[k] = __ldcg(e->rd + w.y);
      }
    }
#pragma unroll
    for (int k = 0; k < STAGE; ++k)
      if (is_var[k]) sc.val[(j + k) * PC_BLOCK] = v[k];
  }
  // pass 1: projections and entailments, children first
  for (int j = 0; j < n; ++j) {
    const int w = sc.word(j);
    const int kind = w & 31, a = (w >> 8) & 255, b = w >> 16;
    Itv r;
    switch (kind) {
      case K_VAR:
      case K_CONST: continue;  // staged
      case K_FORMULA: {
        const int f = sc.bits(a);
        r = mk(0, 1);
        if (f & 1) r = imeet(r, mk(1, 1));
        if (f & 2) r = imeet(r, mk(0, 0));
        break;
      }
      case K_NEG: r = ineg(sc.v(a)); break;
      case K_ABS: r = iabs(sc.v(a)); break;
      case K_ARG: r = sc.v(a); break;
      case K_NADD:
      case K_NMUL: {
        r = sc.v(a);
        for (int i = 1; i < b; ++i) r = kind == K_NADD ? iadd(r, sc.v(a + i)) : imul(r, sc.v(a + i));
        break;
      }
      case K_PVAR:
      case K_NVAR: {
        const Itv x = sc.v(j);
        sc.req[j * PC_BLOCK] = make_int2(x.l, x.u);  // keep the literal's interval for pass 2
        const int t = !has0(x), f = below_point(x, 0);
        r = mk(kind == K_PVAR ? (t | f << 1) : (f | t << 1), 0);
        break;
      }
      case K_TRUE: r = mk(1, 0); break;
      case K_FALSE: r = mk(2, 0); break;
      case K_LEQ:
      case K_GT:
      case K_EQ:
      case K_NEQ: {
        const Itv x = sc.v(a), y = sc.v(b);
        r = mk((int)cmp_holds(kind, x, y) | (int)cmp_holds(negated(kind), x, y) << 1, 0);
        break;
      }
      case K_AND:
      case K_OR:
      case K_EQUIV:
      case K_IMPLY:
      case K_XOR: {
        const int f = sc.bits(a), g = sc.bits(b);
        const bool af = f & 1, nf = f & 2, ag = g & 1, ng = g & 2;
        bool ask, nask;
        if (kind == K_AND) ask = af && ag, nask = nf || ng;
        else if (kind == K_OR) ask = af || ag, nask = nf && ng;
        else if (kind == K_EQUIV) ask = (af && ag) || (nf && ng), nask = (af && ng) || (nf && ag);
        else if (kind == K_IMPLY) ask = nf || ag, nask = af && ng;
        else ask = (af && ng) || (nf && ag), nask = (af && ag) || (af && ng);  // xor as written (:552-556)
        r = mk((int)ask | (int)nask << 1, 0);
        break;
      }
      default: r = ibinary(kind, sc.v(a), sc.v(b));
    }
    sc.set(j, r);
  }
  // pass 2: requests, parents first
  sc.send(n - 1, RQ_DEDUCE);
  for (int j = n - 1; j >= 0; --j) {
    const int w = sc.word(j);
    const int t = (w >> 5) & 3;
    if (t == RQ_NONE) continue;
    const int kind = w & 31, a = (w >> 8) & 255, b = w >> 16;
    if (t == RQ_EMBED) {
      const int2 uu = sc.req[j * PC_BLOCK];
      const Itv u = mk(uu.x, uu.y);
      switch (kind) {
        case K_VAR: join(e, sc.node[j * PC_BLOCK].y, sc.v(j), u); break;
        case K_CONST: break;
        case K_FORMULA:
          if (below_point(u, 1)) sc.send(a, RQ_DEDUCE);
          else if (below_point(u, 0)) sc.send(a, RQ_CONTRA);
          break;
        case K_NEG: sc.send(a, ineg(u)); break;
        case K_ABS: sc.send(a, ifjoin(u, ineg(u))); break;
        case K_NADD:
        case K_NMUL: {
          const Itv all = sc.v(j);
          if (kind == K_NMUL && is_point(all, 0)) break;
          for (int i = 0; i < b; ++i) {
            const int c = (sc.word(a + i) >> 8) & 255;  // the operand behind slot a + i
            const Itv tmp = sc.v(c);
            sc.send(c, kind == K_NADD ? isub(u, rev_add(all, tmp)) : left_residual(K_MUL, u, idiv(OP_EDIV, all, tmp)));
          }
          break;
        }
        default: {  // binary term
          const Itv xv = sc.v(a), yv = sc.v(b);
          if ((sc.word(a) & 31) != K_CONST) sc.send(a, left_residual(kind, u, yv));
          if ((sc.word(b) & 31) != K_CONST)
            sc.send(b, right_residual(kind, u, xv, (kind >= K_TDIV && kind <= K_EDIV) ? yv : itop()));
        }
      }
      continue;
    }
    const bool c = t == RQ_CONTRA;
    switch (kind) {
      case K_PVAR:
      case K_NVAR: {
        const int2 x = sc.req[j * PC_BLOCK];
        const bool one = (kind == K_PVAR) != c;
        join(e, sc.node[j * PC_BLOCK].y, mk(x.x, x.y), one ? mk(1, 1) : mk(0, 0));
        break;
      }
      case K_TRUE:
        if (c) e->failed = 1;
        break;
      case K_FALSE:
        if (!c) e->failed = 1;
        break;
      case K_LEQ:
      case K_GT:
      case K_EQ:
      case K_NEQ: {
        const int k = c ? negated(kind) : kind;
        const bool lc = (sc.word(a) & 31) == K_CONST, rc = (sc.word(b) & 31) == K_CONST;
        const Itv l = sc.v(a), r = sc.v(b);
        if (k == K_EQ) {
          if (!rc) sc.send(b, l);
          if (!lc) sc.send(a, r);
        } else if (k == K_NEQ) {
          if (!rc && l.l == l.u) sc.send(b, ifjoin(mk(max(r.l, prev_lb(l.l)), r.u), mk(r.l, min(r.u, prev_ub(l.u)))));
          else if (!lc && r.l == r.u)
            sc.send(a, ifjoin(mk(max(l.l, prev_lb(r.l)), l.u), mk(l.l, min(l.u, prev_ub(r.u)))));
        } else if (k == K_LEQ) {
          if (!lc) sc.send(a, mk(MINF, r.u));
          if (!rc) sc.send(b, mk(l.l, INF));
        } else {  // GT
          if (!lc) sc.send(a, mk(max(r.l, prev_lb(r.l)), INF));
          if (!rc) sc.send(b, mk(MINF, min(l.u, prev_ub(l.u))));
        }
        break;
      }
      default: {  // connectives
        const int f = sc.bits(a), g = sc.bits(b);
        const bool af = f & 1, nf = f & 2, ag = g & 1, ng = g & 2;
        switch (kind) {
          case K_AND:
            if (!c) {
              sc.send(a, RQ_DEDUCE);
              sc.send(b, RQ_DEDUCE);
            } else if (af) sc.send(b, RQ_CONTRA);
            else if (ag) sc.send(a, RQ_CONTRA);
            break;
          case K_OR:
            if (c) {
              sc.send(a, RQ_CONTRA);
              sc.send(b, RQ_CONTRA);
            } else if (nf) sc.send(b, RQ_DEDUCE);
            else if (ng) sc.send(a, RQ_DEDUCE);
            break;
          case K_EQUIV:
            if (af) sc.send(b, c ? RQ_CONTRA : RQ_DEDUCE);
            else if (nf) sc.send(b, c ? RQ_DEDUCE : RQ_CONTRA);
            else if (ag) sc.send(a, c ? RQ_CONTRA : RQ_DEDUCE);
            else if (ng) sc.send(a, c ? RQ_DEDUCE : RQ_CONTRA);
            break;
          case K_IMPLY:
            if (af) sc.send(b, c ? RQ_CONTRA : RQ_DEDUCE);
            else if (ng) sc.send(a, c ? RQ_DEDUCE : RQ_CONTRA);
            break;
          default:  // XOR
            if (af) sc.send(b, c ? RQ_DEDUCE : RQ_CONTRA);
            else if (nf) sc.send(b, c ? RQ_CONTRA : RQ_DEDUCE);
            else if (ag) sc.send(a, c ? RQ_DEDUCE : RQ_CONTRA);
            else if (ng) sc.send(a, c ? RQ_CONTRA : RQ_DEDUCE);
        }
      }
    }
  }
}

// Persistent fixpoint over the PC propagators in Jacobi rounds: a round runs
// every propagator once on store A (a), joining into B (b, equal to A when
// the round starts); the round's changed / failed bits meet at the first
// grid barrier; then B is copied into A (two variables per 16-byte access),
// empty variables are counted, and the second barrier ends the round.
// Event schedule of the Jacobi rounds: a round runs only the formulas whose
// variables the previous round narrowed.  A formula's deduction is a pure
// function of its variables' intervals, so one whose variables did not change
// since it last ran would produce the joins it produced then, which are
// already in the store: the rounds, the stores and the result are those of
// the full rounds.  adj_ptr / adj: variable -> formulas (engine indices,
// CSR); stamp: per formula the last round it was listed for; list / cnt: the
// frontier of the next round (two buffers); execs: executions counted.
struct PcEvents {
  const int *adj_ptr, *adj;
  unsigned *stamp;
  int *list0, *list1;
  unsigned *cnt;  // cnt[2]
};
constexpr int PC_EXPAND = 8;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Lists the formulas of variable v for round `next` (each once: the stamp),
// eight adjacency entries per step, one atomic per step and warp.
__device__ __forceinline__ void pc_schedule(const PcEvents &ev, int v, unsigned next) {
  int *list = (next & 1u) ? ev.list1 : ev.list0;
  unsigned *cnt = ev.cnt + (next & 1u);
  const int beg = __ldg(ev.adj_ptr + v), end = __ldg(ev.adj_ptr + v + 1);
  for (int k0 = beg; k0 < end; k0 += PC_EXPAND) {
    int q[PC_EXPAND];
    unsigned take = 0;
#pragma unroll
    for (int j = 0; j < PC_EXPAND; ++j) {
      q[j] = k0 + j < end ? __ldg(ev.adj + k0 + j) : -1;
      if (q[j] >= 0 && atomicMax(ev.stamp + q[j], next) < next) take |= 1u << j;
    }
    const unsigned m = __activemask();
    unsigned before = 0, total = 0, bal[PC_EXPAND];
#pragma unroll
    for (int j = 0; j < PC_EXPAND; ++j) {
      bal[j] = __ballot_sync(m, (take >> j) & 1u);
      total += __popc(bal[j]);
    }
    const int leader = __ffs(m) - 1, lane = threadIdx.x & 31;
    unsigned slot = 0;
    if (lane == leader && total) slot = atomicAdd(cnt, total);
    slot = __shfl_sync(m, slot, leader);
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < PC_EXPAND; ++j) {
      if ((take >> j) & 1u) list[slot + before + __popc(bal[j] & lt)] = q[j];
      before += __popc(bal[j]);
    }
  }
}

template <bool EVENTS>
__global__ void __launch_bounds__(PC_BLOCK) k_pc_fixpoint(const int4 *tape, const int *roots, const int *bases,
                                                         int nprops, int2 *a, int2 *b, int nvars, Control *ctl,
                                                         long long max_rounds, long long timeout_ns,
                                                         PcEvents ev) {
  __shared__ unsigned s_bits[2], s_word[2];
  extern __shared__ __align__(16) unsigned char pc_smem[];
  TreeScratch sc;
  int2 *s0 = reinterpret_cast<int2 *>(pc_smem);
  sc.node = s0 + threadIdx.x;
  sc.val = s0 + PC_TREE_MAX * PC_BLOCK + threadIdx.x;
  sc.req = s0 + 2 * PC_TREE_MAX * PC_BLOCK + threadIdx.x;
  PcEval e;
  e.tape = tape;
  e.rd = a;
  e.wr = b;
  e.narrowed = 0;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
  long long round = 0, bar = 0;
  unsigned long long narrowed = 0;
  if (threadIdx.x == 0) s_bits[0] = s_bits[1] = 0u;
  __syncthreads();
  // one grid barrier with an OR of (changed, failed); returns the barrier word
  auto sync = [&](unsigned mine) {
    const int p = (int)(bar & 1);
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, mine);
    if ((threadIdx.x & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned v = s_bits[p];
      s_bits[p ^ 1] = 0u;
      s_word[p] = grid_sync_rot(ctl, gridDim.x, bar, v & 1u, v & 2u, timeout_ns);
    }
    __syncthreads();
    const unsigned w = s_word[p];
    ++bar;
    return w;
  };
  constexpr bool events = EVENTS;
  unsigned long long execs = 0;
  for (;;) {
    int failed = 0;
    e.narrowed = 0;
    // this round's formulas: all of them, or the frontier the previous round listed
    const int count = (!events || round == 0) ? nprops : (int)*(volatile unsigned *)(ev.cnt + (round & 1));
    const int *frontier = (round & 1) ? ev.list1 : ev.list0;
    if (events && blockIdx.x == 0 && threadIdx.x == 0) ev.cnt[(round + 1) & 1] = 0u;  // the next frontier
    execs += count;
    for (int k = gtid; k < count; k += gstride) {
      const int i = (!events || round == 0) ? k : __ldcg(frontier + k);
      e.failed = 0;
      const int base = __ldg(bases + i);
      if (base >= 0) tree_deduce(&e, __ldg(roots + i), base, sc);
      else f_deduce(&e, __ldg(roots + i));
      failed |= e.failed;
    }
    narrowed += e.narrowed;
    unsigned w = sync((e.narrowed ? 1u : 0u) | (failed ? 2u : 0u));
    ++round;
    bool stop = (w & BIT_ERROR) || (w & BIT_FAILED) || !(w & BIT_CHANGED);
    if (!stop) {
      // A := B and a count of empty variables; with events, only the changed
      // variables are copied and their formulas listed for the next round
      int empty = 0;
      if (events) {
        for (int v = gtid; v < nvars; v += gstride) {
          const int2 x = __ldcg(a + v), y = __ldcg(b + v);
          if (x.x != y.x || x.y != y.y) {
            a[v] = y;
            empty |= is_bot(mk(y.x, y.y));
            pc_schedule(ev, v, (unsigned)round);
          }
        }
      } else {
        const int npairs = nvars >> 1;
        const int4 *src = reinterpret_cast<const int4 *>(b);
        int4 *dst = reinterpret_cast<int4 *>(a);
        for (int i = gtid; i < npairs; i += gstride) {
          const int4 v = __ldcg(src + i);
          dst[i] = v;
          empty |= is_bot(mk(v.x, v.y)) | is_bot(mk(v.z, v.w));
        }
        if ((nvars & 1) && gtid == 0) {
          const int2 v = __ldcg(b + nvars - 1);
          a[nvars - 1] = v;
          empty |= is_bot(mk(v.x, v.y));
        }
      }
      const unsigned w2 = sync(empty ? 2u : 0u);
      if ((w2 & BIT_ERROR) || (w2 & BIT_FAILED)) {
        w = w2 | (w & BIT_CHANGED);
        stop = true;
      } else if (max_rounds > 0 && round >= max_rounds) {
        stop = true;
      }
    }
    if (stop) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->rounds = round;
        ctl->executions = execs;
        if (w & BIT_FAILED) ctl->failed = 1;
        if ((w & BIT_CHANGED) && !(w & (BIT_FAILED | BIT_ERROR))) ctl->changed[0] = 1;
      }
      break;
    }
  }
  const unsigned long long nar = warp_sum64(narrowed);
  if ((threadIdx.x & 31) == 0 && nar) atomicAdd(&ctl->narrowed, nar);
}

// deduce(int i) of one propagator, reading its own joins as the reference
// does: changed[0] = the reference's has_changed, changed[1] = a bound moved,
// failed = the store became bot.
__global__ void k_pc_deduce_one(const int4 *tape, int root, int2 *store, Control *ctl) {
  PcEval e;
  e.tape = tape;
  e.rd = store;
  e.wr = store;
  e.failed = 0;
  e.narrowed = 0;
  const bool ch = f_deduce(&e, root);
  ctl->changed[0] = ch ? 1 : 0;
  ctl->changed[1] = e.narrowed ? 1 : 0;
  ctl->narrowed = e.narrowed;
  if (e.failed) ctl->failed = 1;
}

__global__ void k_pc_ask_all(const int4 *tape, const int *roots, int nprops, int2 *store, int failed,
                             unsigned char *out) {
  PcEval e;
  e.tape = tape;
  e.rd = store;
  e.wr = store;
  e.failed = failed;
  e.narrowed = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nprops; i += gridDim.x * blockDim.x)
    out[i] = f_ask(&e, __ldg(roots + i)) ? 1 : 0;
}

// ------------------------------------------------------------------ host --
bool term_kind(int k) { return k >= K_VAR && k <= K_NMUL; }
bool formula_kind(int k) { return (k >= K_PVAR && k <= K_XOR) || k == K_AE; }
bool item_kind(int k) { return k >= K_TELL && k <= K_NASK_OUT; }

PcState *pc_state(pirgpu_ctx *ctx) {
  if (!ctx->pc) ctx->pc = new PcState();
  return ctx->pc;
}

// Per-thread call stack for trees of depth `depth`.  A call either goes one
// node down or stays on its node through a fixed chain (t_embed -> t_project
// on an n-ary node; f_embed -> f_deduce -> cmp_deduce and f_project -> f_ask
// -> cmp_ask on a formula), and the non-recursive helpers (residuals,
// division) sit only at the end of a chain.  With the frames ptxas reports
// (-Xptxas -v: t_embed_rec <= 112 B, t_project_rec <= 80 B, f_embed 16 B +
// f_deduce_rec 64 B + cmp_deduce <= 88 B, idiv_hull <= 112 B; the residuals
// are inlined) a level needs at most 192 B and the end of the chain 112 B
// more; 256 B per level plus 1 KB covers both.
constexpr size_t PC_FRAME_BYTES = 256;
size_t pc_stack_need(int depth) { return (size_t)(depth + 2) * PC_FRAME_BYTES + 1024; }

int pc_prepare_stack(pirgpu_ctx *ctx, PcState *s) {
  const size_t need = pc_stack_need(s->max_depth);
  if (need <= s->stack_bytes) return PIR_OK;
  size_t cur = 0;
  PIR_CK(cudaDeviceGetLimit(&cur, cudaLimitStackSize));
  if (cur < need) {
    PIR_CK(cudaStreamSynchronize(ctx->stream));
    PIR_CK(cudaDeviceSetLimit(cudaLimitStackSize, need));
  }
  s->stack_bytes = need;
  return PIR_OK;
}

// First node of root's tree when the nodes reached from root are each
// reached once, form the contiguous range [base, root] and number at most
// PC_TREE_MAX; else -1.
int tree_base_of(PcState *s, int root) {
  if (s->stamp.size() < s->tape.size()) s->stamp.resize(s->tape.size(), 0u);
  if (++s->stamp_gen == 0u) {
    std::fill(s->stamp.begin(), s->stamp.end(), 0u);
    s->stamp_gen = 1u;
  }
  const unsigned gen = s->stamp_gen;
  int todo[2 * PC_TREE_MAX + 2];
  int top = 0, count = 0, lo = root;
  todo[top++] = root;
  while (top > 0) {
    const int n = todo[--top];
    if (s->stamp[(size_t)n] == gen || ++count > PC_TREE_MAX) return -1;
    s->stamp[(size_t)n] = gen;
    lo = std::min(lo, n);
    const int4 d = s->tape[(size_t)n];
    const int k = d.x;
    if (k == K_AE) return -1;  // store formulas take the recursive path
    int kids[PC_TREE_MAX + 2];
    int nk = 0;
    if (k == K_FORMULA || k == K_NEG || k == K_ABS || k == K_ARG) kids[nk++] = d.y;
    else if (k == K_NADD || k == K_NMUL) {
      if (d.z > PC_TREE_MAX) return -1;
      for (int i = 0; i < d.z; ++i) kids[nk++] = d.y + i;
    } else if ((k >= K_ADD && k <= K_MAX) || (k >= K_LEQ && k <= K_XOR)) {
      kids[nk++] = d.y;
      kids[nk++] = d.z;
    }
    if (top + nk > 2 * PC_TREE_MAX + 2) return -1;
    for (int i = 0; i < nk; ++i) todo[top++] = kids[i];
  }
  return lo == root - count + 1 ? lo : -1;
}

// The variable -> formula adjacency of the event schedule (CSR over the
// engine order): the distinct variable leaves of every formula.
int pc_build_csr(pirgpu_ctx *ctx, PcState *s) {
  const int nv = ctx->nvars, np = (int)s->roots.size();
  // on the host's threads; the same arrays as a sequential walk
  std::vector<int> deg((size_t)nv + 1, 0), adj;
  if (!build_formula_adjacency(np, s->roots.data(), reinterpret_cast<const int32_t *>(s->tape.data()), nv, deg.data(),
                               adj, adjacency_threads((long long)s->tape.size(), 0, nv)))
    return set_err(ctx, PIR_EINVAL, "PC event schedule: more than 2^31 - 1 adjacency entries");
  int r;
  if ((r = ensure(ctx, (void **)&s->d_adj_ptr, &s->cap_adj_ptr, deg.size() * sizeof(int)))) return r;
  if ((r = ensure(ctx, (void **)&s->d_adj, &s->cap_adj, std::max<size_t>(adj.size(), 1) * sizeof(int)))) return r;
  if ((r = ensure(ctx, (void **)&s->d_list, &s->cap_list, (size_t)2 * np * sizeof(int)))) return r;
  if ((r = ensure(ctx, (void **)&s->d_pstamp, &s->cap_pstamp, (size_t)np * sizeof(unsigned)))) return r;
  if ((r = ensure(ctx, (void **)&s->d_cnt, &s->cap_cnt, 2 * sizeof(unsigned)))) return r;
  PIR_CK(cudaMemcpyAsync(s->d_adj_ptr, deg.data(), deg.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (!adj.empty())
    PIR_CK(cudaMemcpyAsync(s->d_adj, adj.data(), adj.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  s->csr_valid = true;
  s->csr_nvars = nv;
  return PIR_OK;
}

int pc_upload(pirgpu_ctx *ctx, PcState *s) {
  int r;
  s->csr_valid = false;
  if (!s->tape.empty()) {
    if ((r = ensure(ctx, (void **)&s->d_tape, &s->cap_tape, s->tape.size() * sizeof(int4)))) return r;
    PIR_CK(cudaMemcpyAsync(s->d_tape, s->tape.data(), s->tape.size() * sizeof(int4), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  std::vector<int> bases(s->roots.size());
  if (!s->roots.empty()) {
    if ((r = ensure(ctx, (void **)&s->d_roots, &s->cap_roots, s->roots.size() * sizeof(int)))) return r;
    PIR_CK(cudaMemcpyAsync(s->d_roots, s->roots.data(), s->roots.size() * sizeof(int), cudaMemcpyHostToDevice,
                           ctx->stream));
    for (size_t i = 0; i < s->roots.size(); ++i) bases[i] = s->tree_base[(size_t)s->roots[i]];
    if ((r = ensure(ctx, (void **)&s->d_bases, &s->cap_bases, bases.size() * sizeof(int)))) return r;
    PIR_CK(cudaMemcpyAsync(s->d_bases, bases.data(), bases.size() * sizeof(int), cudaMemcpyHostToDevice,
                           ctx->stream));
  }
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

}  // namespace

void destroy_pc_state(pirgpu_ctx *ctx) {
  if (!ctx->pc) return;
  if (ctx->pc->d_tape) cudaFree(ctx->pc->d_tape);
  if (ctx->pc->d_roots) cudaFree(ctx->pc->d_roots);
  if (ctx->pc->d_next) cudaFree(ctx->pc->d_next);
  if (ctx->pc->d_bases) cudaFree(ctx->pc->d_bases);
  for (void *q : {(void *)ctx->pc->d_adj_ptr, (void *)ctx->pc->d_adj, (void *)ctx->pc->d_list,
                  (void *)ctx->pc->d_pstamp, (void *)ctx->pc->d_cnt})
    if (q) cudaFree(q);
  delete ctx->pc;
  ctx->pc = nullptr;
}

int pc_max_var_used(const pirgpu_ctx *ctx) { return ctx->pc ? ctx->pc->max_var : -1; }
long long pc_count(const pirgpu_ctx *ctx) { return ctx->pc ? (long long)ctx->pc->roots.size() : 0; }

// restore(): pops propagators from the end of the engine order (pc.hpp:717-724)
int pc_truncate(pirgpu_ctx *ctx, long long n) {
  if (!ctx->pc || (long long)ctx->pc->roots.size() <= n) return PIR_OK;
  ctx->pc->roots.resize((size_t)n);
  return pc_upload(ctx, ctx->pc);
}

}  // namespace pirgpu

using namespace pirgpu;

extern "C" {

int pc_tell(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
            const int32_t *c, int32_t nprops, const int32_t *roots) {
  if (!ctx) return PIR_EINVAL;
  if (nnodes < 0 || nprops < 0) return set_err(ctx, PIR_EINVAL, "negative size");
  if (nnodes > 0 && (!kind || !a || !b || !c)) return set_err(ctx, PIR_EINVAL, "null tape");
  if (nprops > 0 && !roots) return set_err(ctx, PIR_EINVAL, "null roots");
  PcState *s = pc_state(ctx);
  const long long base = (long long)s->tape.size();
  if (base + nnodes > INT_MAX / 2) return set_err(ctx, PIR_EINVAL, "tape too large");
  // check every node: kinds, children before parents and of the right sort,
  // variables in range, depth
  std::vector<int> depth((size_t)nnodes, 1);
  int max_var = s->max_var;
  for (int32_t i = 0; i < nnodes; ++i) {
    const int k = kind[i];
    bool ok = c[i] == 0 || item_kind(k);
    int dep = 1;
    auto child = [&](int x, bool term) {
      return x >= 0 && x < i && (term ? term_kind(kind[x]) : formula_kind(kind[x]));
    };
    switch (k) {
      case K_VAR:
      case K_PVAR:
      case K_NVAR:
      case K_TELL:
      case K_NTELL:
      case K_ASK:
      case K_NASK:
      case K_ASK_OUT:
      case K_NASK_OUT:
        ok = ok && a[i] >= 0 && a[i] < ctx->nvars;
        if (ok) max_var = std::max(max_var, a[i]);
        break;
      case K_AE:
        ok = ok && b[i] >= 0 && a[i] >= 0 && (long long)a[i] + b[i] <= i;
        for (int j = 0; ok && j < b[i]; ++j) ok = item_kind(kind[a[i] + j]);
        break;
      case K_CONST:
      case K_TRUE:
      case K_FALSE: break;
      case K_FORMULA:
        ok = ok && child(a[i], false);
        if (ok) dep = 1 + depth[(size_t)a[i]];
        break;
      case K_NEG:
      case K_ABS:
      case K_ARG:
        ok = ok && child(a[i], true);
        if (ok) dep = (k == K_ARG ? 0 : 1) + depth[(size_t)a[i]];
        break;
      case K_NADD:
      case K_NMUL:
        ok = ok && b[i] >= 1 && a[i] >= 0 && (long long)a[i] + b[i] <= i;
        for (int j = 0; ok && j < b[i]; ++j) {
          ok = kind[a[i] + j] == K_ARG;
          if (ok) dep = std::max(dep, 1 + depth[(size_t)(a[i] + j)]);
        }
        break;
      default:
        if ((k >= K_ADD && k <= K_MAX) || (k >= K_LEQ && k <= K_NEQ)) ok = ok && child(a[i], true) && child(b[i], true);
        else if (k >= K_AND && k <= K_XOR) ok = ok && child(a[i], false) && child(b[i], false);
        else ok = false;
        if (ok) dep = 1 + std::max(depth[(size_t)a[i]], depth[(size_t)b[i]]);
    }
    if (!ok) return set_err(ctx, PIR_EINVAL, "tape node %d (kind %d): bad kind, operand or variable", i, k);
    if (dep > PC_MAX_DEPTH) return set_err(ctx, PIR_EINVAL, "tape node %d: depth %d > %d", i, dep, PC_MAX_DEPTH);
    depth[(size_t)i] = dep;
  }
  int max_depth = s->max_depth;
  for (int32_t p = 0; p < nprops; ++p) {
    if (roots[p] < 0 || roots[p] >= nnodes || !formula_kind(kind[roots[p]]))
      return set_err(ctx, PIR_EINVAL, "propagator %d: root %d is not a formula node of this tape", p, roots[p]);
    max_depth = std::max(max_depth, depth[(size_t)roots[p]]);
  }
  // append, with the tree lengths (Formula::length / Term::length) the order uses
  const int off = (int)base;
  for (int32_t i = 0; i < nnodes; ++i) {
    const int k = kind[i];
    const bool refs_a = !(k == K_VAR || k == K_PVAR || k == K_NVAR || k == K_CONST || k == K_TRUE || k == K_FALSE ||
                          item_kind(k));
    const bool refs_b = (k >= K_ADD && k <= K_MAX) || (k >= K_LEQ && k <= K_XOR);
    int4 nd;
    nd.x = k;
    nd.y = refs_a ? a[i] + off : a[i];
    nd.z = refs_b ? b[i] + off : b[i];
    nd.w = item_kind(k) ? c[i] : 0;
    s->tape.push_back(nd);
    long long len = 1;
    auto L = [&](int x) { return s->len[(size_t)x]; };
    if (k == K_FORMULA || k == K_ARG) len = L(nd.y);
    else if (k == K_NEG || k == K_ABS) len = 1 + L(nd.y);
    else if (k == K_NADD || k == K_NMUL) {
      for (int j = 0; j < b[i]; ++j) len += L(nd.y + j);
    } else if (refs_b) len = 1 + L(nd.y) + L(nd.z);
    s->len.push_back(std::min(len, 1ll << 40));
    s->depth.push_back(depth[(size_t)i]);
  }
  s->tree_base.resize(s->tape.size(), -1);
  for (int32_t p = 0; p < nprops; ++p) {
    s->roots.push_back(roots[p] + off);
    s->tree_base[(size_t)(roots[p] + off)] = tree_base_of(s, roots[p] + off);
  }
  const std::vector<int4> &T = s->tape;
  parallel_stable_sort(s->roots, [&](int x, int y) {
    if (T[(size_t)x].x != T[(size_t)y].x) return T[(size_t)x].x < T[(size_t)y].x;
    return s->len[(size_t)x] < s->len[(size_t)y];
  }, adjacency_threads((long long)s->roots.size()));
  s->max_var = max_var;
  s->max_depth = max_depth;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = pc_prepare_stack(ctx, s))) return r;
  return pc_upload(ctx, s);
}

int64_t pc_num_deductions(const pirgpu_ctx *ctx) { return ctx ? pc_count(ctx) : 0; }

int64_t pc_tape_size(const pirgpu_ctx *ctx) { return (ctx && ctx->pc) ? (int64_t)ctx->pc->tape.size() : 0; }

int pc_get_roots(pirgpu_ctx *ctx, int32_t *roots) {
  if (!ctx) return PIR_EINVAL;
  if (!ctx->pc || ctx->pc->roots.empty()) return PIR_OK;
  if (!roots) return set_err(ctx, PIR_EINVAL, "null output");
  std::copy(ctx->pc->roots.begin(), ctx->pc->roots.end(), roots);
  return PIR_OK;
}

int pc_get_tape(pirgpu_ctx *ctx, int32_t *kind, int32_t *a, int32_t *b, int32_t *c) {
  if (!ctx) return PIR_EINVAL;
  if (!ctx->pc || ctx->pc->tape.empty()) return PIR_OK;
  if (!kind || !a || !b || !c) return set_err(ctx, PIR_EINVAL, "null output");
  for (size_t i = 0; i < ctx->pc->tape.size(); ++i) {
    kind[i] = ctx->pc->tape[i].x;
    a[i] = ctx->pc->tape[i].y;
    b[i] = ctx->pc->tape[i].z;
    c[i] = ctx->pc->tape[i].w;
  }
  return PIR_OK;
}

int pc_fixpoint(pirgpu_ctx *ctx, const pir_opts *opts_in, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  PIR_CK(cudaSetDevice(ctx->device));
  const long long n = pc_count(ctx);
  if (ctx->failed || n == 0) {
    st.status = ctx->failed ? PIR_FAILED : PIR_OK;
    if (stats) *stats = st;
    return st.status;
  }
  ++ctx->store_version;
  PcState *s = ctx->pc;
  int r;
  if ((r = pc_prepare_stack(ctx, s))) return r;
  const long long max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  const long long timeout = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  const bool events = opts.sched == PIR_SCHED_EVENTS;
  const void *kfn = events ? (const void *)k_pc_fixpoint<true> : (const void *)k_pc_fixpoint<false>;
  // shared memory: the per-thread scratch of the trees' two passes
  PIR_CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PC_TREE_SMEM));
  PIR_CK(cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, PC_BLOCK, PC_TREE_SMEM));
  if (occ < 1) return set_err(ctx, PIR_ECUDA, "PC kernel does not fit on an SM");
  const int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ;
  const int grid = (int)std::max(1ll, std::min((long long)ctx->num_sms * per_sm, (n + PC_BLOCK - 1) / PC_BLOCK));
  if ((r = ensure(ctx, (void **)&s->d_next, &s->cap_next, (size_t)ctx->nvars * sizeof(int2)))) return r;
  if ((r = reset_control(ctx))) return r;
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  PIR_CK(cudaMemcpyAsync(s->d_next, ctx->d_store, (size_t)ctx->nvars * sizeof(int2), cudaMemcpyDeviceToDevice,
                         ctx->stream));
  PcEvents ev;
  std::memset(&ev, 0, sizeof(ev));
  if (events) {
    if ((!s->csr_valid || s->csr_nvars != ctx->nvars) && (r = pc_build_csr(ctx, s))) return r;
    PIR_CK(cudaMemsetAsync(s->d_pstamp, 0, (size_t)n * sizeof(unsigned), ctx->stream));
    PIR_CK(cudaMemsetAsync(s->d_cnt, 0, 2 * sizeof(unsigned), ctx->stream));
    ev.adj_ptr = s->d_adj_ptr;
    ev.adj = s->d_adj;
    ev.stamp = s->d_pstamp;
    ev.list0 = s->d_list;
    ev.list1 = s->d_list + n;
    ev.cnt = s->d_cnt;
  }
  const int4 *tape = s->d_tape;
  const int *roots = s->d_roots, *bases = s->d_bases;
  int nprops = (int)n, nvars = ctx->nvars;
  void *args[] = {(void *)&tape, (void *)&roots, (void *)&bases, &nprops, &ctx->d_store, &s->d_next, &nvars,
                  &ctx->d_ctl, (void *)&max_rounds, (void *)&timeout, (void *)&ev};
  PIR_CK(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(PC_BLOCK), args, PC_TREE_SMEM, ctx->stream));
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  st.rounds = h.rounds;
  st.executions = events ? (int64_t)h.executions : h.rounds * n;
  st.narrowed = (int64_t)h.narrowed;
  int status;
  if (h.status) status = h.status;
  else if (h.failed) status = PIR_FAILED;
  else if (h.changed[0]) status = PIR_TIMEOUT;
  else status = PIR_OK;
  if (status == PIR_FAILED) ctx->failed = true;
  if (h.narrowed) ctx->at_fixpoint = false;
  ctx->last_grid = grid;
  st.status = status;
  if (stats) *stats = st;
  if (status == PIR_BARRIER_TIMEOUT) set_err(ctx, status, "grid barrier wait exceeded %lld ns", timeout);
  return status;
}

int pc_deduce_one(pirgpu_ctx *ctx, int64_t i, int *changed) {
  if (!ctx) return PIR_EINVAL;
  if (i < 0 || i >= pc_count(ctx)) return set_err(ctx, PIR_EINVAL, "deduce(%lld) out of range", (long long)i);
  ++ctx->store_version;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = pc_prepare_stack(ctx, ctx->pc))) return r;
  if ((r = reset_control(ctx))) return r;
  k_pc_deduce_one<<<1, 1, 0, ctx->stream>>>(ctx->pc->d_tape, ctx->pc->roots[(size_t)i], ctx->d_store, ctx->d_ctl);
  PIR_CK(cudaGetLastError());
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  if (h.failed) ctx->failed = true;
  if (h.changed[1]) ctx->at_fixpoint = false;
  if (changed) *changed = h.changed[0];
  return PIR_OK;
}

int pc_ask_all(pirgpu_ctx *ctx, uint8_t *entailed) {
  if (!ctx) return PIR_EINVAL;
  const long long n = pc_count(ctx);
  if (n == 0) return PIR_OK;
  if (!entailed) return set_err(ctx, PIR_EINVAL, "null output");
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = pc_prepare_stack(ctx, ctx->pc))) return r;
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, (size_t)n))) return r;
  unsigned char *d = (unsigned char *)ctx->d_scratch;
  const int grid = (int)std::min<long long>(ctx->num_sms * 4, (n + PC_BLOCK - 1) / PC_BLOCK);
  k_pc_ask_all<<<grid, PC_BLOCK, 0, ctx->stream>>>(ctx->pc->d_tape, ctx->pc->d_roots, (int)n, ctx->d_store,
                                                   ctx->failed ? 1 : 0, d);
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaMemcpyAsync(entailed, d, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int pc_ask(pirgpu_ctx *ctx, int64_t i, int *entailed) {
  if (!ctx || !entailed) return PIR_EINVAL;
  if (i < 0 || i >= pc_count(ctx)) return set_err(ctx, PIR_EINVAL, "ask(%lld) out of range", (long long)i);
  std::vector<uint8_t> all((size_t)pc_count(ctx));
  int r = pc_ask_all(ctx, all.data());
  if (r) return r;
  *entailed = all[(size_t)i];
  return PIR_OK;
}

int pc_is_extractable(pirgpu_ctx *ctx, int *extractable) {
  if (!ctx || !extractable) return PIR_EINVAL;
  *extractable = 0;
  if (ctx->failed) return PIR_OK;
  std::vector<uint8_t> all((size_t)pc_count(ctx));
  int r = pc_ask_all(ctx, all.data());
  if (r) return r;
  for (uint8_t v : all)
    if (!v) return PIR_OK;
  *extractable = 1;
  return PIR_OK;
}

}  // extern "C"
