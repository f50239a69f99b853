// lala_gpu::fzn::compile_pc -- FlatZinc front end for lala_gpu::PC.
//
// lala-pc's PC tests build their instances from FlatZinc through lala-parsing
// and PC::interpret (create_and_interpret_and_tell / interpret_must_succeed,
// tests/pc_test.cpp).  Neither lala-parsing nor lala-core is part of lala-pc;
// this header restates the job for the FlatZinc subset of those tests: every
// constraint is interpreted as one formula tree (pc.hpp:505-573) instead of
// being ternarized, and a comparison of one variable with a constant goes to
// the store, as PC lets its VStore interpret it first (pc.hpp:576-605).
//
// Constraint position imposes a formula, argument position makes a term
// (integer functions) or a formula (boolean functions; as a term, a formula
// is its truth value, pc.hpp:261-297):
//   int_le int_lt int_ge int_gt int_eq int_ne, bool_le bool_lt bool_eq
//   bool_ne (+ _reif):         <=, >, ==, != on terms (a < b is b > a,
//                              a >= b is b <= a, pc.hpp:565-566); == and !=
//                              between formulas are <=> and xor (pc.hpp:553-560)
//   int_plus int_minus int_times int_div (truncating) int_tdiv int_fdiv
//   int_cdiv int_ediv int_min int_max (2 arguments: the term; 3: x op y == z),
//   int_abs int_negate (1 argument: the term; 2: == ), int_mod int_tmod
//   int_fmod int_cmod int_emod (y - z * (y div z)), bool2int
//   int_lin_eq int_lin_ne int_lin_le int_lin_lt int_lin_ge int_lin_gt: a
//                              binary sum for two terms, an n-ary one beyond
//                              (pc.hpp:278-297)
//   bool_lin_eq bool_lin_le:   as int_lin_*
//   array_int_maximum array_int_minimum: m == max (min) chain of the terms
//   fzn_all_different_int all_different_int: a conjunction of pairwise !=
//   bool_and bool_or bool_xor bool_not, array_bool_and array_bool_or,
//   array_bool_xor, bool_clause: connectives, clauses as right-nested
//                              disjunctions of literals (binarize, pc.hpp:467-476)
//   f_imp(args..., r):         r => f(args...) for every boolean f
//   set_in (+ _reif):          a range is a store bound; a set is a
//                              disjunction of its runs (x == v, or
//                              lo <= x and x <= hi)
//   array_int_element array_var_int_element array_bool_element
//   array_var_bool_element:    one propagator (i == k) => (x == a[k]) per k
// Declarations as in compile(): a set domain gives the store its hull plus
// the membership formula.
#ifndef PIRGPU_FZN_PC_HPP
#define PIRGPU_FZN_PC_HPP

#include "pirgpu_fzn.hpp"
#include "pirgpu_pc.hpp"

namespace lala_gpu {
namespace fzn {

// A model for PC: the store (user variables in declaration order), the
// formula propagators, and what the last compile_pc call added.
struct PcModel {
  std::vector<Itv> dom;
  std::vector<std::string> name;
  std::vector<pc::Formula> props;
  std::map<std::string, int> var_index;
  std::map<std::string, std::vector<int>> var_arrays;
  std::map<std::string, long long> params;
  std::map<std::string, std::vector<long long>> param_arrays;
  // last compile_pc: variables before it, propagators before it, and its
  // store meets on variables that existed before it
  size_t nvars0 = 0, nprops0 = 0;
  std::vector<std::pair<int, Itv>> meets;

  int index_of(const std::string &n) const {
    auto it = var_index.find(n);
    return it == var_index.end() ? -1 : it->second;
  }
};

namespace detail {

class PcCompiler {
 public:
  using T = pc::Term;
  using F = pc::Formula;

  PcCompiler(PcModel &m, IDiagnostics &d) : m_(m), d_(d) {}

  bool error(const std::string &msg) {
    d_.errors.push_back(msg);
    return false;
  }

  int declare(const std::string &n, Itv d) {
    m_.dom.push_back(d);
    m_.name.push_back(n);
    m_.var_index[n] = (int)m_.dom.size() - 1;
    return (int)m_.dom.size() - 1;
  }

  // a store part: x in [lo, hi]
  void restrict(int v, long long lo, long long hi) {
    const int32_t l = (int32_t)std::max<long long>(INT32_MIN, std::min<long long>(INT32_MAX, lo));
    const int32_t u = (int32_t)std::max<long long>(INT32_MIN, std::min<long long>(INT32_MAX, hi));
    Itv &d = m_.dom[(size_t)v];
    d.lb = std::max(d.lb, l);
    d.ub = std::min(d.ub, u);
    if ((size_t)v < m_.nvars0) m_.meets.emplace_back(v, Itv(l, u));
  }

  bool var_of(const Expr &e, int &v) {
    if (e.kind == Expr::IDENT) {
      v = m_.index_of(e.id);
      return v >= 0;
    }
    if (e.kind == Expr::ACCESS) {
      auto a = m_.var_arrays.find(e.id);
      if (a == m_.var_arrays.end() || e.v < 1 || e.v > (long long)a->second.size()) return false;
      v = a->second[(size_t)e.v - 1];
      return true;
    }
    return false;
  }
  bool const_of(const Expr &e, long long &c) {
    if (e.kind == Expr::INT || e.kind == Expr::BOOL) {
      c = e.v;
      return true;
    }
    if (e.kind == Expr::IDENT) {
      auto p = m_.params.find(e.id);
      if (p == m_.params.end()) return false;
      c = p->second;
      return true;
    }
    if (e.kind == Expr::ACCESS) {
      auto p = m_.param_arrays.find(e.id);
      if (p == m_.param_arrays.end() || e.v < 1 || e.v > (long long)p->second.size()) return false;
      c = p->second[(size_t)e.v - 1];
      return true;
    }
    return false;
  }
  static T konst(long long c) {
    const int32_t v = (int32_t)std::max<long long>(INT32_MIN, std::min<long long>(INT32_MAX, c));
    return T::make_constant(Itv(v, v));
  }

  // elements of an array argument, as expressions
  bool elements(const Expr &e, std::vector<Expr> &out) {
    if (e.kind == Expr::ARRAY) {
      out = e.args;
      return true;
    }
    if (e.kind == Expr::IDENT) {
      auto a = m_.var_arrays.find(e.id);
      if (a != m_.var_arrays.end()) {
        for (size_t k = 0; k < a->second.size(); ++k) {
          Expr x;
          x.kind = Expr::ACCESS;
          x.id = e.id;
          x.v = (long long)k + 1;
          out.push_back(x);
        }
        return true;
      }
      auto p = m_.param_arrays.find(e.id);
      if (p != m_.param_arrays.end()) {
        for (long long c : p->second) {
          Expr x;
          x.kind = Expr::INT;
          x.v = c;
          out.push_back(x);
        }
        return true;
      }
    }
    return error("array expected");
  }
  bool ints(const Expr &e, std::vector<long long> &out) {
    if (e.kind == Expr::RANGE) {
      for (long long k = e.v; k <= e.hi; ++k) out.push_back(k);
      return true;
    }
    std::vector<Expr> xs;
    if (e.kind == Expr::SET) xs = e.args;
    else if (!elements(e, xs)) return false;
    for (const Expr &x : xs) {
      long long c;
      if (!const_of(x, c)) return error("constant expected");
      out.push_back(c);
    }
    return true;
  }

  static bool is_bool_fn(const std::string &f) {
    static const char *names[] = {"int_le", "int_lt", "int_ge", "int_gt", "int_eq", "int_ne", "bool_le",
                                  "bool_lt", "bool_eq", "bool_ne", "bool_and", "bool_or", "bool_xor",
                                  "bool_not", "bool_clause", "array_bool_and", "array_bool_or", "set_in",
                                  "int_lin_eq", "int_lin_ne", "int_lin_le", "int_lin_lt", "int_lin_ge",
                                  "int_lin_gt", "bool_lin_eq", "bool_lin_le", "array_bool_xor"};
    for (const char *n : names)
      if (f == n) return true;
    return (f.size() > 5 && f.compare(f.size() - 5, 5, "_reif") == 0) ||
           (f.size() > 4 && f.compare(f.size() - 4, 4, "_imp") == 0);
  }
  bool is_predicate(const Expr &e) const { return e.kind == Expr::CALL && is_bool_fn(e.id); }

  // negation of a formula (lala-core's negate(), which PC applies to a
  // negated sub-formula, pc.hpp:334-343): literals flip, comparisons complement,
  // De Morgan for and / or, <=> and xor exchange, not (f => g) is f and not g
  static F negate(const F &f) {
    const pc::NodePtr &n = f.node();
    auto kid = [&](size_t i) { return F(n->kids[i]); };
    auto term = [&](size_t i) { return T(n->kids[i]); };
    switch (n->kind) {
      case PC_PVAR: return F::make_nvarlit(n->a);
      case PC_NVAR: return F::make_pvarlit(n->a);
      case PC_TRUE: return F::make_false();
      case PC_FALSE: return F::make_true();
      case PC_LEQ: return F::make_gt(term(0), term(1));
      case PC_GT: return F::make_leq(term(0), term(1));
      case PC_EQ: return F::make_neq(term(0), term(1));
      case PC_NEQ: return F::make_eq(term(0), term(1));
      case PC_AND: return F::make_disj(negate(kid(0)), negate(kid(1)));
      case PC_OR: return F::make_conj(negate(kid(0)), negate(kid(1)));
      case PC_EQUIV: return F::make_xor(kid(0), kid(1));
      case PC_XOR: return F::make_bicond(kid(0), kid(1));
      default: return F::make_conj(kid(0), negate(kid(1)));  // IMPLY
    }
  }

  // -- terms --------------------------------------------------------------
  bool term(const Expr &e, T &out) {
    int v;
    long long c;
    if (var_of(e, v)) {
      out = T::make_var(v);
      return true;
    }
    if (const_of(e, c)) {
      out = konst(c);
      return true;
    }
    if (e.kind != Expr::CALL) return error("not a term");
    const std::string &f = e.id;
    if (is_bool_fn(f)) {  // a formula used as a term (pc.hpp:268-277)
      F g;
      if (!formula(e, g)) return false;
      out = T::make_formula(g);
      return true;
    }
    std::vector<T> a(e.args.size());
    for (size_t k = 0; k < e.args.size(); ++k)
      if (!term(e.args[k], a[k])) return false;
    if (a.size() == 1) {
      if (f == "int_abs") return out = T::make_abs(a[0]), true;
      if (f == "int_negate" || f == "int_neg") return out = T::make_neg(a[0]), true;
      if (f == "bool2int") return out = a[0], true;
    }
    if (a.size() == 2) {
      if (f == "int_plus") return out = T::make_add(a[0], a[1]), true;
      if (f == "int_minus") return out = T::make_sub(a[0], a[1]), true;
      if (f == "int_times") return out = T::make_mul(a[0], a[1]), true;
      if (f == "int_div" || f == "int_tdiv") return out = T::make_tdiv(a[0], a[1]), true;
      if (f == "int_fdiv") return out = T::make_fdiv(a[0], a[1]), true;
      if (f == "int_cdiv") return out = T::make_cdiv(a[0], a[1]), true;
      if (f == "int_ediv") return out = T::make_ediv(a[0], a[1]), true;
      if (f == "int_min") return out = T::make_min(a[0], a[1]), true;
      if (f == "int_max") return out = T::make_max(a[0], a[1]), true;
      if (f == "int_mod" || f == "int_tmod" || f == "int_fmod" || f == "int_cmod" || f == "int_emod") {
        const T q = f == "int_fmod"   ? T::make_fdiv(a[0], a[1])
                    : f == "int_cmod" ? T::make_cdiv(a[0], a[1])
                    : f == "int_emod" ? T::make_ediv(a[0], a[1])
                                      : T::make_tdiv(a[0], a[1]);
        out = T::make_sub(a[0], T::make_mul(a[1], q));
        return true;
      }
    }
    return error("unsupported term " + f);
  }

  // sum_k c[k] * x[k]: a binary sum for two terms, an n-ary one beyond
  bool linear(const Expr &cs, const Expr &xs, T &out) {
    std::vector<long long> c;
    std::vector<Expr> x;
    if (!ints(cs, c) || !elements(xs, x)) return false;
    if (c.size() != x.size()) return error("int_lin: coefficient and variable counts differ");
    std::vector<T> ts;
    for (size_t k = 0; k < c.size(); ++k) {
      T t;
      if (!term(x[k], t)) return false;
      ts.push_back(c[k] == 1 ? t : T::make_mul(konst(c[k]), t));
    }
    if (ts.empty()) out = konst(0);
    else if (ts.size() == 1) out = ts[0];
    else if (ts.size() == 2) out = T::make_add(ts[0], ts[1]);
    else out = T::make_naryadd(ts);
    return true;
  }

  // x in S: a disjunction over the runs of S
  bool member(const T &x, const Expr &S, F &out) {
    std::vector<long long> v;
    if (!ints(S, v)) return false;
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    if (v.empty()) return out = F::make_false(), true;
    std::vector<F> runs;
    for (size_t i = 0; i < v.size();) {
      size_t j = i;
      while (j + 1 < v.size() && v[j + 1] == v[j] + 1) ++j;
      runs.push_back(i == j ? F::make_eq(x, konst(v[i]))
                            : F::make_conj(F::make_leq(konst(v[i]), x), F::make_leq(x, konst(v[j]))));
      i = j + 1;
    }
    out = disjunction(runs);
    return true;
  }
  static F disjunction(const std::vector<F> &fs) {
    F r = fs.back();
    for (size_t k = fs.size() - 1; k-- > 0;) r = F::make_disj(fs[k], r);
    return r;
  }
  static F conjunction(const std::vector<F> &fs) {
    F r = fs.back();
    for (size_t k = fs.size() - 1; k-- > 0;) r = F::make_conj(fs[k], r);
    return r;
  }

  // -- formulas -------------------------------------------------------------
  bool formula(const Expr &e, F &out) {
    int v;
    long long c;
    if (var_of(e, v)) return out = F::make_pvarlit(v), true;
    if (const_of(e, c)) return out = c ? F::make_true() : F::make_false(), true;
    if (e.kind != Expr::CALL) return error("not a formula");
    const std::string &f = e.id;
    const std::vector<Expr> &A = e.args;
    if (f.size() > 5 && f.compare(f.size() - 5, 5, "_reif") == 0) {  // r <=> f(args)
      if (A.empty()) return error(f + ": no arguments");
      Expr inner = e;
      inner.id = f.substr(0, f.size() - 5);
      inner.args.pop_back();
      F r, g;
      if (!formula(A.back(), r) || !formula(inner, g)) return false;
      out = F::make_bicond(r, g);
      return true;
    }
    if (f.size() > 4 && f.compare(f.size() - 4, 4, "_imp") == 0) {  // r => f(args)
      if (A.empty()) return error(f + ": no arguments");
      Expr inner = e;
      inner.id = f.substr(0, f.size() - 4);
      inner.args.pop_back();
      F r, g;
      if (!formula(A.back(), r) || !formula(inner, g)) return false;
      out = F::make_imply(r, g);
      return true;
    }
    const bool cmp = f == "int_le" || f == "int_lt" || f == "int_ge" || f == "int_gt" || f == "int_eq" ||
                     f == "int_ne" || f == "bool_le" || f == "bool_lt" || f == "bool_eq" || f == "bool_ne";
    if (cmp || f == "bool_and" || f == "bool_or" || f == "bool_xor") {
      if (A.size() == 3) {  // f(a, b, r): r <=> f(a, b)
        Expr inner = e;
        inner.args.pop_back();
        F r, g;
        if (!formula(A[2], r) || !formula(inner, g)) return false;
        out = F::make_bicond(r, g);
        return true;
      }
      if (A.size() != 2) return error(f + ": expected 2 arguments");
      if (!cmp || ((f == "int_eq" || f == "int_ne" || f == "bool_eq" || f == "bool_ne") &&
                   (is_predicate(A[0]) || is_predicate(A[1])))) {
        F p, q;
        if (!formula(A[0], p) || !formula(A[1], q)) return false;
        if (f == "bool_and") out = F::make_conj(p, q);
        else if (f == "bool_or") out = F::make_disj(p, q);
        else if (f == "bool_xor" || f == "int_ne" || f == "bool_ne") out = F::make_xor(p, q);
        else out = F::make_bicond(p, q);
        return true;
      }
      T a, b;
      if (!term(A[0], a) || !term(A[1], b)) return false;
      if (f == "int_le" || f == "bool_le") out = F::make_leq(a, b);
      else if (f == "int_lt" || f == "bool_lt") out = F::make_gt(b, a);
      else if (f == "int_ge") out = F::make_leq(b, a);
      else if (f == "int_gt") out = F::make_gt(a, b);
      else if (f == "int_eq" || f == "bool_eq") out = F::make_eq(a, b);
      else out = F::make_neq(a, b);
      return true;
    }
    if (f == "bool_not") {
      F p;
      if (A.empty() || A.size() > 2 || !formula(A[0], p)) return A.empty() ? error("bool_not: no argument") : false;
      if (A.size() == 1) return out = negate(p), true;
      F q;
      if (!formula(A[1], q)) return false;
      out = F::make_bicond(q, negate(p));
      return true;
    }
    if (f == "bool_clause") {
      std::vector<Expr> pos, neg;
      if (A.size() != 2 || !elements(A[0], pos) || !elements(A[1], neg)) return error("bool_clause: two arrays");
      std::vector<F> lits;
      for (const Expr &x : pos) {
        F l;
        if (!formula(x, l)) return false;
        lits.push_back(l);
      }
      for (const Expr &x : neg) {
        F l;
        if (!formula(x, l)) return false;
        lits.push_back(negate(l));
      }
      out = lits.empty() ? F::make_false() : disjunction(lits);
      return true;
    }
    if (f == "array_bool_and" || f == "array_bool_or") {
      std::vector<Expr> xs;
      if (A.empty() || A.size() > 2 || !elements(A[0], xs)) return error(f + ": an array");
      std::vector<F> fs;
      for (const Expr &x : xs) {
        F l;
        if (!formula(x, l)) return false;
        fs.push_back(l);
      }
      F g = fs.empty() ? (f == "array_bool_and" ? F::make_true() : F::make_false())
                       : (f == "array_bool_and" ? conjunction(fs) : disjunction(fs));
      if (A.size() == 1) return out = g, true;
      F r;
      if (!formula(A[1], r)) return false;
      out = F::make_bicond(r, g);
      return true;
    }
    if (f == "set_in") {
      T x;
      if (A.size() == 3) {
        Expr inner = e;
        inner.args.pop_back();
        F r, g;
        if (!formula(A[2], r) || !formula(inner, g)) return false;
        return out = F::make_bicond(r, g), true;
      }
      if (A.size() != 2 || !term(A[0], x)) return error("set_in: two arguments");
      return member(x, A[1], out);
    }
    if (f == "array_bool_xor") {  // odd parity: x1 xor (x2 xor (... xor xn))
      std::vector<Expr> xs;
      if (A.size() != 1 || !elements(A[0], xs)) return error(f + ": an array");
      if (xs.empty()) return out = F::make_false(), true;
      F r;
      if (!formula(xs.back(), r)) return false;
      for (size_t k = xs.size() - 1; k-- > 0;) {
        F l;
        if (!formula(xs[k], l)) return false;
        r = F::make_xor(l, r);
      }
      out = r;
      return true;
    }
    if (f == "fzn_all_different_int" || f == "all_different_int") {  // pairwise !=, as one conjunction
      std::vector<Expr> xs;
      if (A.size() != 1 || !elements(A[0], xs)) return error(f + ": an array");
      std::vector<T> ts(xs.size());
      for (size_t k = 0; k < xs.size(); ++k)
        if (!term(xs[k], ts[k])) return false;
      std::vector<F> ne;
      for (size_t i = 0; i < ts.size(); ++i)
        for (size_t j = i + 1; j < ts.size(); ++j) ne.push_back(F::make_neq(ts[i], ts[j]));
      out = ne.empty() ? F::make_true() : conjunction(ne);
      return true;
    }
    if (f == "array_int_maximum" || f == "array_int_minimum") {  // m == max (min) of xs
      std::vector<Expr> xs;
      T m;
      if (A.size() != 2 || !term(A[0], m) || !elements(A[1], xs)) return error(f + ": a term and an array");
      if (xs.empty()) return error(f + ": empty array");
      T acc;
      if (!term(xs[0], acc)) return false;
      for (size_t k = 1; k < xs.size(); ++k) {
        T t;
        if (!term(xs[k], t)) return false;
        acc = f == "array_int_maximum" ? T::make_max(acc, t) : T::make_min(acc, t);
      }
      out = F::make_eq(m, acc);
      return true;
    }
    if (f.compare(0, 8, "int_lin_") == 0 || f.compare(0, 9, "bool_lin_") == 0) {
      if (A.size() != 3) return error(f + ": expected 3 arguments");
      T s, k;
      if (!linear(A[0], A[1], s) || !term(A[2], k)) return false;
      const std::string op = f.substr(f[0] == 'i' ? 8 : 9);
      if (op == "eq") out = F::make_eq(s, k);
      else if (op == "ne") out = F::make_neq(s, k);
      else if (op == "le") out = F::make_leq(s, k);
      else if (op == "lt") out = F::make_gt(k, s);
      else if (op == "ge") out = F::make_leq(k, s);
      else if (op == "gt") out = F::make_gt(s, k);
      else return error("unsupported " + f);
      return true;
    }
    // a function with its result: x op y == z, |x| == y, -x == y, x == y
    if ((A.size() == 3 && !is_bool_fn(f)) ||
        (A.size() == 2 && (f == "int_abs" || f == "int_negate" || f == "int_neg" || f == "bool2int"))) {
      Expr inner = e;
      inner.args.pop_back();
      T l, r;
      if (!term(inner, l) || !term(A.back(), r)) return false;
      out = F::make_eq(l, r);
      return true;
    }
    return error("unsupported constraint " + f);
  }

  // -- constraints ------------------------------------------------------------
  // a comparison of one variable with a constant, interpreted by the store
  bool store_bound(const Expr &e) {
    if (e.kind != Expr::CALL || e.args.size() != 2) return false;
    const std::string &f = e.id;
    int v;
    long long c;
    if (f == "set_in") {
      if (!var_of(e.args[0], v) || e.args[1].kind != Expr::RANGE) return false;
      restrict(v, e.args[1].v, e.args[1].hi);
      return true;
    }
    const bool vl = var_of(e.args[0], v) && const_of(e.args[1], c);
    const bool vr = !vl && const_of(e.args[0], c) && var_of(e.args[1], v);
    if (!vl && !vr) return false;
    const long long inf = LLONG_MAX / 4;
    if (f == "int_eq" || f == "bool_eq") restrict(v, c, c);
    else if (f == "int_le" || f == "bool_le") vl ? restrict(v, -inf, c) : restrict(v, c, inf);
    else if (f == "int_ge") vl ? restrict(v, c, inf) : restrict(v, -inf, c);
    else if (f == "int_lt" || f == "bool_lt") vl ? restrict(v, -inf, c - 1) : restrict(v, c + 1, inf);
    else if (f == "int_gt") vl ? restrict(v, c + 1, inf) : restrict(v, -inf, c - 1);
    else return false;
    return true;
  }

  bool constraint(const Expr &e) {
    if (e.kind != Expr::CALL) return error("constraint: a call is expected");
    if (store_bound(e)) return true;
    const std::string &f = e.id;
    if (f == "array_int_element" || f == "array_var_int_element" || f == "array_bool_element" ||
        f == "array_var_bool_element") {
      std::vector<Expr> arr;
      int i;
      if (e.args.size() != 3 || !var_of(e.args[0], i) || !elements(e.args[1], arr))
        return error(f + ": (index variable, array, value) expected");
      if (arr.empty()) return error(f + ": empty array");
      T x;
      if (!term(e.args[2], x)) return false;
      restrict(i, 1, (long long)arr.size());
      int xv;
      if (var_of(e.args[2], xv)) {
        long long lo = LLONG_MAX, hi = LLONG_MIN;
        for (const Expr &a : arr) {
          long long c;
          int w;
          if (const_of(a, c)) {
            lo = std::min(lo, c);
            hi = std::max(hi, c);
          } else if (var_of(a, w)) {
            lo = std::min<long long>(lo, m_.dom[(size_t)w].lb);
            hi = std::max<long long>(hi, m_.dom[(size_t)w].ub);
          }
        }
        restrict(xv, lo, hi);
      }
      for (size_t k = 0; k < arr.size(); ++k) {
        T ak;
        if (!term(arr[k], ak)) return false;
        m_.props.push_back(F::make_imply(F::make_eq(T::make_var(i), konst((long long)k + 1)), F::make_eq(x, ak)));
      }
      return true;
    }
    F g;
    if (!formula(e, g)) return false;
    m_.props.push_back(g);
    return true;
  }

  bool domain_of(const Expr &t, Itv &d, std::vector<long long> *set) {
    if (t.kind == Expr::IDENT && t.id == "int") return d = Itv::top(), true;
    if (t.kind == Expr::IDENT && t.id == "bool") return d = Itv(0, 1), true;
    if (t.kind == Expr::RANGE) return d = Itv((int32_t)t.v, (int32_t)t.hi), true;
    if (t.kind == Expr::SET) {
      std::vector<long long> v;
      if (!ints(t, v) || v.empty()) return error("empty set domain");
      d = Itv((int32_t)*std::min_element(v.begin(), v.end()), (int32_t)*std::max_element(v.begin(), v.end()));
      if (set) *set = v;
      return true;
    }
    return error("unsupported type");
  }

  // a declared variable with a set domain: the membership formula
  bool declare_set(int v, const Expr &S) {
    F g;
    if (!member(T::make_var(v), S, g)) return false;
    m_.props.push_back(g);
    return true;
  }

 private:
  PcModel &m_;
  IDiagnostics &d_;
};

}  // namespace detail

// Parses `text` and adds its variables, store bounds and formulas to `m` (which
// may already hold a model, so that a later tell refers to its variables).
inline bool compile_pc(const std::string &text, PcModel &m, IDiagnostics &diag) {
  m.nvars0 = m.dom.size();
  m.nprops0 = m.props.size();
  m.meets.clear();
  detail::Parser P(text);
  detail::PcCompiler C(m, diag);
  while (!P.eof()) {
    if (P.accept("constraint")) {
      detail::Expr e;
      if (!P.expr(e)) break;
      P.annotations();
      if (!P.expect(";")) break;
      if (!C.constraint(e)) return false;
      continue;
    }
    if (P.accept("solve")) {
      P.skip_to(';');
      continue;
    }
    if (P.accept("predicate")) {
      // predicate name(params); -- a declaration a solver's library adds; nothing to compile
      std::string name;
      if (!P.ident(name) || !P.peek("(")) {
        P.fail("predicate name and parameters expected");
        break;
      }
      P.skip_parens();
      if (!P.expect(";")) break;
      continue;
    }
    if (P.accept("array")) {
      detail::Expr range;
      if (!P.expect("[") || !P.expr(range) || !P.expect("]") || !P.expect("of")) break;
      const bool isvar = P.accept("var");
      detail::Expr t;
      if (!P.expr(t) || !P.expect(":")) break;
      std::string name;
      if (!P.ident(name)) return C.error("array name expected");
      P.annotations();
      detail::Expr init;
      const bool has_init = P.accept("=") && P.expr(init);
      if (!P.expect(";")) break;
      const long long n = range.kind == detail::Expr::RANGE ? range.hi - range.v + 1 : 0;
      if (!isvar) {
        std::vector<long long> vals;
        if (!has_init || !C.ints(init, vals)) return C.error("constant array " + name + " needs its values");
        m.param_arrays[name] = vals;
        continue;
      }
      std::vector<int> vars;
      if (has_init) {
        std::vector<detail::Expr> xs;
        if (!C.elements(init, xs)) return false;
        for (const detail::Expr &x : xs) {
          int v;
          if (!C.var_of(x, v)) return C.error("array " + name + ": variables expected");
          vars.push_back(v);
        }
      } else {
        Itv d;
        std::vector<long long> set;
        if (!C.domain_of(t, d, &set)) return false;
        for (long long k = 0; k < n; ++k) {
          const int v = C.declare(name + "[" + std::to_string(k + 1) + "]", d);
          if (!set.empty() && !C.declare_set(v, t)) return false;
          vars.push_back(v);
        }
      }
      m.var_arrays[name] = vars;
      continue;
    }
    if (P.accept("var")) {
      detail::Expr t;
      if (!P.expr(t) || !P.expect(":")) break;
      std::string name;
      if (!P.ident(name)) return C.error("variable name expected");
      P.annotations();
      Itv d;
      std::vector<long long> set;
      if (!C.domain_of(t, d, &set)) return false;
      const int v = C.declare(name, d);
      if (!set.empty() && !C.declare_set(v, t)) return false;
      if (P.accept("=")) {
        detail::Expr init;
        if (!P.expr(init)) break;
        detail::Expr eq;
        eq.kind = detail::Expr::CALL;
        eq.id = "int_eq";
        detail::Expr self;
        self.kind = detail::Expr::IDENT;
        self.id = name;
        eq.args = {self, init};
        if (!C.constraint(eq)) return false;
      }
      if (!P.expect(";")) break;
      continue;
    }
    std::string ty;
    if (P.ident(ty) && (ty == "int" || ty == "bool")) {
      std::string name;
      detail::Expr init;
      if (!P.expect(":") || !P.ident(name) || !P.expect("=") || !P.expr(init) || !P.expect(";")) break;
      if (init.kind != detail::Expr::INT && init.kind != detail::Expr::BOOL)
        return C.error("parameter " + name + ": constant expected");
      m.params[name] = init.v;
      continue;
    }
    P.fail("declaration, constraint or solve item expected");
    break;
  }
  if (!P.ok()) return C.error("FlatZinc: " + P.error());
  return true;
}

// create_and_interpret_and_tell<IPC> of lala-pc's tests: a PC holding the
// model's store and formulas.
inline std::unique_ptr<PC> make_pc(const PcModel &m, int device = 0) {
  std::unique_ptr<PC> pc(new PC(m.dom, device));
  PC::tell_type t;
  t.props = m.props;
  pc->deduce(t);
  return pc;
}

// A later tell (interpret_must_succeed in lala-pc's tests): new variables
// grow the store, bounds on existing ones are met into it, new formulas are
// told.  Returns has_changed.
inline bool interpret_and_tell(PC &pc, PcModel &m, const std::string &text, IDiagnostics &diag) {
  if (!compile_pc(text, m, diag)) return false;
  bool changed = false;
  if (m.dom.size() > m.nvars0) {
    pc.add_vars(std::vector<Itv>(m.dom.begin() + (long)m.nvars0, m.dom.end()));
    changed = true;
  }
  PC::tell_type t;
  t.sub_value = m.meets;
  t.props.assign(m.props.begin() + (long)m.nprops0, m.props.end());
  changed |= pc.deduce(t);
  return changed;
}

}  // namespace fzn
}  // namespace lala_gpu

#endif
