// lala_gpu::fzn -- a FlatZinc front end for lala_gpu::PIR.
//
// lala-pc's tests build their PIR instances from FlatZinc through lala-parsing
// and lala-core's ternarizer (create_and_interpret_and_tell, used throughout
// tests/pir_test.cpp; the generated variables are listed at
// tests/pir_test.cpp:193-206).  Neither library is part of lala-pc, so this
// header restates the job: parse the FlatZinc subset those tests use
// (declarations, parameters, arrays, nested calls) and compile every
// constraint to ternary propagators x = y op z over fresh variables and
// singleton constants.  The variable numbering of the generated variables is
// this front end's own; the user variables keep their declaration order.
//
// Supported (constraint position imposes the formula, argument position
// reifies it into a 0/1 variable):
//   int_eq int_ne int_le int_lt int_ge int_gt (+ _reif), int_plus int_minus
//   int_times int_div int_tdiv int_fdiv int_cdiv int_ediv int_mod int_tmod
//   int_fmod int_emod int_min int_max int_abs int_negate,
//   int_lin_eq int_lin_ne int_lin_le int_lin_lt int_lin_ge (+ _reif),
//   bool_lin_eq bool_lin_le, array_int_maximum array_int_minimum,
//   bool_eq bool_ne bool_le bool_lt bool_not bool_and bool_or bool_xor
//   bool_clause bool2int array_bool_and array_bool_or array_bool_xor
//   (+ bool_*_reif), set_in set_in_reif, array_int_element
//   array_var_int_element array_bool_element array_var_bool_element; every
//   reifiable one also half-reified, f_imp(args..., r): r -> f(args...);
//   fzn_all_different_int / all_different_int as pairwise !=.
// Decompositions: x < y is 0 = (y <= x); x != y is 0 = (x == y);
// x = y - z is y = x + z; -x is 0 = t + x; |x| = max(x, -x); integer
// modulo m of y by z is q = y div z, p = q * z, y = p + m; a linear sum is a
// chain of ADD over MUL terms; and / or are min / max; bool_not is
// 1 = a + b; set membership is a max of reified equalities; element(i, a, x)
// is, for every k, (i == k) <= (x == a[k]) with x within the array's range.
#ifndef PIRGPU_FZN_HPP
#define PIRGPU_FZN_HPP

#include <algorithm>
#include <cctype>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "pirgpu.hpp"

namespace lala_gpu {
namespace fzn {

// A compiled model: one interval per variable (user variables first in
// declaration order, then generated ones), the propagators, and the names.
struct Model {
  std::vector<Itv> dom;
  std::vector<std::string> name;  // "" for generated variables
  std::vector<bytecode_type> props;
  std::map<std::string, int> var_index;
  std::map<std::string, std::vector<int>> var_arrays;
  std::map<std::string, long long> params;
  std::map<std::string, std::vector<long long>> param_arrays;

  int index_of(const std::string &n) const {
    auto it = var_index.find(n);
    return it == var_index.end() ? -1 : it->second;
  }
};

namespace detail {

// ---------------------------------------------------------------- syntax --
struct Expr {
  enum Kind { INT, BOOL, IDENT, ACCESS, CALL, ARRAY, RANGE, SET } kind = INT;
  long long v = 0, hi = 0;  // INT / BOOL value; RANGE v..hi; ACCESS index
  std::string id;           // IDENT, ACCESS, CALL
  std::vector<Expr> args;   // CALL arguments, ARRAY elements, SET elements
};

class Parser {
 public:
  explicit Parser(const std::string &s) : s_(s) {}
  bool ok() const { return err_.empty(); }
  const std::string &error() const { return err_; }

  void ws() {
    for (;;) {
      while (p_ < s_.size() && std::isspace((unsigned char)s_[p_])) ++p_;
      if (p_ < s_.size() && s_[p_] == '%') {
        while (p_ < s_.size() && s_[p_] != '\n') ++p_;
        continue;
      }
      break;
    }
  }
  bool eof() {
    ws();
    return p_ >= s_.size();
  }
  bool peek(const char *t) {
    ws();
    return s_.compare(p_, std::char_traits<char>::length(t), t) == 0;
  }
  bool accept(const char *t) {
    if (!peek(t)) return false;
    p_ += std::char_traits<char>::length(t);
    return true;
  }
  bool expect(const char *t) {
    if (accept(t)) return true;
    fail(std::string("expected '") + t + "'");
    return false;
  }
  void fail(const std::string &m) {
    if (err_.empty()) err_ = m + " at offset " + std::to_string(p_);
  }
  bool ident(std::string &out) {
    ws();
    size_t q = p_;
    if (q < s_.size() && (std::isalpha((unsigned char)s_[q]) || s_[q] == '_')) {
      while (q < s_.size() && (std::isalnum((unsigned char)s_[q]) || s_[q] == '_')) ++q;
      out = s_.substr(p_, q - p_);
      p_ = q;
      return true;
    }
    return false;
  }
  bool integer(long long &out) {
    ws();
    size_t q = p_;
    if (q < s_.size() && (s_[q] == '-' || s_[q] == '+')) ++q;
    if (q >= s_.size() || !std::isdigit((unsigned char)s_[q])) return false;
    while (q < s_.size() && std::isdigit((unsigned char)s_[q])) ++q;
    out = std::strtoll(s_.substr(p_, q - p_).c_str(), nullptr, 10);
    p_ = q;
    return true;
  }
  // annotations: "::" ident [ "(" ... ")" ], skipped
  void annotations() {
    while (accept("::")) {
      std::string a;
      ident(a);
      if (peek("(")) skip_parens();
    }
  }
  void skip_to(char c) {
    while (p_ < s_.size() && s_[p_] != c) ++p_;
    if (p_ < s_.size()) ++p_;
  }
  void skip_parens() {
    int depth = 0;
    do {
      ws();
      if (p_ >= s_.size()) return fail("unbalanced parentheses");
      if (s_[p_] == '(') ++depth;
      if (s_[p_] == ')') --depth;
      ++p_;
    } while (depth > 0);
  }

  bool expr(Expr &e) {
    long long v;
    std::string id;
    if (accept("[")) {
      e.kind = Expr::ARRAY;
      if (!accept("]")) {
        do {
          Expr x;
          if (!expr(x)) return false;
          e.args.push_back(x);
        } while (accept(","));
        if (!expect("]")) return false;
      }
      return true;
    }
    if (accept("{")) {
      e.kind = Expr::SET;
      if (!accept("}")) {
        do {
          Expr x;
          if (!integer(v)) return fail("set element"), false;
          x.kind = Expr::INT;
          x.v = v;
          e.args.push_back(x);
        } while (accept(","));
        if (!expect("}")) return false;
      }
      return true;
    }
    if (integer(v)) {
      if (accept("..")) {
        long long hi;
        if (!integer(hi)) return fail("range bound"), false;
        e.kind = Expr::RANGE;
        e.v = v;
        e.hi = hi;
        return true;
      }
      e.kind = Expr::INT;
      e.v = v;
      return true;
    }
    if (ident(id)) {
      if (id == "true" || id == "false") {
        e.kind = Expr::BOOL;
        e.v = id == "true";
        return true;
      }
      if (accept("(")) {
        e.kind = Expr::CALL;
        e.id = id;
        if (!accept(")")) {
          do {
            Expr x;
            if (!expr(x)) return false;
            e.args.push_back(x);
          } while (accept(","));
          if (!expect(")")) return false;
        }
        return true;
      }
      if (accept("[")) {
        if (!integer(v)) return fail("array index"), false;
        if (!expect("]")) return false;
        e.kind = Expr::ACCESS;
        e.id = id;
        e.v = v;
        return true;
      }
      e.kind = Expr::IDENT;
      e.id = id;
      return true;
    }
    fail("expression");
    return false;
  }

 private:
  const std::string &s_;
  size_t p_ = 0;
  std::string err_;
};

// ------------------------------------------------------------- compiler --
constexpr int32_t ADD = (int32_t)Sig::ADD, MUL = (int32_t)Sig::MUL, TDIV = (int32_t)Sig::TDIV,
                  FDIV = (int32_t)Sig::FDIV, CDIV = (int32_t)Sig::CDIV, EDIV = (int32_t)Sig::EDIV,
                  MIN = (int32_t)Sig::MIN, MAX = (int32_t)Sig::MAX, EQ = (int32_t)Sig::EQ, LEQ = (int32_t)Sig::LEQ;

class Compiler {
 public:
  Compiler(Model &m, IDiagnostics &d) : m_(m), d_(d) {
    for (int v = 0; v < (int)m_.dom.size(); ++v)
      if (m_.name[(size_t)v].empty() && m_.dom[(size_t)v].lb == m_.dom[(size_t)v].ub)
        consts_.emplace(m_.dom[(size_t)v].lb, v);
  }

  bool error(const std::string &msg) {
    d_.errors.push_back(msg);
    return false;
  }

  int fresh(Itv d, const std::string &n = "") {
    m_.dom.push_back(d);
    m_.name.push_back(n);
    return (int)m_.dom.size() - 1;
  }
  int boolvar() { return fresh(Itv(0, 1)); }
  int constant(long long c) {
    const int32_t v = (int32_t)std::max<long long>(INT32_MIN, std::min<long long>(INT32_MAX, c));
    auto it = consts_.find(v);
    if (it != consts_.end()) return it->second;
    const int x = fresh(Itv(v, v));
    consts_.emplace(v, x);
    return x;
  }
  void prop(int32_t op, int x, int y, int z) { m_.props.push_back(bytecode_type{(Sig)op, x, y, z}); }
  void meet(int v, long long lb, long long ub) {
    Itv &d = m_.dom[(size_t)v];
    d.lb = (int32_t)std::max<long long>(d.lb, lb);
    d.ub = (int32_t)std::min<long long>(d.ub, ub);
  }

  // a variable holding the value of an integer expression
  bool value(const Expr &e, int &out) {
    switch (e.kind) {
      case Expr::INT:
      case Expr::BOOL: out = constant(e.v); return true;
      case Expr::IDENT: {
        const int v = m_.index_of(e.id);
        if (v >= 0) {
          out = v;
          return true;
        }
        auto p = m_.params.find(e.id);
        if (p != m_.params.end()) {
          out = constant(p->second);
          return true;
        }
        return error("unknown identifier " + e.id);
      }
      case Expr::ACCESS: {
        auto a = m_.var_arrays.find(e.id);
        if (a != m_.var_arrays.end()) {
          if (e.v < 1 || e.v > (long long)a->second.size()) return error("index out of range: " + e.id);
          out = a->second[(size_t)e.v - 1];
          return true;
        }
        auto p = m_.param_arrays.find(e.id);
        if (p != m_.param_arrays.end()) {
          if (e.v < 1 || e.v > (long long)p->second.size()) return error("index out of range: " + e.id);
          out = constant(p->second[(size_t)e.v - 1]);
          return true;
        }
        return error("unknown array " + e.id);
      }
      case Expr::CALL: return call(e, VALUE, out);
      default: return error("not an integer expression");
    }
  }

  bool values(const Expr &e, std::vector<int> &out) {
    if (e.kind == Expr::IDENT) {
      auto a = m_.var_arrays.find(e.id);
      if (a != m_.var_arrays.end()) {
        out = a->second;
        return true;
      }
      auto p = m_.param_arrays.find(e.id);
      if (p != m_.param_arrays.end()) {
        for (long long c : p->second) out.push_back(constant(c));
        return true;
      }
      return error("unknown array " + e.id);
    }
    if (e.kind != Expr::ARRAY) return error("array expected");
    for (const Expr &x : e.args) {
      int v;
      if (!value(x, v)) return false;
      out.push_back(v);
    }
    return true;
  }

  bool ints(const Expr &e, std::vector<long long> &out) {
    if (e.kind == Expr::IDENT) {
      auto p = m_.param_arrays.find(e.id);
      if (p == m_.param_arrays.end()) return error("constant array expected: " + e.id);
      out = p->second;
      return true;
    }
    if (e.kind == Expr::RANGE) {
      for (long long k = e.v; k <= e.hi; ++k) out.push_back(k);
      return true;
    }
    if (e.kind != Expr::ARRAY && e.kind != Expr::SET) return error("constant array expected");
    for (const Expr &x : e.args) {
      if (x.kind == Expr::INT || x.kind == Expr::BOOL) out.push_back(x.v);
      else if (x.kind == Expr::IDENT && m_.params.count(x.id)) out.push_back(m_.params[x.id]);
      else return error("constant expected");
    }
    return true;
  }

  // -x, |x|, sums
  int negate(int x) {
    const int t = fresh(Itv::top());
    prop(ADD, constant(0), t, x);  // 0 = t + x
    return t;
  }
  int sum(const std::vector<int> &xs) {
    if (xs.empty()) return constant(0);
    int s = xs[0];
    for (size_t k = 1; k < xs.size(); ++k) {
      const int t = fresh(Itv::top());
      prop(ADD, t, s, xs[k]);
      s = t;
    }
    return s;
  }
  bool linear(const Expr &cs, const Expr &xs, int &out) {
    std::vector<long long> c;
    std::vector<int> v;
    if (!ints(cs, c) || !values(xs, v)) return false;
    if (c.size() != v.size()) return error("int_lin: coefficient and variable counts differ");
    std::vector<int> terms;
    for (size_t k = 0; k < c.size(); ++k) {
      if (c[k] == 0) continue;
      if (c[k] == 1) terms.push_back(v[k]);
      else if (c[k] == -1) terms.push_back(negate(v[k]));
      else {
        const int t = fresh(Itv::top());
        prop(MUL, t, constant(c[k]), v[k]);
        terms.push_back(t);
      }
    }
    out = sum(terms);
    return true;
  }

  // comparisons: impose (r < 0) or reify into r
  void cmp_le(int a, int b, int r) { prop(LEQ, r < 0 ? constant(1) : r, a, b); }
  void cmp_lt(int a, int b, int r) {
    if (r < 0) return prop(LEQ, constant(0), b, a);
    const int t = boolvar();
    prop(LEQ, t, b, a);
    prop(ADD, constant(1), r, t);  // r = not (b <= a)
  }
  void cmp_eq(int a, int b, int r) { prop(EQ, r < 0 ? constant(1) : r, a, b); }
  void cmp_ne(int a, int b, int r) {
    if (r < 0) return prop(EQ, constant(0), a, b);
    const int t = boolvar();
    prop(EQ, t, a, b);
    prop(ADD, constant(1), r, t);
  }
  // x in S (a constant set): r = max_k (x == s_k), or for a range r = min(lo <= x, x <= hi)
  bool member(int x, const Expr &S, int r) {
    if (S.kind == Expr::RANGE) {
      if (r < 0) {
        restrict(x, S.v, S.hi);
        return true;
      }
      const int a = boolvar(), b = boolvar();
      prop(LEQ, a, constant(S.v), x);
      prop(LEQ, b, x, constant(S.hi));
      prop(MIN, r, a, b);
      return true;
    }
    std::vector<long long> vals;
    if (!ints(S, vals)) return false;
    if (vals.empty()) {
      prop(EQ, r < 0 ? constant(1) : r, constant(0), constant(1));  // false
      return true;
    }
    std::sort(vals.begin(), vals.end());
    vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
    if (r < 0) restrict(x, vals.front(), vals.back());
    std::vector<int> bs;
    for (long long c : vals) {
      const int b = boolvar();
      prop(EQ, b, x, constant(c));
      bs.push_back(b);
    }
    int m = bs[0];
    for (size_t k = 1; k < bs.size(); ++k) {
      const int t = (k + 1 == bs.size() && r >= 0) ? r : boolvar();
      prop(MAX, t, m, bs[k]);
      m = t;
    }
    if (r < 0) cmp_eq(m, constant(1), -1);
    else if (bs.size() == 1) cmp_eq(r, m, -1);
    return true;
  }
  // a unary constraint lo <= x <= hi: met into x's interval (the sub-domain
  // part of a tell, as PIR interprets unary bounds through its VStore,
  // pir.hpp:299-303)
  void restrict(int x, long long lo, long long hi) { meet(x, lo, hi); }

  // element(i, a, x) with a 1-based array of variables
  void element(int i, const std::vector<int> &a, int x, long long lo, long long hi) {
    restrict(i, 1, (long long)a.size());
    restrict(x, lo, hi);
    for (size_t k = 0; k < a.size(); ++k) {
      const int bi = boolvar(), bx = boolvar();
      prop(EQ, bi, i, constant((long long)k + 1));
      prop(EQ, bx, x, a[k]);
      prop(LEQ, constant(1), bi, bx);  // i == k+1 implies x == a[k]
    }
  }

  // A call of the built-in `f(args)`.  r == IMPOSE: a constraint; r == VALUE:
  // an argument -- a boolean function is reified into a fresh 0/1 variable,
  // an integer function gives its value; r >= 0: reified into variable r.
  // `out` is the variable holding the result.
  static constexpr int IMPOSE = -1, VALUE = -2;
  bool call(const Expr &e, int r, int &out) {
    const std::string &f = e.id;
    const std::vector<Expr> &A = e.args;
    auto arity = [&](size_t n) { return A.size() == n ? true : error(f + ": expected " + std::to_string(n) + " arguments"); };
    auto vals = [&](std::initializer_list<int *> outs) {
      size_t k = 0;
      for (int *o : outs)
        if (!value(A[k++], *o)) return false;
      return true;
    };
    const bool reif_form = f.size() > 5 && f.compare(f.size() - 5, 5, "_reif") == 0;
    const std::string g = reif_form ? f.substr(0, f.size() - 5) : f;
    if (reif_form) {
      // f_reif(args..., r): r <=> f(args...)
      if (A.empty()) return error(f + ": no arguments");
      int rr;
      if (!value(A.back(), rr)) return false;
      Expr inner = e;
      inner.id = g;
      inner.args.pop_back();
      int dummy;
      if (!call(inner, rr, dummy)) return false;
      out = rr;
      return true;
    }
    const bool imp_form = f.size() > 4 && f.compare(f.size() - 4, 4, "_imp") == 0;
    if (imp_form) {
      // f_imp(args..., r): r -> f(args...), as r <= (f reified into a fresh 0/1 variable)
      if (A.empty()) return error(f + ": no arguments");
      int rr;
      if (!value(A.back(), rr)) return false;
      Expr inner = e;
      inner.id = f.substr(0, f.size() - 4);
      inner.args.pop_back();
      const int t = boolvar();
      int dummy;
      if (!call(inner, t, dummy)) return false;
      cmp_le(rr, t, -1);
      out = rr;
      return true;
    }
    // boolean functions: the variable they are reified into (-1: imposed)
    auto reified = [&](int &rv) {
      rv = r >= 0 ? r : (r == VALUE ? boolvar() : -1);
      return true;
    };
    int a, b, c;
    if (g == "int_le" || g == "int_lt" || g == "int_ge" || g == "int_gt" || g == "int_eq" || g == "int_ne" ||
        g == "bool_le" || g == "bool_lt" || g == "bool_eq" || g == "bool_ne") {
      if (A.size() == 3 && (g == "bool_eq" || g == "bool_ne")) {  // bool_eq(a, b, r) spelled without _reif
        int rr;
        if (!value(A[2], rr)) return false;
        Expr inner = e;
        inner.args.pop_back();
        return call(inner, rr, out);
      }
      if (!arity(2) || !vals({&a, &b})) return false;
      int rv;
      reified(rv);
      if (g == "int_le" || g == "bool_le") cmp_le(a, b, rv);
      else if (g == "int_lt" || g == "bool_lt") cmp_lt(a, b, rv);
      else if (g == "int_ge") cmp_le(b, a, rv);
      else if (g == "int_gt") cmp_lt(b, a, rv);
      else if (g == "int_eq" || g == "bool_eq") cmp_eq(a, b, rv);
      else cmp_ne(a, b, rv);
      out = rv;
      return true;
    }
    if (g == "int_plus" || g == "int_minus" || g == "int_times" || g == "int_div" || g == "int_tdiv" ||
        g == "int_fdiv" || g == "int_cdiv" || g == "int_ediv" || g == "int_min" || g == "int_max" ||
        g == "int_mod" || g == "int_tmod" || g == "int_fmod" || g == "int_cmod" || g == "int_emod") {
      if (A.size() != 2 && !arity(3)) return false;
      if (!vals({&a, &b})) return false;
      if (A.size() == 3) {
        if (!value(A[2], c)) return false;
      } else {
        c = fresh(Itv::top());
      }
      if (g == "int_plus") prop(ADD, c, a, b);
      else if (g == "int_minus") prop(ADD, a, c, b);
      else if (g == "int_times") prop(MUL, c, a, b);
      else if (g == "int_div" || g == "int_tdiv") prop(TDIV, c, a, b);
      else if (g == "int_fdiv") prop(FDIV, c, a, b);
      else if (g == "int_cdiv") prop(CDIV, c, a, b);
      else if (g == "int_ediv") prop(EDIV, c, a, b);
      else if (g == "int_min") prop(MIN, c, a, b);
      else if (g == "int_max") prop(MAX, c, a, b);
      else {  // modulo: q = a div b, p = q * b, a = p + c
        const int32_t d = (g == "int_mod" || g == "int_tmod") ? TDIV
                          : g == "int_fmod"                   ? FDIV
                          : g == "int_cmod"                   ? CDIV
                                                              : EDIV;
        const int q = fresh(Itv::top()), p = fresh(Itv::top());
        prop(d, q, a, b);
        prop(MUL, p, q, b);
        prop(ADD, a, p, c);
      }
      if (r >= 0) return error(f + " is not a boolean function");
      out = c;
      return true;
    }
    if (g == "int_abs" || g == "int_negate") {
      if (r >= 0) return error(f + " is not a boolean function");
      if (A.size() != 1 && !arity(2)) return false;
      if (!value(A[0], a)) return false;
      if (A.size() == 2) {
        if (!value(A[1], c)) return false;
      } else {
        c = fresh(Itv::top());
      }
      if (g == "int_negate") prop(ADD, constant(0), c, a);
      else prop(MAX, c, a, negate(a));
      out = c;
      return true;
    }
    if (g == "int_lin_eq" || g == "int_lin_ne" || g == "int_lin_le" || g == "int_lin_lt" || g == "int_lin_ge" ||
        g == "bool_lin_eq" || g == "bool_lin_le") {
      if (!arity(3)) return false;
      int s;
      if (!linear(A[0], A[1], s) || !value(A[2], c)) return false;
      int rv;
      reified(rv);
      if (g == "int_lin_eq" || g == "bool_lin_eq") cmp_eq(s, c, rv);
      else if (g == "int_lin_ne") cmp_ne(s, c, rv);
      else if (g == "int_lin_le" || g == "bool_lin_le") cmp_le(s, c, rv);
      else if (g == "int_lin_lt") cmp_lt(s, c, rv);
      else cmp_le(c, s, rv);
      out = rv;
      return true;
    }
    if (g == "bool_not") {
      if (A.size() == 1) {  // not(a) as a formula: true iff a is 0
        if (!value(A[0], a)) return false;
        int rv;
        reified(rv);
        if (rv < 0) cmp_eq(a, constant(0), -1);
        else prop(ADD, constant(1), a, rv);
        out = rv < 0 ? a : rv;
        return true;
      }
      if (!arity(2) || !vals({&a, &b})) return false;
      if (r != IMPOSE) {  // r <=> (b == not a) <=> (a != b)
        int rv;
        reified(rv);
        cmp_ne(a, b, rv);
        out = rv;
        return true;
      }
      prop(ADD, constant(1), a, b);
      out = b;
      return true;
    }
    if (g == "bool_and" || g == "bool_or" || g == "bool_xor") {
      if (A.size() == 3) {  // bool_and(a, b, r): r <=> a op b
        int rr;
        if (!value(A[2], rr)) return false;
        Expr inner = e;
        inner.args.pop_back();
        return call(inner, rr, out);
      }
      if (!arity(2) || !vals({&a, &b})) return false;
      if (g == "bool_xor") {
        int rv;
        reified(rv);
        cmp_ne(a, b, rv);
        out = rv;
        return true;
      }
      int rv;
      reified(rv);
      const int t = rv >= 0 ? rv : boolvar();
      prop(g == "bool_and" ? MIN : MAX, t, a, b);
      if (rv < 0) cmp_eq(t, constant(1), -1);
      out = t;
      return true;
    }
    if (g == "array_int_maximum" || g == "array_int_minimum") {
      // m = max (min) of xs: a chain of MAX (MIN) ending in m
      if (r >= 0) return error(f + " is not a boolean function");
      if (!arity(2)) return false;
      int m;
      std::vector<int> xs;
      if (!value(A[0], m) || !values(A[1], xs)) return false;
      if (xs.empty()) return error(f + ": empty array");
      const int32_t op = g == "array_int_maximum" ? MAX : MIN;
      if (xs.size() == 1) cmp_eq(m, xs[0], -1);
      int acc = xs[0];
      for (size_t k = 1; k < xs.size(); ++k) {
        const int t = k + 1 == xs.size() ? m : fresh(Itv::top());
        prop(op, t, acc, xs[k]);
        acc = t;
      }
      out = m;
      return true;
    }
    if (g == "fzn_all_different_int" || g == "all_different_int") {
      // pairwise x_i != x_j (left to the solver by MiniZinc when it declares the predicate)
      if (r != IMPOSE) return error(f + " cannot be reified");
      std::vector<int> xs;
      if (!arity(1) || !values(A[0], xs)) return false;
      for (size_t i = 0; i < xs.size(); ++i)
        for (size_t j = i + 1; j < xs.size(); ++j) cmp_ne(xs[i], xs[j], -1);
      out = -1;
      return true;
    }
    if (g == "array_bool_xor") {
      // odd parity: p_k = (p_{k-1} != x_k)
      std::vector<int> xs;
      if (!arity(1) || !values(A[0], xs)) return false;
      int rv;
      reified(rv);
      int p = xs.empty() ? constant(0) : xs[0];
      for (size_t k = 1; k < xs.size(); ++k) {
        const int t = boolvar();
        cmp_ne(p, xs[k], t);
        p = t;
      }
      if (rv >= 0) {
        cmp_eq(rv, p, -1);
        out = rv;
      } else {
        cmp_eq(p, constant(1), -1);
        out = p;
      }
      return true;
    }
    if (g == "array_bool_and" || g == "array_bool_or") {
      std::vector<int> xs;
      if (A.empty() || !values(A[0], xs)) return false;
      int rr;
      reified(rr);
      if (A.size() == 2 && !value(A[1], rr)) return false;
      if (xs.empty()) xs.push_back(constant(g == "array_bool_and" ? 1 : 0));
      int m = xs[0];
      for (size_t k = 1; k < xs.size(); ++k) {
        const int t = boolvar();
        prop(g == "array_bool_and" ? MIN : MAX, t, m, xs[k]);
        m = t;
      }
      if (rr >= 0) {
        cmp_eq(rr, m, -1);
        out = rr;
      } else {
        cmp_eq(m, constant(1), -1);
        out = m;
      }
      return true;
    }
    if (g == "bool_clause") {
      std::vector<int> pos, neg;
      if (!arity(2) || !values(A[0], pos) || !values(A[1], neg)) return false;
      std::vector<int> lits = pos;
      for (int x : neg) {
        const int t = boolvar();
        prop(ADD, constant(1), t, x);  // t = not x
        lits.push_back(t);
      }
      if (lits.empty()) lits.push_back(constant(0));
      int m = lits[0];
      for (size_t k = 1; k < lits.size(); ++k) {
        const int t = boolvar();
        prop(MAX, t, m, lits[k]);
        m = t;
      }
      int rv;
      reified(rv);
      if (rv >= 0) {
        cmp_eq(rv, m, -1);
        out = rv;
      } else {
        cmp_eq(m, constant(1), -1);
        out = m;
      }
      return true;
    }
    if (g == "bool2int") {
      if (r >= 0) return error(f + " cannot be reified");
      if (A.size() == 1) {
        if (!value(A[0], a)) return false;
        out = a;
        return true;
      }
      if (!arity(2) || !vals({&a, &b})) return false;
      prop(EQ, constant(1), a, b);
      out = b;
      return true;
    }
    if (g == "set_in") {
      if (A.size() == 3) {
        int rr;
        if (!value(A[2], rr)) return false;
        Expr inner = e;
        inner.args.pop_back();
        return call(inner, rr, out);
      }
      if (!arity(2) || !value(A[0], a)) return false;
      int rv;
      reified(rv);
      if (!member(a, A[1], rv)) return false;
      out = rv < 0 ? a : rv;
      return true;
    }
    if (g == "array_int_element" || g == "array_var_int_element" || g == "array_bool_element" ||
        g == "array_var_bool_element") {
      if (r >= 0) return error(f + " cannot be reified");
      if (!arity(3)) return false;
      int i, x;
      std::vector<int> arr;
      if (!value(A[0], i) || !values(A[1], arr) || !value(A[2], x)) return false;
      if (arr.empty()) return error(f + ": empty array");
      long long lo = LLONG_MAX, hi = LLONG_MIN;
      for (int v : arr) {
        lo = std::min<long long>(lo, m_.dom[(size_t)v].lb);
        hi = std::max<long long>(hi, m_.dom[(size_t)v].ub);
      }
      element(i, arr, x, lo, hi);
      out = x;
      return true;
    }
    return error("unsupported constraint " + f);
  }

  // declarations ------------------------------------------------------------
  bool domain_of(const Expr &t, Itv &d, std::vector<long long> *set) {
    if (t.kind == Expr::IDENT && (t.id == "int")) {
      d = Itv::top();
      return true;
    }
    if (t.kind == Expr::IDENT && t.id == "bool") {
      d = Itv(0, 1);
      return true;
    }
    if (t.kind == Expr::RANGE) {
      d = Itv((int32_t)t.v, (int32_t)t.hi);
      return true;
    }
    if (t.kind == Expr::SET) {
      std::vector<long long> v;
      if (!ints(t, v) || v.empty()) return error("empty set domain");
      d = Itv((int32_t)*std::min_element(v.begin(), v.end()), (int32_t)*std::max_element(v.begin(), v.end()));
      if (set) *set = v;
      return true;
    }
    return error("unsupported type");
  }

  Model &m_;
  IDiagnostics &d_;
  std::map<int32_t, int> consts_;
};

}  // namespace detail

// Parses and compiles `text` into `m` (which may already hold variables, so
// that later constraints refer to them).  False with messages in `diag` on an
// error.
inline bool compile(const std::string &text, Model &m, IDiagnostics &diag) {
  detail::Parser P(text);
  detail::Compiler C(m, diag);
  auto declare = [&](const std::string &name, Itv d) {
    const int v = C.fresh(d, name);
    m.var_index[name] = v;
    return v;
  };
  while (!P.eof()) {
    std::string kw;
    if (P.accept("constraint")) {
      detail::Expr e;
      if (!P.expr(e)) break;
      P.annotations();
      if (!P.expect(";")) break;
      int out;
      if (e.kind != detail::Expr::CALL) return C.error("constraint: a call is expected");
      if (!C.call(e, -1, out)) return false;
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
      // array [1..n] of [var] T: name [ann] = [ ... ];
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
        if (!C.values(init, vars)) return false;
      } else {
        Itv d;
        std::vector<long long> set;
        if (!C.domain_of(t, d, &set)) return false;
        for (long long k = 0; k < n; ++k) {
          const int v = declare(name + "[" + std::to_string(k + 1) + "]", d);
          if (!set.empty()) {
            detail::Expr S = t;
            if (!C.member(v, S, -1)) return false;
          }
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
      const int v = declare(name, d);
      if (!set.empty() && !C.member(v, t, -1)) return false;
      if (P.accept("=")) {
        detail::Expr init;
        if (!P.expr(init)) break;
        int w;
        if (!C.value(init, w)) return false;
        C.cmp_eq(v, w, -1);
      }
      if (!P.expect(";")) break;
      continue;
    }
    // parameter: int: n = 5;  bool: b = true;
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

// create_and_interpret_and_tell of lala-pc's tests (tests/pir_test.cpp): a
// PIR holding the model's variables and propagators.
inline std::unique_ptr<PIR> make_pir(const Model &m, int device = 0) {
  std::unique_ptr<PIR> pir(new PIR(m.dom, device));
  PIR::tell_type t;
  t.bytecodes = m.props;
  pir->deduce(t);
  return pir;
}

// A later tell of more FlatZinc into an existing PIR (interpret_must_succeed
// in lala-pc's tests): the constraints are compiled against the model, new
// variables are appended to the store, the intervals of existing variables
// are met with what the constraints restricted, and the new propagators are
// told (pir.hpp:326-352).  Returns has_changed, like deduce(tell).
inline bool interpret_and_tell(PIR &pir, Model &m, const std::string &text, IDiagnostics &diag) {
  const size_t nv0 = m.dom.size(), np0 = m.props.size();
  const std::vector<Itv> before(m.dom);
  if (!compile(text, m, diag)) return false;
  bool changed = false;
  if (m.dom.size() > nv0) {
    std::vector<Itv> cur;
    pir.extract(cur);
    cur.insert(cur.end(), m.dom.begin() + (long)nv0, m.dom.end());
    std::vector<int32_t> lb(cur.size()), ub(cur.size());
    for (size_t v = 0; v < cur.size(); ++v) {
      lb[v] = cur[v].lb;
      ub[v] = cur[v].ub;
    }
    if (pir_load_store(pir.ctx(), (int32_t)cur.size(), lb.data(), ub.data()) != PIR_OK)
      throw std::runtime_error("pirgpu: cannot grow the store");
    changed = true;
  }
  PIR::tell_type t;
  for (size_t v = 0; v < nv0; ++v)
    if (m.dom[v] != before[v]) t.sub_value.emplace_back((int32_t)v, m.dom[v]);
  t.bytecodes.assign(m.props.begin() + (long)np0, m.props.end());
  changed |= pir.deduce(t);
  return changed;
}

}  // namespace fzn
}  // namespace lala_gpu

#endif
