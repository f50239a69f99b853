// lala_gpu::PC — C++ facade of the tree propagators (the pc_* calls of
// include/pirgpu.h).
//
// Mirrors lala-pc's PC abstract domain (include/lala/pc.hpp:39-789) over a
// VStore<Interval<ZLB<int>>>:
//
//   pc::Term / pc::Formula    the trees of terms.hpp / formula.hpp, built with
//                             the reference's factory names (make_var,
//                             make_add, make_leq, make_conj, ...)
//   interpret_tell / _ask     pc.hpp:609-617: a comparison of one variable with
//                             a constant is interpreted by the store (the
//                             sub-domain is tried first, pc.hpp:576-605), any
//                             other formula becomes a propagator
//   deduce(tell), deduce(i)   pc.hpp:625-648, :671-681
//   ask(i), ask(ask_type)     pc.hpp:652-663
//   num_deductions, vars      pc.hpp:665-667, :707-709
//   embed, operator[], project, is_bot, is_top     pc.hpp:647-649, :685-705
//   snapshot / restore        pc.hpp:712-724
//   is_extractable / extract  pc.hpp:727-752
//
// plus fixpoint(), the GPU driver that replaces the tests'
// GaussSeidelIteration{}.fixpoint(num_deductions(), deduce) loop
// (tests/pc_test.cpp:91-94).  Header only; link with libpirgpu.so.
#ifndef PIRGPU_PC_HPP
#define PIRGPU_PC_HPP

#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "pirgpu.hpp"

namespace lala_gpu {
namespace pc {

// One node of a term or formula tree: kind (enum pc_kind), the node's own
// data (variable, constant bounds) and its children.
struct Node {
  int32_t kind = PC_TRUE;
  int32_t a = 0, b = 0, c = 0;
  std::vector<std::shared_ptr<const Node>> kids;
};
using NodePtr = std::shared_ptr<const Node>;

inline NodePtr make_node(int32_t kind, std::vector<NodePtr> kids = {}, int32_t a = 0, int32_t b = 0) {
  auto n = std::make_shared<Node>();
  n->kind = kind;
  n->a = a;
  n->b = b;
  n->kids = std::move(kids);
  return n;
}

class Formula;

// Term (terms.hpp:528-760)
class Term {
 public:
  Term() = default;
  explicit Term(NodePtr n) : n_(std::move(n)) {}
  static Term make_var(int32_t x) { return Term(make_node(PC_VAR, {}, x)); }
  static Term make_constant(Itv k) { return Term(make_node(PC_CONST, {}, k.lb, k.ub)); }
  static Term make_formula(const Formula &f);
  static Term make_neg(const Term &t) { return un(PC_NEG, t); }
  static Term make_abs(const Term &t) { return un(PC_ABS, t); }
  static Term make_add(const Term &x, const Term &y) { return bin(PC_ADD, x, y); }
  static Term make_sub(const Term &x, const Term &y) { return bin(PC_SUB, x, y); }
  static Term make_mul(const Term &x, const Term &y) { return bin(PC_MUL, x, y); }
  static Term make_tdiv(const Term &x, const Term &y) { return bin(PC_TDIV, x, y); }
  static Term make_fdiv(const Term &x, const Term &y) { return bin(PC_FDIV, x, y); }
  static Term make_cdiv(const Term &x, const Term &y) { return bin(PC_CDIV, x, y); }
  static Term make_ediv(const Term &x, const Term &y) { return bin(PC_EDIV, x, y); }
  static Term make_min(const Term &x, const Term &y) { return bin(PC_MIN, x, y); }
  static Term make_max(const Term &x, const Term &y) { return bin(PC_MAX, x, y); }
  static Term make_naryadd(const std::vector<Term> &ts) { return nary(PC_NADD, ts); }
  static Term make_narymul(const std::vector<Term> &ts) { return nary(PC_NMUL, ts); }

  bool is(int32_t kind) const { return n_ && n_->kind == kind; }
  const NodePtr &node() const { return n_; }

 private:
  NodePtr n_;
  static Term un(int32_t k, const Term &t) { return Term(make_node(k, {t.n_})); }
  static Term bin(int32_t k, const Term &x, const Term &y) { return Term(make_node(k, {x.n_, y.n_})); }
  static Term nary(int32_t k, const std::vector<Term> &ts) {
    std::vector<NodePtr> kids;
    for (const Term &t : ts) kids.push_back(t.n_);
    return Term(make_node(k, std::move(kids)));
  }
};

// Formula (formula.hpp:863-1141)
class Formula {
 public:
  Formula() = default;
  explicit Formula(NodePtr n) : n_(std::move(n)) {}
  static Formula make_pvarlit(int32_t x) { return Formula(make_node(PC_PVAR, {}, x)); }
  static Formula make_nvarlit(int32_t x) { return Formula(make_node(PC_NVAR, {}, x)); }
  static Formula make_true() { return Formula(make_node(PC_TRUE)); }
  static Formula make_false() { return Formula(make_node(PC_FALSE)); }
  static Formula make_leq(const Term &l, const Term &r) { return cmp(PC_LEQ, l, r); }
  static Formula make_gt(const Term &l, const Term &r) { return cmp(PC_GT, l, r); }
  static Formula make_eq(const Term &l, const Term &r) { return cmp(PC_EQ, l, r); }
  static Formula make_neq(const Term &l, const Term &r) { return cmp(PC_NEQ, l, r); }
  static Formula make_conj(const Formula &f, const Formula &g) { return con(PC_AND, f, g); }
  static Formula make_disj(const Formula &f, const Formula &g) { return con(PC_OR, f, g); }
  static Formula make_bicond(const Formula &f, const Formula &g) { return con(PC_EQUIV, f, g); }
  static Formula make_imply(const Formula &f, const Formula &g) { return con(PC_IMPLY, f, g); }
  static Formula make_xor(const Formula &f, const Formula &g) { return con(PC_XOR, f, g); }
  // AbstractElement (formula.hpp:14-78): a formula of the store itself, as
  // the store's tell / ask items (variable, interval) of the formula and of
  // its negation
  // (asks of "var != c" miss an interval: the _out lists)
  using items = std::vector<std::pair<int32_t, Itv>>;
  static Formula make_abstract_element(const items &tellv, const items &not_tellv, const items &askv,
                                       const items &not_askv, const items &ask_outv = {},
                                       const items &not_ask_outv = {}) {
    std::vector<NodePtr> kids;
    const std::pair<int32_t, const items *> lists[6] = {
        {PC_TELL, &tellv},        {PC_NTELL, &not_tellv},   {PC_ASK, &askv},
        {PC_NASK, &not_askv},     {PC_ASK_OUT, &ask_outv}, {PC_NASK_OUT, &not_ask_outv}};
    for (const auto &l : lists)
      for (const auto &it : *l.second) {
        auto n = std::make_shared<Node>();
        n->kind = l.first;
        n->a = it.first;
        n->b = it.second.lb;
        n->c = it.second.ub;
        kids.push_back(n);
      }
    return Formula(make_node(PC_AE, std::move(kids)));
  }

  int32_t kind() const { return n_ ? n_->kind : -1; }
  const NodePtr &node() const { return n_; }

 private:
  NodePtr n_;
  static Formula cmp(int32_t k, const Term &l, const Term &r) { return Formula(make_node(k, {l.node(), r.node()})); }
  static Formula con(int32_t k, const Formula &f, const Formula &g) {
    return Formula(make_node(k, {f.node(), g.node()}));
  }
};

inline Term Term::make_formula(const Formula &f) { return Term(make_node(PC_FORMULA, {f.node()})); }

// Flattens trees into the tape format of pc_tell: children first, a node
// shared by several trees is written once.
class TapeWriter {
 public:
  std::vector<int32_t> kind, a, b, c, roots;

  int32_t emit(const NodePtr &n) {
    auto it = seen_.find(n.get());
    if (it != seen_.end()) return it->second;
    int32_t id;
    switch (n->kind) {
      case PC_VAR:
      case PC_PVAR:
      case PC_NVAR:
      case PC_CONST:
      case PC_TRUE:
      case PC_FALSE: id = push(n->kind, n->a, n->b); break;
      case PC_FORMULA:
      case PC_NEG:
      case PC_ABS: id = push(n->kind, emit(n->kids.at(0)), 0); break;
      case PC_NADD:
      case PC_NMUL: {
        std::vector<int32_t> ops;
        for (const NodePtr &k : n->kids) ops.push_back(emit(k));
        const int32_t first = (int32_t)kind.size();
        for (int32_t o : ops) push(PC_ARG, o, 0);
        id = push(n->kind, first, (int32_t)ops.size());
        break;
      }
      case PC_AE: {
        const int32_t first = (int32_t)kind.size();
        for (const NodePtr &k : n->kids) push(k->kind, k->a, k->b, k->c);
        id = push(PC_AE, first, (int32_t)n->kids.size());
        break;
      }
      default: {
        const int32_t x = emit(n->kids.at(0));
        const int32_t y = emit(n->kids.at(1));
        id = push(n->kind, x, y);
      }
    }
    seen_.emplace(n.get(), id);
    return id;
  }
  void prop(const Formula &f) { roots.push_back(emit(f.node())); }

 private:
  std::unordered_map<const Node *, int32_t> seen_;
  int32_t push(int32_t k, int32_t x, int32_t y, int32_t z = 0) {
    kind.push_back(k);
    a.push_back(x);
    b.push_back(y);
    c.push_back(z);
    return (int32_t)kind.size() - 1;
  }
};

}  // namespace pc

class PC {
 public:
  // interpreted_type (pc.hpp:107-130): store meets + propagators
  struct interpreted_type {
    std::vector<std::pair<int32_t, Itv>> sub_value;
    std::vector<pc::Formula> props;
  };
  using tell_type = interpreted_type;
  using ask_type = interpreted_type;

  // snapshot_type (pc.hpp:49-70): the store and the number of propagators
  struct snapshot_type {
    std::shared_ptr<pirgpu_snapshot> snap;
    int64_t num_props;
  };

  explicit PC(int32_t nvars, int device = 0) : PC(std::vector<Itv>((size_t)nvars, Itv::top()), device) {}
  explicit PC(const std::vector<Itv> &store, int device = 0) {
    pirgpu_ctx *c = nullptr;
    if (pir_ctx_create(&c, device) != PIR_OK) throw std::runtime_error("pirgpu: cannot create a context");
    ctx_.reset(c);
    device_ = device;
    load(store);
  }

  // pc.hpp:576-617: a comparison of a variable with a constant goes to the
  // store, anything else becomes a propagator (after its variables were
  // checked).
  bool interpret_tell(const pc::Formula &f, tell_type &tell, IDiagnostics &diagnostics) const {
    return interpret(f, tell, diagnostics);
  }
  bool interpret_ask(const pc::Formula &f, ask_type &ask, IDiagnostics &diagnostics) const {
    return interpret(f, ask, diagnostics);
  }

  // deduce(tell), pc.hpp:625-648
  bool deduce(const tell_type &t) {
    bool changed = false;
    for (const auto &m : t.sub_value) changed |= embed(m.first, m.second);
    if (!t.props.empty()) {
      pc::TapeWriter w;
      for (const pc::Formula &f : t.props) w.prop(f);
      check(pc_tell(ctx(), (int32_t)w.kind.size(), w.kind.data(), w.a.data(), w.b.data(), w.c.data(),
                    (int32_t)w.roots.size(), w.roots.data()));
      changed = true;
    }
    return changed;
  }
  // deduce(int i), pc.hpp:671-681
  bool deduce(int64_t i) {
    int ch = 0;
    check(pc_deduce_one(ctx(), i, &ch));
    return ch != 0;
  }
  pir_status fixpoint(const pir_opts *opts = nullptr, pir_stats *stats = nullptr) {
    const int rc = pc_fixpoint(ctx(), opts, stats);
    if (rc != PIR_OK && rc != PIR_FAILED && rc != PIR_TIMEOUT) fail(rc);
    return (pir_status)rc;
  }
  bool embed(int32_t x, const Itv &dom) {
    int ch = 0;
    check(pir_embed(ctx(), x, dom.lb, dom.ub, &ch));
    return ch != 0;
  }
  bool ask(int64_t i) const {
    int e = 0;
    check(pc_ask(ctx(), i, &e));
    return e != 0;
  }
  // ask(ask_type), pc.hpp:652-659: every propagator of the ask entailed, and
  // every store part included in the store
  bool ask(const ask_type &a) const {
    for (const auto &m : a.sub_value) {
      const Itv v = (*this)[m.first];
      if (!(v.is_bot() || (v.lb >= m.second.lb && v.ub <= m.second.ub))) return false;
    }
    if (a.props.empty()) return true;
    // entailment of formulas that are not told: a scratch context on a copy of the store
    PC tmp(extract_all(), device_);
    tell_type t;
    t.props = a.props;
    tmp.deduce(t);
    for (int64_t i = 0; i < tmp.num_deductions(); ++i)
      if (!tmp.ask(i)) return false;
    return true;
  }

  int64_t num_deductions() const { return pc_num_deductions(ctx()); }
  int32_t vars() const { return pir_vars(ctx()); }
  Itv operator[](int32_t x) const {
    Itv r;
    check(pir_project(ctx(), x, &r.lb, &r.ub));
    return r;
  }
  Itv project(int32_t x) const { return (*this)[x]; }
  bool is_bot() const {
    int b = 0;
    check(pir_is_bot(ctx(), &b));
    return b != 0;
  }
  // is_top(), pc.hpp:690-692: a top store and no propagator
  bool is_top() const {
    if (num_deductions() != 0 || is_bot()) return false;
    for (const Itv &v : extract_all())
      if (!v.is_top()) return false;
    return true;
  }
  snapshot_type snapshot() const {
    pirgpu_snapshot *s = nullptr;
    check(pir_snapshot(ctx(), &s));
    return snapshot_type{std::shared_ptr<pirgpu_snapshot>(s, pir_snapshot_free), num_deductions()};
  }
  void restore(const snapshot_type &s) { check(pir_restore(ctx(), s.snap.get())); }
  bool is_extractable() const {
    int e = 0;
    check(pc_is_extractable(ctx(), &e));
    return e != 0;
  }
  void extract(std::vector<Itv> &ua) const { ua = extract_all(); }

  // grows the store by the given variables (a later tell that declares some)
  void add_vars(const std::vector<Itv> &dom) {
    std::vector<Itv> cur = extract_all();
    cur.insert(cur.end(), dom.begin(), dom.end());
    load(cur);
  }

  pirgpu_ctx *ctx() const { return ctx_.get(); }

 private:
  struct Deleter {
    void operator()(pirgpu_ctx *c) const { pir_ctx_destroy(c); }
  };
  std::unique_ptr<pirgpu_ctx, Deleter> ctx_;
  int device_ = 0;

  void check(int rc) const {
    if (rc != PIR_OK) fail(rc);
  }
  [[noreturn]] void fail(int rc) const {
    throw std::runtime_error(std::string("pirgpu error ") + std::to_string(rc) + ": " + pir_last_error(ctx()));
  }
  void load(const std::vector<Itv> &store) {
    std::vector<int32_t> lb(store.size()), ub(store.size());
    for (size_t i = 0; i < store.size(); ++i) {
      lb[i] = store[i].lb;
      ub[i] = store[i].ub;
    }
    check(pir_load_store(ctx(), (int32_t)store.size(), lb.data(), ub.data()));
  }
  std::vector<Itv> extract_all() const {
    const int32_t n = vars();
    std::vector<int32_t> lb((size_t)n), ub((size_t)n);
    check(pir_read_store(ctx(), lb.data(), ub.data()));
    std::vector<Itv> r((size_t)n);
    for (int32_t i = 0; i < n; ++i) r[(size_t)i] = Itv(lb[(size_t)i], ub[(size_t)i]);
    return r;
  }

  // a comparison var <op> constant as a store part (the VStore interprets
  // it); returns false for any other shape
  static bool as_bound(const pc::Formula &f, int32_t &x, Itv &d) {
    const pc::NodePtr &n = f.node();
    if (!n || n->kids.size() != 2 || n->kind < PC_LEQ || n->kind > PC_EQ) return false;
    const pc::NodePtr &l = n->kids[0], &r = n->kids[1];
    const bool lv = l->kind == PC_VAR, rv = r->kind == PC_VAR;
    const bool lc = l->kind == PC_CONST && l->a == l->b, rc = r->kind == PC_CONST && r->a == r->b;
    if (!((lv && rc) || (lc && rv))) return false;
    x = lv ? l->a : r->a;
    const int64_t k = lv ? r->a : l->a;
    d = Itv::top();
    auto clamp = [](int64_t v) { return (int32_t)std::max<int64_t>(INT32_MIN, std::min<int64_t>(INT32_MAX, v)); };
    switch (n->kind) {
      case PC_LEQ: (lv ? d.ub : d.lb) = clamp(k); break;            // x <= k  /  k <= x
      case PC_GT: (lv ? d.lb : d.ub) = clamp(lv ? k + 1 : k - 1); break;  // x > k  /  k > x
      default: d = Itv(clamp(k), clamp(k));                          // x == k
    }
    return true;
  }

  bool interpret(const pc::Formula &f, interpreted_type &out, IDiagnostics &diagnostics) const {
    if (!f.node()) {
      diagnostics.errors.push_back("Empty formula.");
      return false;
    }
    int32_t x;
    Itv d;
    if (as_bound(f, x, d)) {
      if (x < 0 || x >= vars()) {
        diagnostics.errors.push_back("Could not interpret the variables in the environment.");
        return false;
      }
      out.sub_value.emplace_back(x, d);
      return true;
    }
    // variables in range, terms and formulas where they belong
    std::vector<const pc::Node *> stack{f.node().get()};
    while (!stack.empty()) {
      const pc::Node *n = stack.back();
      stack.pop_back();
      if ((n->kind == PC_VAR || n->kind == PC_PVAR || n->kind == PC_NVAR || (n->kind >= PC_TELL && n->kind <= PC_NASK_OUT)) &&
          (n->a < 0 || n->a >= vars())) {
        diagnostics.errors.push_back("Could not interpret the variables in the environment.");
        return false;
      }
      for (const pc::NodePtr &k : n->kids) stack.push_back(k.get());
    }
    out.props.push_back(f);
    return true;
  }
};

}  // namespace lala_gpu

#endif
