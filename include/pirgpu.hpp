// lala_gpu::PIR — C++ facade over the pirgpu C ABI (include/pirgpu.h).
//
// Mirrors the abstract-domain surface of lala-pc's lala::PIR
// (include/lala/pir.hpp:53-942) over a VStore<Interval<ZLB<int>>>, so that code
// written against it switches by changing the type and the fixpoint call:
//
//   interpret_tell / interpret_ask   pir.hpp:315-323 (the X = Y op Z subset of :261-284,
//                                    plus the unary bounds the VStore interprets)
//   deduce(tell), deduce(i)          pir.hpp:326-352, :387-390
//   ask(i), ask(ask_type)            pir.hpp:368-380
//   embed, operator[], project       pir.hpp:354-356, :840-851
//   num_deductions, vars             pir.hpp:382-384, :853-855
//   is_bot, is_top                   pir.hpp:831-838
//   snapshot / restore               pir.hpp:857-870
//   is_extractable / extract         pir.hpp:873-898
//
// and adds fixpoint(), the GPU driver that replaces the caller's
// GaussSeidelIteration{}.fixpoint(num_deductions(), [&](size_t i){ return deduce(i); })
// loop (tests/pir_test.cpp:60-62).  Interpretation failures return false and
// add a message to IDiagnostics, as the reference does; CUDA failures throw
// std::runtime_error.  Header only; link with libpirgpu.so.
#ifndef PIRGPU_HPP
#define PIRGPU_HPP

#include <algorithm>
#include <climits>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pirgpu.h"

namespace lala_gpu {

// Interval<ZLB<int>>: INT32_MIN / INT32_MAX are the infinite bounds.
struct Itv {
  int32_t lb = INT32_MIN, ub = INT32_MAX;
  Itv() = default;
  Itv(int32_t l, int32_t u) : lb(l), ub(u) {}
  static Itv top() { return Itv(INT32_MIN, INT32_MAX); }
  static Itv bot() { return Itv(INT32_MAX, INT32_MIN); }
  bool is_bot() const { return lb > ub || lb == INT32_MAX || ub == INT32_MIN; }
  bool is_top() const { return lb == INT32_MIN && ub == INT32_MAX; }
  bool operator==(const Itv &o) const { return lb == o.lb && ub == o.ub; }
  bool operator!=(const Itv &o) const { return !(*this == o); }
};

// The Sig values PIR accepts (pir.hpp:270-273), numbered as in the C ABI.
enum class Sig : int32_t { ADD = 0, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, EQ, LEQ };

// bytecode_type, pir.hpp:37-47: the propagator X = Y op Z.
struct bytecode_type {
  Sig op;
  int32_t x, y, z;
};

// The formulas the facade interprets: a ternary propagator X = Y op Z
// (pir.hpp:261-284), or a unary bound x <= c, x >= c, x == c (interpreted by
// the sub-domain, as PIR tries the VStore first, pir.hpp:299-303).
struct Formula {
  enum Kind { TERNARY, LEQ_CONST, GEQ_CONST, EQ_CONST } kind = TERNARY;
  Sig op = Sig::ADD;
  int32_t x = -1, y = -1, z = -1;
  int32_t c = 0;
  static Formula ternary(int32_t x, Sig op, int32_t y, int32_t z) {
    Formula f;
    f.kind = TERNARY;
    f.op = op;
    f.x = x;
    f.y = y;
    f.z = z;
    return f;
  }
  static Formula bound(int32_t x, Kind k, int32_t c) {
    Formula f;
    f.kind = k;
    f.x = x;
    f.c = c;
    return f;
  }
};

struct IDiagnostics {
  std::vector<std::string> errors;
  bool has_error() const { return !errors.empty(); }
};

class PIR {
 public:
  // interpreted_type (pir.hpp:124-150): sub-domain meets + bytecodes.
  struct interpreted_type {
    std::vector<std::pair<int32_t, Itv>> sub_value;
    std::vector<bytecode_type> bytecodes;
  };
  using tell_type = interpreted_type;
  using ask_type = interpreted_type;

  struct snapshot_type {
    std::shared_ptr<pirgpu_snapshot> snap;
    int64_t num_bytecodes;
  };

  // A PIR over `nvars` unbounded variables on `device`.
  explicit PIR(int32_t nvars, int device = 0) : PIR(std::vector<Itv>((size_t)nvars, Itv::top()), device) {}

  // A PIR over the given initial store.
  explicit PIR(const std::vector<Itv> &store, int device = 0) {
    pirgpu_ctx *c = nullptr;
    if (pir_ctx_create(&c, device) != PIR_OK) throw std::runtime_error("pirgpu: cannot create a context");
    ctx_.reset(c);
    std::vector<int32_t> lb(store.size()), ub(store.size());
    for (size_t i = 0; i < store.size(); ++i) {
      lb[i] = store[i].lb;
      ub[i] = store[i].ub;
    }
    check(pir_load_store(ctx(), (int32_t)store.size(), lb.data(), ub.data()));
  }

  // pir.hpp:255-287 and :291-311: unary bounds go to the store, X = Y op Z to
  // the bytecode; anything else is an interpretation error.
  bool interpret_tell(const Formula &f, tell_type &tell, IDiagnostics &diagnostics) const {
    return interpret(f, tell, diagnostics);
  }
  bool interpret_ask(const Formula &f, ask_type &ask, IDiagnostics &diagnostics) const {
    return interpret(f, ask, diagnostics);
  }

  // pir.hpp:326-352: meets the sub-domain part, appends the propagators (reified
  // targets forced to [0,1], bytecode re-sorted).  Returns has_changed.
  bool deduce(const tell_type &t) {
    bool changed = false;
    for (const auto &m : t.sub_value) changed |= embed(m.first, m.second);
    if (!t.bytecodes.empty()) {
      std::vector<int32_t> op, x, y, z;
      for (const auto &b : t.bytecodes) {
        op.push_back((int32_t)b.op);
        x.push_back(b.x);
        y.push_back(b.y);
        z.push_back(b.z);
      }
      int ch = 0;
      check(pir_tell(ctx(), (int32_t)op.size(), op.data(), x.data(), y.data(), z.data(), &ch));
      changed |= ch != 0;
    }
    return changed;
  }

  // pir.hpp:387-390: one propagator of the engine order.
  bool deduce(int64_t i) {
    int ch = 0;
    check(pir_deduce_one(ctx(), i, &ch));
    return ch != 0;
  }

  // The GPU fixpoint loop: propagates every propagator until nothing changes.
  // Returns PIR_OK, PIR_FAILED (the store is empty) or PIR_TIMEOUT.
  pir_status fixpoint(const pir_opts *opts = nullptr, pir_stats *stats = nullptr) {
    const int rc = pir_fixpoint(ctx(), opts, stats);
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
    check(pir_ask(ctx(), i, &e));
    return e != 0;
  }

  // pir.hpp:372-380: every propagator of `a` entailed and every bound of its
  // sub-domain part entailed by the store.
  bool ask(const ask_type &a) const {
    for (const auto &m : a.sub_value) {
      const Itv v = (*this)[m.first];
      if (!(v.lb >= m.second.lb && v.ub <= m.second.ub)) return false;
    }
    if (a.bytecodes.empty()) return true;
    std::vector<int32_t> op, x, y, z;
    for (const auto &b : a.bytecodes) {
      op.push_back((int32_t)b.op);
      x.push_back(b.x);
      y.push_back(b.y);
      z.push_back(b.z);
    }
    std::vector<uint8_t> e(op.size());
    check(pir_ask_bytecodes(ctx(), (int32_t)op.size(), op.data(), x.data(), y.data(), z.data(), e.data()));
    for (uint8_t v : e)
      if (!v) return false;
    return true;
  }

  int64_t num_deductions() const { return pir_num_deductions(ctx()); }
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
  bool is_top() const {
    int t = 0;
    check(pir_is_top(ctx(), &t));
    return t != 0;
  }

  snapshot_type snapshot() const {
    pirgpu_snapshot *s = nullptr;
    check(pir_snapshot(ctx(), &s));
    return snapshot_type{std::shared_ptr<pirgpu_snapshot>(s, pir_snapshot_free), num_deductions()};
  }
  void restore(const snapshot_type &s) { check(pir_restore(ctx(), s.snap.get())); }

  bool is_extractable() const {
    int e = 0;
    check(pir_is_extractable(ctx(), &e));
    return e != 0;
  }
  // pir.hpp:891-898: copies the store out (the propagators are entailed).
  void extract(std::vector<Itv> &ua) const {
    const int32_t n = vars();
    std::vector<int32_t> lb((size_t)n), ub((size_t)n);
    check(pir_read_store(ctx(), lb.data(), ub.data()));
    ua.resize((size_t)n);
    for (int32_t i = 0; i < n; ++i) ua[(size_t)i] = Itv(lb[(size_t)i], ub[(size_t)i]);
  }

  // Depth-first search over the decision variables `dec` (pir_search): the
  // branch / propagate / restore loop a solver runs around PIR
  // (pir.hpp:857-870), children propagated in batches on the GPU.  Keeps at
  // most opts.max_solutions solutions (0: counts them only).
  struct search_result {
    pir_status status;
    std::vector<std::vector<int32_t>> solutions;
    pir_search_stats stats;
  };
  search_result search(const std::vector<int32_t> &dec, const pir_search_opts &opts) {
    search_result res;
    std::vector<int32_t> buf((size_t)std::max<int64_t>(opts.max_solutions, 1) * dec.size());
    const int rc = pir_search(ctx(), (int32_t)dec.size(), dec.data(), &opts, buf.data(), &res.stats);
    if (rc != PIR_OK && rc != PIR_TIMEOUT) fail(rc);
    res.status = (pir_status)res.stats.status;
    const int64_t kept = opts.max_solutions > 0 ? res.stats.solutions : 0;
    for (int64_t k = 0; k < kept; ++k)
      res.solutions.emplace_back(buf.begin() + (size_t)k * dec.size(), buf.begin() + (size_t)(k + 1) * dec.size());
    return res;
  }

  pirgpu_ctx *ctx() const { return ctx_.get(); }

 private:
  struct Deleter {
    void operator()(pirgpu_ctx *c) const { pir_ctx_destroy(c); }
  };
  std::unique_ptr<pirgpu_ctx, Deleter> ctx_;

  void check(int rc) const {
    if (rc != PIR_OK) fail(rc);
  }
  [[noreturn]] void fail(int rc) const {
    throw std::runtime_error(std::string("pirgpu error ") + std::to_string(rc) + ": " + pir_last_error(ctx()));
  }

  bool interpret(const Formula &f, interpreted_type &out, IDiagnostics &diagnostics) const {
    const int32_t n = vars();
    auto bad = [&](int32_t v) { return v < 0 || v >= n; };
    switch (f.kind) {
      case Formula::LEQ_CONST:
      case Formula::GEQ_CONST:
      case Formula::EQ_CONST: {
        if (bad(f.x)) {
          diagnostics.errors.push_back("Could not interpret the variables in the environment.");
          return false;
        }
        Itv d = Itv::top();
        if (f.kind != Formula::GEQ_CONST) d.ub = f.c;
        if (f.kind != Formula::LEQ_CONST) d.lb = f.c;
        out.sub_value.emplace_back(f.x, d);
        return true;
      }
      case Formula::TERNARY: {
        const int32_t op = (int32_t)f.op;
        if (op < 0 || op > (int32_t)Sig::LEQ) {
          diagnostics.errors.push_back("The shape of this formula is not supported.");
          return false;
        }
        if (bad(f.x) || bad(f.y) || bad(f.z)) {
          diagnostics.errors.push_back("Could not interpret the variables in the environment.");
          return false;
        }
        out.bytecodes.push_back(bytecode_type{f.op, f.x, f.y, f.z});
        return true;
      }
    }
    diagnostics.errors.push_back("The shape of this formula is not supported.");
    return false;
  }
};

}  // namespace lala_gpu

#endif
