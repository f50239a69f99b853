// Known-answer cases of lala-pc's tests/pir_test.cpp written against the
// lala_gpu::PIR facade (include/pirgpu.hpp), the way the reference's tests use
// lala::PIR: interpret_tell, deduce(tell), then the fixpoint, then operator[]
// and is_extractable.  Exit code 0 iff every expectation holds.
#include <cstdio>
#include <vector>

#include "pirgpu.hpp"
#include "pirgpu_fzn.hpp"
#include "pirgpu_fzn_pc.hpp"
#include "pirgpu_pc.hpp"

using namespace lala_gpu;

static int failures = 0;
#define EXPECT(cond)                                                    \
  do {                                                                  \
    if (!(cond)) {                                                      \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);       \
      ++failures;                                                       \
    }                                                                   \
  } while (0)

static void tell(PIR &pir, const Formula &f) {
  IDiagnostics d;
  PIR::tell_type t;
  EXPECT(pir.interpret_tell(f, t, d));
  pir.deduce(t);
}

// tests/pir_test.cpp:175-182: x, y in [0, 10], z = 5, x + y = z.
static void ternary_problem() {
  PIR pir(std::vector<Itv>{Itv(0, 10), Itv(0, 10), Itv(5, 5)});
  tell(pir, Formula::ternary(2, Sig::ADD, 0, 1));
  EXPECT(pir.num_deductions() == 1);
  EXPECT(pir[0] == Itv(0, 10));
  EXPECT(pir.fixpoint() == PIR_OK);
  EXPECT(pir[0] == Itv(0, 5));
  EXPECT(pir[1] == Itv(0, 5));
  EXPECT(pir[2] == Itv(5, 5));
  EXPECT(!pir.is_extractable());
}

// tests/pir_test.cpp:321-329: x, y, z in [3, 10], x + y + z <= 8 fails.
static void top_prop() {
  PIR pir(std::vector<Itv>{Itv(3, 10), Itv(3, 10), Itv(3, 10), Itv::top(), Itv(INT32_MIN, 8)});
  tell(pir, Formula::ternary(3, Sig::ADD, 0, 1));
  tell(pir, Formula::ternary(4, Sig::ADD, 3, 2));
  EXPECT(pir.num_deductions() == 2);
  EXPECT(pir.fixpoint() == PIR_FAILED);
  EXPECT(pir.is_bot());
}

// tests/pir_test.cpp:936-946: b = (x <= 5); then b = 0 gives x >= 6.
static void infinite_domain2() {
  PIR pir(std::vector<Itv>{Itv::top(), Itv::top(), Itv(5, 5)});  // x, b, the constant 5
  tell(pir, Formula::ternary(1, Sig::LEQ, 0, 2));
  EXPECT(pir[1] == Itv(0, 1));  // reified target forced to [0, 1] at install
  EXPECT(pir.fixpoint() == PIR_OK);
  EXPECT(pir[0] == Itv::top());
  tell(pir, Formula::bound(1, Formula::EQ_CONST, 0));
  EXPECT(pir.fixpoint() == PIR_OK);
  EXPECT(pir[0] == Itv(6, INT32_MAX));
  EXPECT(pir.is_extractable());
}

// tests/pir_test.cpp:625-640: min(x, y) = z with incremental tells.
static void min_constraint1() {
  PIR pir(std::vector<Itv>{Itv(0, 4), Itv(2, 5), Itv(0, 10)});
  tell(pir, Formula::ternary(2, Sig::MIN, 0, 1));
  pir.fixpoint();
  EXPECT(pir[2] == Itv(0, 4));
  tell(pir, Formula::bound(2, Formula::LEQ_CONST, 3));
  pir.fixpoint();
  EXPECT(pir[0] == Itv(0, 4) && pir[1] == Itv(2, 5) && pir[2] == Itv(0, 3));
  tell(pir, Formula::bound(0, Formula::LEQ_CONST, 1));
  pir.fixpoint();
  EXPECT(pir[2] == Itv(0, 1));
  tell(pir, Formula::bound(0, Formula::LEQ_CONST, 0));
  pir.fixpoint();
  EXPECT(pir[2] == Itv(0, 0));
  EXPECT(pir.is_extractable());
}

// tests/pir_test.cpp:895-903: x = y tdiv z with x in [2,10], y in [-25,25], z in [-2,3].
static void int_tdiv1() {
  PIR pir(std::vector<Itv>{Itv(2, 10), Itv(-25, 25), Itv(-2, 3)});
  tell(pir, Formula::ternary(0, Sig::TDIV, 1, 2));
  pir.fixpoint();
  EXPECT(pir[1] == Itv(-21, 25));
}

// The snapshot / embed / fixpoint / restore loop of
// tests/bound_consistency_test.hpp:162-196 on int_times over [-3, 3].
static void snapshot_loop() {
  PIR pir(std::vector<Itv>{Itv(-3, 3), Itv(-3, 3), Itv(-3, 3)});
  tell(pir, Formula::ternary(0, Sig::MUL, 1, 2));
  auto snap = pir.snapshot();
  int checked = 0;
  for (int yl = -3; yl <= 3; ++yl)
    for (int zl = -3; zl <= 3; zl += 2) {
      pir.restore(snap);
      pir.embed(1, Itv(yl, yl));
      pir.embed(2, Itv(zl, zl));
      EXPECT(pir.fixpoint() == (yl * zl >= -3 && yl * zl <= 3 ? PIR_OK : PIR_FAILED));
      if (!pir.is_bot()) {
        EXPECT(pir[0] == Itv(yl * zl, yl * zl));
        EXPECT(pir.is_extractable());
      }
      ++checked;
    }
  pir.restore(snap);
  EXPECT(pir[1] == Itv(-3, 3));
  EXPECT(checked == 28);
}

// deduce(i) driven the way the reference tests drive it (a Gauss-Seidel loop
// over i) reaches the fixpoint the GPU driver reaches.
static void gauss_seidel_drop_in() {
  std::vector<Itv> store{Itv(0, 10), Itv(0, 10), Itv(INT32_MIN, 5), Itv(-4, 3), Itv(2, 2), Itv::top()};
  PIR a(store), b(store);
  for (PIR *p : {&a, &b}) {
    tell(*p, Formula::ternary(2, Sig::ADD, 0, 1));
    tell(*p, Formula::ternary(5, Sig::MUL, 3, 4));
    tell(*p, Formula::ternary(0, Sig::MAX, 3, 4));
  }
  bool changed = true;
  while (changed) {
    changed = false;
    for (int64_t i = 0; i < a.num_deductions(); ++i) changed |= a.deduce(i);
  }
  EXPECT(b.fixpoint() == PIR_OK);
  for (int v = 0; v < 6; ++v) EXPECT(a[v] == b[v]);
}

// Interpretation errors go to IDiagnostics (pir.hpp:282-286).
static void interpretation_error() {
  PIR pir(3);
  IDiagnostics d;
  PIR::tell_type t;
  EXPECT(!pir.interpret_tell(Formula::ternary(0, Sig::ADD, 1, 7), t, d));
  EXPECT(d.has_error());
  EXPECT(t.bytecodes.empty());
}

// 6 queens through the facade: 4 solutions (the search driver around PIR).
static void queens6() {
  const int n = 6;
  std::vector<Itv> dom;
  for (int i = 0; i < n; ++i) dom.push_back(Itv(0, n - 1));
  std::vector<std::pair<int, int>> pairs;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) pairs.emplace_back(i, j);
  for (size_t t = 0; t < pairs.size(); ++t) dom.push_back(Itv(-(n - 1), n - 1));  // d_ij
  const int c0 = (int)dom.size();
  for (int k = -(n - 1); k < n; ++k) dom.push_back(Itv(k, k));
  const int f = (int)dom.size();
  dom.push_back(Itv(0, 0));
  PIR pir(dom);
  for (size_t t = 0; t < pairs.size(); ++t) {
    const int i = pairs[t].first, j = pairs[t].second, d = n + (int)t;
    tell(pir, Formula::ternary(i, Sig::ADD, d, j));
    for (int k : {0, j - i, i - j}) tell(pir, Formula::ternary(f, Sig::EQ, d, c0 + k + n - 1));
  }
  std::vector<int32_t> dec;
  for (int i = 0; i < n; ++i) dec.push_back(i);
  pir_search_opts o{};
  o.max_solutions = 10;
  PIR::search_result r = pir.search(dec, o);
  EXPECT(r.status == PIR_OK);
  EXPECT(r.stats.solutions == 4);
  EXPECT(r.solutions.size() == 4);
}

// The element constraint through the FlatZinc front end, told in three steps
// (the user variables' bounds of tests/pir_test.cpp:569-582).
static void element_fzn() {
  fzn::Model m;
  IDiagnostics d;
  EXPECT(fzn::compile("array [1..3] of int: a = [10, 11, 12]; var 1..3: b; var 10..12: c;"
                      " constraint array_int_element(b, a, c);",
                      m, d));
  std::unique_ptr<PIR> pir = fzn::make_pir(m);
  const int b = m.index_of("b"), c = m.index_of("c");
  EXPECT(pir->fixpoint() == PIR_OK);
  EXPECT((*pir)[b] == Itv(1, 3) && (*pir)[c] == Itv(10, 12));
  EXPECT(fzn::interpret_and_tell(*pir, m, "constraint int_le(c, 11);", d));
  EXPECT(pir->fixpoint() == PIR_OK);
  EXPECT((*pir)[b] == Itv(1, 2) && (*pir)[c] == Itv(10, 11));
  fzn::interpret_and_tell(*pir, m, "var 0..1: fresh; constraint int_ge(c, 11); constraint int_le(fresh, 0);", d);
  EXPECT(pir->fixpoint() == PIR_OK);
  EXPECT((*pir)[b] == Itv(2, 2) && (*pir)[c] == Itv(11, 11));
  EXPECT((*pir)[m.index_of("fresh")] == Itv(0, 0));
  EXPECT(pir->is_extractable());
  EXPECT(!d.has_error());
}

// ---- PC (lala_gpu::PC, include/pirgpu_pc.hpp) ----

// tests/pc_test.cpp:132-139 written with the term / formula factories:
// x, y in [0, 10], x + y <= 5.
static void pc_temporal_constraint1() {
  using T = pc::Term;
  using F = pc::Formula;
  PC ipc(std::vector<Itv>{Itv(0, 10), Itv(0, 10)});
  IDiagnostics d;
  PC::tell_type t;
  EXPECT(ipc.interpret_tell(F::make_leq(T::make_add(T::make_var(0), T::make_var(1)), T::make_constant(Itv(5, 5))), t, d));
  EXPECT(ipc.interpret_tell(F::make_leq(T::make_var(0), T::make_constant(Itv(4, 4))), t, d));  // a store bound
  EXPECT(ipc.deduce(t));
  EXPECT(ipc.num_deductions() == 1);
  EXPECT(ipc.fixpoint() == PIR_OK);
  EXPECT(ipc[0] == Itv(0, 4) && ipc[1] == Itv(0, 5));
  EXPECT(!ipc.is_extractable());
}

// tests/pc_test.cpp:360-371 through the FlatZinc front end, in two tells.
static void pc_resource_constraint1() {
  fzn::PcModel m;
  IDiagnostics d;
  EXPECT(fzn::compile_pc("var int: x; var int: y; var int: b; constraint int_ge(x, 5); constraint int_le(x, 10);"
                         " constraint int_ge(y, 9); constraint int_le(y, 15); constraint int_ge(b, 0);"
                         " constraint int_le(b, 1); constraint int_eq(b, bool_and(int_le(int_minus(x, y), 0),"
                         " int_le(int_minus(y, x), 2)));",
                         m, d));
  std::unique_ptr<PC> ipc = fzn::make_pc(m);
  EXPECT(ipc->num_deductions() == 1);
  EXPECT(ipc->fixpoint() == PIR_OK);
  EXPECT((*ipc)[0] == Itv(5, 10) && (*ipc)[1] == Itv(9, 15));
  EXPECT(fzn::interpret_and_tell(*ipc, m, "constraint int_eq(b, 1);", d));
  EXPECT(ipc->fixpoint() == PIR_OK);
  EXPECT((*ipc)[0] == Itv(7, 10) && (*ipc)[1] == Itv(9, 12) && (*ipc)[2] == Itv(1, 1));
  EXPECT(!d.has_error());
}

// The reference's loop GaussSeidelIteration{}.fixpoint(num_deductions(),
// deduce) (tests/pc_test.cpp:91-94) over deduce(i), against fixpoint(); and
// snapshot / restore around a tell.
static void pc_drop_in_and_snapshot() {
  fzn::PcModel m;
  IDiagnostics d;
  EXPECT(fzn::compile_pc("var 0..4: x; var 2..5: y; var 0..10: z; constraint int_min(x, y, z);"
                         " constraint int_le(z, 3); constraint int_ne(x, 0);",
                         m, d));
  std::unique_ptr<PC> a = fzn::make_pc(m), b = fzn::make_pc(m);
  bool changed = true;
  while (changed) {
    changed = false;
    for (int64_t i = 0; i < a->num_deductions(); ++i) changed |= a->deduce(i);
  }
  EXPECT(b->fixpoint() == PIR_OK);
  for (int v = 0; v < 3; ++v) EXPECT((*a)[v] == (*b)[v]);
  EXPECT((*b)[0] == Itv(1, 4) && (*b)[2] == Itv(1, 3));
  auto snap = b->snapshot();
  EXPECT(fzn::interpret_and_tell(*b, m, "constraint int_gt(x, y);", d));
  EXPECT(b->num_deductions() == 3);
  EXPECT(b->fixpoint() == PIR_OK);
  EXPECT((*b)[0] == Itv(3, 4) && (*b)[1] == Itv(2, 3));
  // restore pops from the end of the sorted propagators (pc.hpp:717-724): the
  // count and the store come back, the propagator dropped is the last in the
  // (kind, length) order -- here x != 0, not the x > y just told
  b->restore(snap);
  EXPECT(b->num_deductions() == 2);
  EXPECT((*b)[0] == Itv(1, 4));
  EXPECT(!d.has_error());
}

int main() {
  ternary_problem();
  top_prop();
  infinite_domain2();
  min_constraint1();
  int_tdiv1();
  snapshot_loop();
  gauss_seidel_drop_in();
  interpretation_error();
  queens6();
  element_fzn();
  pc_temporal_constraint1();
  pc_resource_constraint1();
  pc_drop_in_and_snapshot();
  std::printf("%d failures\n", failures);
  return failures ? 1 : 0;
}
