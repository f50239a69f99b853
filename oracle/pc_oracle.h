/* CPU oracle for PC, lala-pc's tree propagators — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this code (it is linked into oracle/_build/liboracle.so next to the PIR
 * oracle).  The product never links or calls it.
 *
 * A plain C++ restatement of lala-pc's PC abstract domain:
 *   terms    include/lala/terms.hpp   (Constant, Variable, Unary NEG/ABS,
 *            Binary over the Group* operator tables, Nary ADD/MUL),
 *   formulas include/lala/formula.hpp (variable literals, true/false,
 *            <=, >, ==, !=, and, or, <=>, =>, xor; formulas used as terms),
 *   domain   include/lala/pc.hpp      (deduce(tell) appends and sorts the
 *            propagators by (kind, length) :625-648, deduce(i) :671,
 *            ask(i) :661, is_extractable :727),
 * and of the Gauss-Seidel loop the reference tests drive it with
 * (tests/pc_test.cpp:85-104).
 *
 * The interval arithmetic PC calls (Interval<ZLB<int>>::project for NEG, ABS,
 * ADD, SUB, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, plus meet / fjoin / fmeet /
 * prev) lives in lala-core, which the reference does not vendor; it is restated
 * from its mathematical meaning in pc_oracle.cpp.
 *
 * Tape: nnodes nodes {kind[i], a[i], b[i], c[i]} (int32), kinds and fields as
 * in pc_kind below; every child index is smaller than its parent's.  A
 * propagator is the index of its root formula node.  Store layout as in the PIR
 * oracle: store[2v] = lb, store[2v+1] = ub. */
#ifndef PC_ORACLE_H
#define PC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  /* terms, in the order of lala::pc::Term's variant (terms.hpp:572-589) */
  ORC_PC_VAR = 0,     /* a = variable */
  ORC_PC_CONST = 1,   /* the constant interval [a, b] */
  ORC_PC_FORMULA = 2, /* a = formula node, read as 0/1 */
  ORC_PC_NEG = 3, ORC_PC_ABS = 4, /* a = operand */
  ORC_PC_ADD = 5, ORC_PC_SUB = 6, ORC_PC_MUL = 7, ORC_PC_TDIV = 8, ORC_PC_FDIV = 9,
  ORC_PC_CDIV = 10, ORC_PC_EDIV = 11, ORC_PC_MIN = 12, ORC_PC_MAX = 13, /* a, b = operands */
  ORC_PC_NADD = 14, ORC_PC_NMUL = 15, /* a = first ORC_PC_ARG node, b = operand count */
  /* formulas, in the order of lala::pc::Formula's variant (formula.hpp:905-920) */
  ORC_PC_PVAR = 16, ORC_PC_NVAR = 17, /* a = variable */
  ORC_PC_TRUE = 18, ORC_PC_FALSE = 19,
  ORC_PC_LEQ = 20, ORC_PC_GT = 21, ORC_PC_EQ = 22, ORC_PC_NEQ = 23, /* a, b = terms */
  ORC_PC_AND = 24, ORC_PC_OR = 25, ORC_PC_EQUIV = 26, ORC_PC_IMPLY = 27, ORC_PC_XOR = 28, /* a, b = formulas */
  ORC_PC_ARG = 29, /* operand slot of NADD / NMUL: a = term */
  ORC_PC_AE = 30,  /* AbstractElement: items a .. a+b-1 */
  ORC_PC_TELL = 31, ORC_PC_NTELL = 32, ORC_PC_ASK = 33, ORC_PC_NASK = 34, /* items {kind, var, lb, ub} */
  ORC_PC_ASK_OUT = 35, ORC_PC_NASK_OUT = 36, /* asks that the variable misses [lb, ub] */
  ORC_PC_NUM_KINDS = 37
};

/* Checks a tape against nvars; returns the deepest root's depth (nodes on the
 * longest path, >= 1), or -1 - (index of the first bad node), or -1 - nnodes
 * for a bad root. */
int32_t orc_pc_validate(int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
                        const int32_t *c, int32_t nprops, const int32_t *roots, int32_t nvars);

/* The propagator order of PC::deduce(tell) (pc.hpp:638-641): a stable sort of
 * roots[] by (formula kind, length), written to out_roots. */
void orc_pc_order(int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
                  const int32_t *c, int32_t nprops, const int32_t *roots, int32_t *out_roots);

/* One deduce(i) (formula.hpp Formula::deduce) of the formula rooted at `root`.
 * Returns the reference's has_changed; *failed is set if the store became
 * empty; *narrowed counts the bounds that moved. */
int32_t orc_pc_deduce(const int32_t *kind, const int32_t *a, const int32_t *b, const int32_t *c,
                      int32_t root, int32_t *store, int32_t *failed, int64_t *narrowed);

/* Formula::ask of the formula rooted at `root` on the store (failed = the
 * store is bot). */
int32_t orc_pc_ask(const int32_t *kind, const int32_t *a, const int32_t *b, const int32_t *c,
                   int32_t root, const int32_t *store, int32_t failed);

/* Term::project / Term::embed of the term rooted at `node`. */
void orc_pc_project(const int32_t *kind, const int32_t *a, const int32_t *b, const int32_t *c,
                    int32_t node, const int32_t *store, int32_t *out_lb, int32_t *out_ub);
int32_t orc_pc_embed(const int32_t *kind, const int32_t *a, const int32_t *b, const int32_t *c,
                     int32_t node, int32_t lb, int32_t ub, int32_t *store, int32_t *failed);

/* Gauss-Seidel fixpoint over the propagators in roots[] order: sweeps until a
 * sweep moves no bound (ORC_OK), a deduction empties the store (ORC_FAILED) or
 * max_sweeps (ORC_TIMEOUT).  out[0] = sweeps, out[1] = propagator executions,
 * out[2] = bounds narrowed, out[3] = OR of the reference's has_changed over all
 * executions. */
int32_t orc_pc_fixpoint(int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
                        const int32_t *c, int32_t nprops, const int32_t *roots, int32_t nvars,
                        int32_t *store, int64_t max_sweeps, int64_t *out);

/* The same fixpoint in Jacobi rounds: every deduction of a round reads the
 * store the round started from (its own joins included only from the next
 * round on) and the round's joins are met into it at the end; a round with
 * no join, or one that leaves a variable empty, ends the loop.  This is the
 * schedule of the GPU engine (a deterministic function of the input).  For
 * propagators that are monotone it reaches the same fixpoint as the
 * Gauss-Seidel loop.  out[0] = rounds, out[1] = executions, out[2] = bounds
 * narrowed. */
int32_t orc_pc_fixpoint_jacobi(int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
                               const int32_t *c, int32_t nprops, const int32_t *roots, int32_t nvars,
                               int32_t *store, int64_t max_rounds, int64_t *out);

/* Interval operators of the restated lala-core arithmetic, for the tests:
 * op = ORC_PC_NEG .. ORC_PC_MAX (unary ones ignore b). */
void orc_pc_itv(int32_t op, int32_t al, int32_t au, int32_t bl, int32_t bu, int32_t *out_l, int32_t *out_u);

#ifdef __cplusplus
}
#endif
#endif
