/* CPU oracle for the PIR propagator fixpoint — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library, and only as the checker or as the timed CPU baseline.  The
 * product (lala-pc_gb300/, libpirgpu.so) never links or calls it.
 *
 * It is a plain C++ restatement of lala-pc's PIR propagators
 * (include/lala/pir.hpp:395-817) and of the Gauss-Seidel fixpoint loop the
 * reference tests drive them with (tests/pir_test.cpp:60-62).  The lattice
 * semantics of lala-core (Interval<ZLB<int>>, VStore::embed, the division
 * functions of cuda-battery) are not vendored in the reference; they are
 * restated from their mathematical definition (see pir_oracle.cpp).
 *
 * Store layout: one int32 pair per variable, store[2*v] = lb, store[2*v+1] = ub.
 * Bytecode layout: structure of arrays op[i], x[i], y[i], z[i] (int32).
 * Arithmetic: every intermediate is computed exactly in int64 and clamped to
 * [INT32_MIN, INT32_MAX] when it becomes a bound; a per-thread counter records
 * each clamp that changed a value (the reference overflows there: parity with it
 * is only claimed when the counter stays 0). */
#ifndef PIR_ORACLE_H
#define PIR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opcodes: the PIR subset of lala-core's Sig accepted at pir.hpp:270-273.
 * The relative order (ADD < MUL < divisions < MIN < MAX < EQ < LEQ) follows
 * the Sig enum, which the CPU sort at pir.hpp:343-347 uses. */
enum {
  ORC_ADD = 0, ORC_MUL = 1, ORC_TDIV = 2, ORC_FDIV = 3, ORC_CDIV = 4,
  ORC_EDIV = 5, ORC_MIN = 6, ORC_MAX = 7, ORC_EQ = 8, ORC_LEQ = 9,
  ORC_NUM_OPS = 10
};

enum { ORC_OK = 0, ORC_FAILED = 1, ORC_TIMEOUT = 2, ORC_EINVAL = 3 };

/* One propagator application, pir.hpp:721-817.  Returns 1 iff a bound of the
 * store narrowed.  *failed is set to 1 if an embed left a variable empty. */
int orc_deduce(int32_t op, int32_t x, int32_t y, int32_t z, int32_t *store, int *failed);

/* deduce(bytecode) (op[k], 0, 1, 2) over `count` private 3-variable stores
 * in_lb/in_ub[3k..3k+2]; host threads.  *overflows = intermediates outside int32. */
int orc_search(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y, const int32_t *z,
               int32_t nvars, const int32_t *store, int32_t ndec, const int32_t *dec, int32_t order,
               int64_t max_solutions, int64_t max_nodes, int32_t *out_solutions, int64_t *out_stats);
void orc_ask_batch(int64_t count, const int32_t *op, const int32_t *in_lb, const int32_t *in_ub, uint8_t *out);
void orc_deduce_batch(int64_t count, const int32_t *op, const int32_t *in_lb, const int32_t *in_ub,
                      int32_t *out_lb, int32_t *out_ub, uint8_t *out_changed, uint8_t *out_failed,
                      int64_t *overflows);

/* Entailment of one propagator, pir.hpp:417-438. */
int orc_ask(int32_t op, int32_t x, int32_t y, int32_t z, const int32_t *store);

/* 1 iff any variable's interval is empty (lb > ub, or a bound at its bottom sentinel). */
int orc_store_is_bot(int32_t nvars, const int32_t *store);

/* Install: PIR::deduce(tell) (pir.hpp:326-352).  Meets x of every EQ/LEQ with
 * [0,1] in the store, and writes into perm[] the stable sort of the n
 * bytecodes by (op, y, x, z) (pir.hpp:343-347).  Returns ORC_FAILED if a meet
 * left the store empty, ORC_EINVAL on an out-of-range var or opcode. */
int orc_install(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                const int32_t *z, int32_t nvars, int32_t *store, int32_t *perm);

/* Gauss-Seidel fixpoint (tests/pir_test.cpp:60-62): sweeps i = 0..n-1 in the
 * given order until a sweep changes nothing.  Stops after the first sweep that
 * leaves the store empty (ORC_FAILED) or after max_sweeps (ORC_TIMEOUT).
 * out[0] = sweeps, out[1] = propagator executions, out[2] = bounds narrowed,
 * out[3] = clamps that changed a value. */
int orc_fixpoint(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                 const int32_t *z, int32_t nvars, int32_t *store,
                 int64_t max_sweeps, int64_t *out);

/* Exactly `sweeps` Gauss-Seidel sweeps in the given order (no stop test) —
 * used to time a bounded sample of sweeps. */
int orc_sweeps(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
               const int32_t *z, int32_t *store, int64_t sweeps, int64_t *out);

/* Batched search nodes (the snapshot/embed/fixpoint/restore loop of
 * tests/bound_consistency_test.hpp:175-196, one store per node).  Each node
 * starts from base_store, meets its tightenings
 * (var[k], lb[k], ub[k] for k in off[j]..off[j+1]-1), then runs the
 * Gauss-Seidel fixpoint.  Nodes run on `threads` host threads.
 * out_store: nnodes * 2 * nvars int32; out_status: nnodes int32;
 * out_stats: nnodes * 4 int64 (same fields as orc_fixpoint's out). */
int orc_fixpoint_nodes(int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                       const int32_t *z, int32_t nvars, const int32_t *base_store,
                       int32_t nnodes, const int32_t *off, const int32_t *var,
                       const int32_t *lb, const int32_t *ub, int64_t max_sweeps,
                       int32_t threads, int32_t *out_store, int32_t *out_status,
                       int64_t *out_stats);

/* Batched independent instances: instance j owns bytecodes
 * prop_off[j]..prop_off[j+1]-1 (var indices local to the instance) and store
 * entries var_off[j]..var_off[j+1]-1 of `store` (updated in place).  With
 * install != 0 each instance is installed first (reified meets, CPU sort). */
int orc_fixpoint_instances(int32_t ninst, const int64_t *prop_off, const int64_t *var_off,
                           const int32_t *op, const int32_t *x, const int32_t *y,
                           const int32_t *z, int32_t *store, int64_t max_sweeps,
                           int32_t threads, int32_t install, int32_t *out_status,
                           int64_t *out_stats);

/* Exhaustive property checks restating tests/bound_consistency_test.hpp.
 * pred: 0 eq_reif, 1 le_reif, 2 plus, 3 min, 4 max, 5 times, 6 ediv, 7 tdiv,
 * 8 cdiv, 9 fdiv, 10 emod, 11 tmod, 12 cmod, 13 fmod
 * (tests/pir_test.cpp:122-171).  Returns the number of violated expectations;
 * out[0] = cases checked, out[1] = first failing case index (or -1). */
int64_t orc_check_exhaustive(int32_t pred, int32_t minval, int32_t maxval,
                             int32_t test_completeness, int64_t *out);
int64_t orc_check_listed(int32_t pred, int32_t test_completeness, int64_t *out);
int64_t orc_check_completeness(int32_t pred, int32_t with_fixpoint, int64_t *out);

/* Builds the PIR decomposition of `constraint pred(y, z, x)` over vars
 * x=0, y=1, z=2 (plus fresh vars 3.. for the modulo decompositions).  Writes at
 * most 4 bytecodes; returns the bytecode count, *nvars the variable count. */
int32_t orc_build_pred(int32_t pred, int32_t *op, int32_t *x, int32_t *y, int32_t *z,
                       int32_t *nvars);

/* Reference division semantics (cuda-battery tdiv/fdiv/cdiv/ediv and the mods). */
int64_t orc_div(int32_t op, int64_t a, int64_t b);
int64_t orc_mod(int32_t kind, int64_t a, int64_t b);

#ifdef __cplusplus
}
#endif
#endif
