// Event-driven fixpoint of one instance: pir_fixpoint with
// opts.sched = PIR_SCHED_EVENTS.
//
// lala-pc's driver sweeps every propagator until a sweep changes nothing
// (GaussSeidelIteration around PIR::deduce(int), tests/pir_test.cpp:60-62);
// the AC-1 kernels do the same, one sweep per round.  Here a round runs only
// the units that have a variable narrowed in the previous round (the first
// round runs all of them), found through the variable -> unit adjacency.
// Every propagator of pir.hpp:721-817 reads only its three intervals, so one
// whose intervals did not change since its last run (which changed nothing)
// cannot change anything: the run ends at the same fixpoint, or the same
// failure, as the sweeps, bit for bit (propagators are monotone, so the order
// of the runs does not matter).  While a round narrows many variables the
// next one is dense (every unit, AC-1 style, noting only the narrowed
// variables: "Dense rounds" below); a final dense round (the certifying
// sweep, opts.certify) checks the fixpoint.
//
// Units.  A unit is a propagator, or a segment: up to SEG_MAX propagators of
// a path joined by link variables (variables with exactly two occurrences,
// pir_segments.h).  A thread runs a propagator; a warp runs a segment: it
// stages the segment's variables in shared memory, one lane sweeps the
// segment's propagators forward and backward until none narrows anything (a
// path of ADD links with constants is solved by the warp in closed form
// instead, seg_solve_path), and the warp joins what changed into the store
// and lists the units of the changed variables that have occurrences outside
// the segment.  A segment
// reached through a link variable is run at once by the same warp (chasing,
// SEG_CHASE per entry).  A long chain x_{i+1} = x_i + c_i then costs a few
// shared-memory accesses per link instead of dependent L2 round trips.
//
// Before this kernel, fixpoint_events runs AC-1 rounds of the persistent
// kernel while the bounds they narrow keep shrinking (ac1_lead, opts.lead):
// this kernel's dense rounds cost several AC-1 rounds, and the lead hands it
// the store once what is left is a steady trickle.
//
// Rounds with a large frontier run on the whole grid, separated by the grid
// barrier.  A round whose frontier has at most `local_max` units runs on CTA
// 0 alone, separated by __syncthreads, while the other CTAs wait at the next
// grid barrier; CTA 0 hands back when the frontier grows or the run ends.
// Within a round, a thread that narrows a variable with few units runs its
// propagators itself at once ("Chasing" below).
#include <algorithm>
#include <climits>
#include <cstring>

#include "pir_engine.h"
#include "pir_kernels.cuh"
#include "pir_segments.h"

namespace pirgpu {

namespace {

constexpr int EV_CONTINUE = 0, EV_FIXPOINT = 1, EV_FAILED = 2, EV_CAP = 3, EV_ERROR = 4;
constexpr int CNT_STRIDE = 32;  // counters one 128-byte line apart
constexpr int EV_BLOCK = 256, EV_WARPS = EV_BLOCK / 32;
constexpr int NO_UNIT = INT_MIN;  // an empty slot among units (a segment s is ~s, never INT_MIN)

struct EvFixArgs {
  const int4 *bc;  // {op, x, y, z} per propagator
  const int *adj_ptr, *adj;  // variable -> unit adjacency: propagator p as p, segment s as ~s
  int2 *store;
  unsigned *pstamp;  // per propagator: the last round it is listed for
  unsigned *sstamp;  // per segment: the last round it is listed for
  unsigned *vstamp;  // per variable: the last round its units were listed for
  int *list0, *list1;  // frontier (units) of round r: list0 for even r, list1 for odd r
  unsigned *cnt;     // frontier sizes: round r in cnt[(r % 3) * CNT_STRIDE]
  Control *ctl;
  long long n;
  long long max_rounds, timeout_ns;
  unsigned local_max;
  int chase;  // runs chased per frontier entry (0: none)
  int certify;  // end with a dense round (every unit once) that narrows nothing
  // path segments (nseg = 0: none; pir_segments.h)
  int nseg;
  const int *seg_pptr, *seg_code, *seg_vptr;
  const unsigned *seg_var, *in_seg;
  const unsigned long long *seg_umask;
  int *seg_busy;   // per segment: 1 while a warp runs it
  int2 *seg_last;  // per local slot: its interval when the segment's last run ended at its own fixpoint
  int *seg_valid;  // per segment: seg_last holds that run's intervals
  // dense rounds (every unit once, AC-1 style): the variables they narrow
  unsigned *cstamp;    // per variable: the last dense round (+ 1) that noted it
  int *cvl0, *cvl1;    // the variables noted by dense round r: cvl0 for even r, cvl1 for odd r
  unsigned *ccnt;      // their counts: round r in ccnt[(r % 3) * CNT_STRIDE]
  unsigned *dsum;      // the sum of their unit degrees, likewise
  unsigned *dflag;     // round r in dflag[(r % 3) * CNT_STRIDE]: a segment has sweeps left, dense again
  int dense_div;       // a dense round whose noted variables have at least n / dense_div units may be followed
                       // by another (0: never)
  int nvars;
};

__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Chasing.  A run that narrows a variable with at most CHASE_DEG units runs
// the propagators among them itself at once (up to `chase` runs per frontier
// entry, CHASE_CAP pending, in shared memory) instead of leaving them to the
// next round; every other narrowed variable has its units listed for the
// next round, and so has whatever is still pending when the runs run out.
// A run is first repeated on its own results (up to CLOSE_RUNS runs; past
// that the propagator is listed), so the propagator that narrowed a variable
// is not chased with the variable's others.  Every unit of a narrowed
// variable thus runs after the narrowing, at once or in the next round,
// which is all the event schedule needs (the propagators are monotone).
// The budget is capped: a chase is dependent L2 round trips (a few us each,
// more when many chasers narrow the same variables), and the grid's other
// CTAs wait for the round at a barrier with a time limit.
constexpr int CHASE_DEG = 4, CHASE_CAP = 8, CLOSE_RUNS = 4, CHASE_DEFAULT = 64, CHASE_MAX = 256, DEFER_CAP = 8;

// Segments: sweeps per run before the rest waits for the next round,
// segments chased per frontier entry, the chase stack of a warp, and the
// frontier's segments a CTA queues for its warps per round (more wait for the
// next round).
constexpr int SEG_PASSES = 16, SEG_CHASE = 32, SEG_STACK = 8, SEG_QUEUE = 256;

// One run's joins: red to the store as RedStore does, and the run's view of
// its three variables (the intervals it read, met with what it joined) for
// a repeat on its own results; hit = the slots whose variable narrowed.
// (Atomics whose old value tells whether a join moved the stored bound would
// let only that run propagate, but waiting for the old value puts an L2
// round trip on every chased step: 62 -> 80 ms on 1M vars / 4M propagators
// plus a 20,000-link chain.)
struct RunView {
  int2 *s;
  int var[3];
  Itv n[3];
  unsigned hit;
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + v);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) {
    int c = 0;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&s[v].x), "r"(r.l) : "memory");
      ++c;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&s[v].y), "r"(r.u) : "memory");
      ++c;
    }
    if (c) {
      const Itv m = mk(max(seen.l, r.l), min(seen.u, r.u));
      if (is_bot(m)) failed = 1;
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (var[k] == v) {
          n[k] = mk(max(n[k].l, m.l), min(n[k].u, m.u));
          hit |= 1u << k;
        }
    }
    return c;
  }
};

// Listing policy of the grid rounds: the first narrowing of a variable in
// round r lists its units for round r + 1 (the round stamps keep every
// variable expanded, and every unit listed, at most once per round).  The
// adjacency is walked EXPAND entries at a time: their loads and stamp
// atomics are independent (one memory round trip each per batch, not per
// entry), and the batch takes its list slots with one atomic.
constexpr int EXPAND = 8;

struct EvSched {
  static constexpr bool kDense = false;
  const int *adj;
  unsigned *pstamp, *sstamp, *vstamp;
  int *next;
  unsigned *next_cnt;
  unsigned next_round;
  __device__ __forceinline__ void note(int) const {}
  __device__ __forceinline__ bool claim(int u) const {
    return atomicMax(u >= 0 ? pstamp + u : sstamp + ~u, next_round) < next_round;
  }
  __device__ __forceinline__ void list_unit(int u) const {
    if (claim(u)) next[atomicAdd(next_cnt, 1u)] = u;
  }
  // Lists the cnt (<= DEFER_CAP) units buf[0], buf[stride], ...
  __device__ __forceinline__ void list_batch(const int *buf, int cnt, int stride) const {
    int q[DEFER_CAP];
    unsigned take = 0;
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j) q[j] = j < cnt ? buf[j * stride] : NO_UNIT;
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j)
      if (q[j] != NO_UNIT && claim(q[j])) take |= 1u << j;
    if (!take) return;
    unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j)
      if (take & (1u << j)) next[slot++] = q[j];
  }
  __device__ __forceinline__ void expand(int2 r, int skip) const {
    for (int k0 = r.x; k0 < r.y; k0 += EXPAND) {
      int q[EXPAND];
#pragma unroll
      for (int j = 0; j < EXPAND; ++j) q[j] = k0 + j < r.y ? __ldg(adj + k0 + j) : NO_UNIT;
      unsigned take = 0;
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (q[j] != NO_UNIT && q[j] != skip && claim(q[j])) take |= 1u << j;
      if (!take) continue;
      unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (take & (1u << j)) next[slot++] = q[j];
    }
  }
  // Lists v's units (adjacency range r) for the next round.
  __device__ __forceinline__ void schedule(int v, int2 r) const {
    if (atomicMax(vstamp + v, next_round) >= next_round) return;
    expand(r, NO_UNIT);
  }
  // The same for a variable a segment narrowed, without the segment itself
  // (it left its variables at its own fixpoint), and without the variable's
  // stamp: a later narrowing of v in this round must still list the segment.
  __device__ __forceinline__ void schedule_but(int v, int2 r, int skip) const { expand(r, skip); }
};

__device__ __forceinline__ EvSched ev_sched(const EvFixArgs &a, long long round) {
  EvSched sc;
  sc.adj = a.adj;
  sc.pstamp = a.pstamp;
  sc.sstamp = a.sstamp;
  sc.vstamp = a.vstamp;
  sc.next = ((round + 1) & 1) ? a.list1 : a.list0;
  sc.next_cnt = a.cnt + ((round + 1) % 3) * CNT_STRIDE;
  sc.next_round = (unsigned)(round + 1);
  return sc;
}

// Runs frontier propagator q and what it chases (stack: this thread's
// CHASE_CAP slots, blockDim.x apart; defer: its DEFER_CAP slots).  Returns
// the bounds narrowed.  A run whose variable is chased is itself listed for
// the next round: its repeat on its own results does not see what a
// concurrent run of the same propagator joined, and the next round reads the
// store after the barrier.  Those listings wait in `defer` and go out
// DEFER_CAP at a time (their stamp atomics in flight together), off the
// chase's critical path.  Segments met on the way are listed.
template <class Sched>
__device__ __forceinline__ int run_entry(int q, const EvFixArgs &a, const Sched &sc, int *stack, int *defer,
                                         int budget, unsigned long long &execs, int &failed) {
  const int stride = blockDim.x;
  const int close = budget > 0 ? CLOSE_RUNS : 1;
  RunView w;
  w.s = a.store;
  int sp = 0, dn = 0, changed = 0;
  for (;;) {
    const int4 b = __ldg(a.bc + q);
    w.var[0] = b.y;
    w.var[1] = b.z;
    w.var[2] = b.w;
    Itv o0 = w.load(b.y), o1 = w.load(b.z), o2 = w.load(b.w);
    const int2 r0 = make_int2(__ldg(a.adj_ptr + b.y), __ldg(a.adj_ptr + b.y + 1));
    const int2 r1 = make_int2(__ldg(a.adj_ptr + b.z), __ldg(a.adj_ptr + b.z + 1));
    const int2 r2 = make_int2(__ldg(a.adj_ptr + b.w), __ldg(a.adj_ptr + b.w + 1));
    unsigned hit = 0;
    int k = 0;
    for (; k < close; ++k) {
      w.n[0] = o0;
      w.n[1] = o1;
      w.n[2] = o2;
      w.hit = 0u;
      changed += deduce_loaded(b.x, b.y, b.z, b.w, o0, o1, o2, w, failed);
      ++execs;
      if (!w.hit || failed) break;
      hit |= w.hit;
      o0 = w.n[0];
      o1 = w.n[1];
      o2 = w.n[2];
    }
    if (failed) return changed;  // the round fails
    if (k == close) sc.list_unit(q);
    bool chased = false;
    // each distinct variable once (a hit marks every slot of its variable)
    if (b.z == b.y) hit &= ~2u;
    if (b.w == b.y || b.w == b.z) hit &= ~4u;
    for (unsigned h = hit; h; h &= h - 1) {
      const int sl = __ffs(h) - 1;
      const int v = sl == 0 ? b.y : (sl == 1 ? b.z : b.w);
      const int2 r = sl == 0 ? r0 : (sl == 1 ? r1 : r2);
      const int deg = r.y - r.x;
      if (budget > 0 && deg <= CHASE_DEG && sp + deg <= CHASE_CAP) {
        int e[CHASE_DEG];
#pragma unroll
        for (int j = 0; j < CHASE_DEG; ++j) e[j] = j < deg ? __ldg(a.adj + r.x + j) : q;
#pragma unroll
        for (int j = 0; j < CHASE_DEG; ++j) {
          if (e[j] == q) continue;
          if (e[j] >= 0)
            stack[(sp++) * stride] = e[j];
          else
            sc.list_unit(e[j]);  // a segment: a warp runs it next round
        }
        chased = true;
      } else {
        sc.schedule(v, r);
      }
    }
    if (chased && k < close) {
      defer[(dn++) * stride] = q;
      if (dn == DEFER_CAP) {
        sc.list_batch(defer, dn, stride);
        dn = 0;
      }
    }
    if (sp == 0) break;
    if (budget <= 0) {
      while (sp > 0) sc.list_unit(stack[(--sp) * stride]);
      break;
    }
    q = stack[(--sp) * stride];
    --budget;
  }
  if (dn) sc.list_batch(defer, dn, stride);
  return changed;
}

// ------------------------------------------------------------- segments ----

// A warp's shared-memory workspace for one segment.
struct SegWork {
  int2 iv[SEG_VARS];                   // the segment's intervals, as its sweeps leave them
  int2 orig[SEG_VARS];                 // as read from the store
  unsigned long long umask[SEG_VARS];  // per local variable: the segment's propagators using it
  unsigned var[SEG_VARS];              // global variable | SEG_BOUNDARY
  int code[SEG_MAX];                   // op | slot_x << 8 | slot_y << 16 | slot_z << 24
  int stack[SEG_STACK];                // segments to chase
  int sp;
};

// The frontier segments a CTA queues in a round for its warps (one queue per
// round parity: the other is reset while this one is in use).
struct SegQueue {
  int q[SEG_QUEUE];
  int n, head;
};

// The sweeps' store: the segment's intervals in shared memory (one lane).  A
// narrowing meets into the current interval and marks the propagators of
// the segment that use the variable for another run.
struct SegStore {
  int2 *iv;
  const unsigned long long *umask;
  unsigned long long dirty;
  __device__ __forceinline__ Itv load(int i) const {
    const int2 t = iv[i];
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int i, Itv, Itv r, int &failed) {
    const int2 t = iv[i];
    const int nl = max(t.x, r.l), nu = min(t.y, r.u);
    const int c = (nl != t.x) + (nu != t.y);
    if (c) {
      iv[i] = make_int2(nl, nu);
      dirty |= umask[i];
      if (is_bot(mk(nl, nu))) failed = 1;
    }
    return c;
  }
};

// The sweeps' store for a propagator over three distinct slots: the lane
// owns the workspace and each slot is joined at most once per run, so the
// interval read at the start of the run is still the current one when its
// join comes (no reload), and the slots' propagator masks are read with the
// intervals instead of after a narrowing.
struct SegStore3 {
  int2 *iv;
  int sx, sy;
  unsigned long long mx, my, mz;  // umask of slots sx, sy, sz
  unsigned long long dirty;
  __device__ __forceinline__ int embed(int i, Itv seen, Itv r, int &failed) {
    const int nl = max(seen.l, r.l), nu = min(seen.u, r.u);
    const int c = (nl != seen.l) + (nu != seen.u);
    if (c) {
      iv[i] = make_int2(nl, nu);
      dirty |= i == sx ? mx : (i == sy ? my : mz);
      if (is_bot(mk(nl, nu))) failed = 1;
    }
    return c;
  }
};

// One propagator of the segment.  ADD, MIN, MAX and the reified EQ / LEQ
// are idempotent (a second run on what the first left narrows nothing;
// checked exhaustively against the oracle), so such a propagator over three
// distinct variables is not marked again by its own narrowings; MUL and the
// divisions are.
__device__ __forceinline__ void seg_run_one(const SegWork &w, SegStore &st, int k, int &failed) {
  const unsigned c = (unsigned)w.code[k];
  const int op = (int)(c & 0xFFu), sx = (int)((c >> 8) & 0xFFu), sy = (int)((c >> 16) & 0xFFu), sz = (int)(c >> 24);
  const unsigned long long bit = 1ull << k;
  st.dirty &= ~bit;
  if (sx != sy && sx != sz && sy != sz) {
    const int2 a = st.iv[sx], b = st.iv[sy], d = st.iv[sz];
    SegStore3 s3{st.iv, sx, sy, st.umask[sx], st.umask[sy], st.umask[sz], 0ull};
    deduce_loaded(op, sx, sy, sz, mk(a.x, a.y), mk(b.x, b.y), mk(d.x, d.y), s3, failed);
    const bool idem = op == OP_ADD || op == OP_MIN || op == OP_MAX || op == OP_EQ || op == OP_LEQ;
    st.dirty |= idem ? (s3.dirty & ~bit) : s3.dirty;
    return;
  }
  deduce(op, sx, sy, sz, st, failed);
}

// seg_run_one for a segment whose propagators are all ADD over three distinct
// slots (the links of a chain x_{i+1} = x_i + c_i): the same arithmetic,
// with the opcode known, so none of the other opcodes' code is on the lane's
// path.
__device__ __forceinline__ void seg_run_add(const SegWork &w, SegStore &st, int k, int &failed) {
  const unsigned c = (unsigned)w.code[k];
  const int sx = (int)((c >> 8) & 0xFFu), sy = (int)((c >> 16) & 0xFFu), sz = (int)(c >> 24);
  const unsigned long long bit = 1ull << k;
  const int2 a = st.iv[sx], b = st.iv[sy], d = st.iv[sz];
  SegStore3 s3{st.iv, sx, sy, st.umask[sx], st.umask[sy], st.umask[sz], 0ull};
  deduce_loaded(OP_ADD, sx, sy, sz, mk(a.x, a.y), mk(b.x, b.y), mk(d.x, d.y), s3, failed);
  st.dirty = (st.dirty | s3.dirty) & ~bit;  // ADD is idempotent: not marked again by its own narrowings
}

// A segment that is a path of ADD links with a constant each: link k relates
// chain variables v_k and v_{k+1} by v_{k+1} = v_k + d_k (d_k = c_k when
// the link reads x = v_{k+1}, y or z = v_k, the other operand the constant
// c_k; d_k = -c_k when it runs the other way), every constant a singleton
// used by its link alone.  The sweeps' fixpoint of such a path is the
// difference-constraint closure along it: with P_0 = 0, P_{k+1} = P_k + d_k,
//   lb(v_j) = P_j + max_i (lb(v_i) - P_i),  ub(v_j) = P_j + min_i (ub(v_i) - P_i),
// and the constants narrow nothing unless the path fails (max > min: every
// variable empty).  Bounds within +-2^28 and constants within +-2^22 keep every
// sum the sweeps would form inside int32, so none of their saturating steps
// saturates and the closure is their fixpoint exactly.  Called by the whole
// warp; returns (warp-uniform) whether it solved the segment, the failure in
// `failed`.
constexpr long long PATH_BOUND = 1ll << 28, PATH_CONST = 1ll << 22;

__device__ __noinline__ bool seg_solve_path(SegWork &w, int np, int &failed) {
  const int lane = threadIdx.x & 31;
  int in[2] = {0, 0}, out[2] = {0, 0};
  long long d[2] = {0, 0};
  bool ok = true;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    if (k >= np) continue;
    const unsigned c = (unsigned)w.code[k];
    const int sx = (int)((c >> 8) & 0xFFu), sy = (int)((c >> 16) & 0xFFu), sz = (int)(c >> 24);
    auto constant = [&](int s) {
      return !(w.var[s] & SEG_BOUNDARY) && w.umask[s] == (1ull << k) && w.iv[s].x == w.iv[s].y;
    };
    const bool cy = constant(sy), cz = constant(sz);
    if (cy == cz) {
      ok = false;
      continue;
    }
    in[h] = cz ? sy : sz;
    out[h] = sx;
    d[h] = cz ? w.iv[sz].x : w.iv[sy].x;
    if (d[h] <= -PATH_CONST || d[h] >= PATH_CONST) ok = false;
  }
  if (!__all_sync(0xFFFFFFFFu, ok)) return false;
  // orientation: forward when link k's input is link k - 1's output, reverse
  // when link k's output is link k - 1's input
  const int pin0 = __shfl_up_sync(0xFFFFFFFFu, in[0], 1), pout0 = __shfl_up_sync(0xFFFFFFFFu, out[0], 1);
  int pin1 = __shfl_up_sync(0xFFFFFFFFu, in[1], 1), pout1 = __shfl_up_sync(0xFFFFFFFFu, out[1], 1);
  const int last_in0 = __shfl_sync(0xFFFFFFFFu, in[0], 31), last_out0 = __shfl_sync(0xFFFFFFFFu, out[0], 31);
  if (lane == 0) {
    pin1 = last_in0;
    pout1 = last_out0;
  }
  bool fwd = true, rev = true;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    if (k == 0 || k >= np) continue;
    const int pi = h ? pin1 : pin0, po = h ? pout1 : pout0;
    fwd = fwd && in[h] == po;
    rev = rev && out[h] == pi;
  }
  fwd = __all_sync(0xFFFFFFFFu, fwd);
  rev = __all_sync(0xFFFFFFFFu, rev);
  if (fwd == rev) return false;  // neither (or a degenerate one-link path)
  // the path's variables must be used by their links alone: v_{k+1} by links
  // k and k + 1, v_0 by link 0
  const int v0 = __shfl_sync(0xFFFFFFFFu, fwd ? in[0] : out[0], 0);
  int vn[2];
  ok = true;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    vn[h] = fwd ? out[h] : in[h];
    if (k >= np) continue;
    if (!fwd) d[h] = -d[h];
    const unsigned long long want = (1ull << k) | (k + 1 < np ? 1ull << (k + 1) : 0ull);
    if (w.umask[vn[h]] != want) ok = false;
  }
  if (lane == 0 && w.umask[v0] != 1ull) ok = false;
  if (!__all_sync(0xFFFFFFFFu, ok)) return false;
  // P_{k+1}: inclusive sums of d over links 0..k (two halves of 32)
  long long s0 = d[0], s1 = d[1];
  for (int o = 1; o < 32; o <<= 1) {
    const long long t0 = __shfl_up_sync(0xFFFFFFFFu, s0, o), t1 = __shfl_up_sync(0xFFFFFFFFu, s1, o);
    if (lane >= o) {
      s0 += t0;
      s1 += t1;
    }
  }
  s1 += __shfl_sync(0xFFFFFFFFu, s0, 31);
  // max of lb - P and min of ub - P over v_0 .. v_np; every bound finite and small
  long long mx = LLONG_MIN, mn = LLONG_MAX;
  auto take = [&](int v, long long P) {
    const int2 t = w.iv[v];
    if (t.x == MINF || t.y == INF || t.x <= -PATH_BOUND || t.y >= PATH_BOUND || t.x >= PATH_BOUND ||
        t.y <= -PATH_BOUND)
      ok = false;
    mx = max(mx, (long long)t.x - P);
    mn = min(mn, (long long)t.y - P);
  };
  if (lane == 0) take(v0, 0);
  if (lane < np) take(vn[0], s0);
  if (lane + 32 < np) take(vn[1], s1);
  if (!__all_sync(0xFFFFFFFFu, ok)) return false;
  for (int o = 16; o; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
    mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o));
  }
  if (mx > mn) {
    failed = 1;
    return true;
  }
  // the closure; every value lies within the variable's own bounds
  if (lane == 0) w.iv[v0] = make_int2((int)mx, (int)mn);
  if (lane < np) w.iv[vn[0]] = make_int2((int)(s0 + mx), (int)(s0 + mn));
  if (lane + 32 < np) w.iv[vn[1]] = make_int2((int)(s1 + mx), (int)(s1 + mn));
  return true;
}

// The lane's sweeps of a segment: each pass runs the marked propagators
// forward, then backward; a mark set during a pass ahead of the current
// position is run in that pass.  Returns the runs.
template <bool ALL_ADD>
__device__ __forceinline__ unsigned long long seg_sweep(const SegWork &w, SegStore &st, int &fl) {
  unsigned long long ex = 0;
  for (int pass = 0; st.dirty && !fl && pass < SEG_PASSES; ++pass) {
    for (int k = -1;;) {
      const unsigned long long ahead = k >= 63 ? 0ull : st.dirty & (~0ull << (k + 1));
      if (!ahead || fl) break;
      k = __ffsll((long long)ahead) - 1;
      if (ALL_ADD) seg_run_add(w, st, k, fl);
      else seg_run_one(w, st, k, fl);
      ++ex;
    }
    for (int k = 64;;) {
      const unsigned long long behind = k >= 64 ? st.dirty : st.dirty & ((1ull << k) - 1ull);
      if (!behind || fl) break;
      k = 63 - __clzll((long long)behind);
      if (ALL_ADD) seg_run_add(w, st, k, fl);
      else seg_run_one(w, st, k, fl);
      ++ex;
    }
  }
  return ex;
}

// Runs segment s on the calling warp (all 32 lanes): stage, sweep, join, and
// list (or push on the warp's chase stack, when `chase`) the units of the
// changed variables that have occurrences outside the segment.  The sweeps
// start from every propagator in a dense round, and otherwise from the
// propagators of the variables that differ from the segment's snapshot (the
// intervals its last run left at its own fixpoint: the others are still at
// their fixpoint).  Returns this lane's count of bounds narrowed in the store.
template <class Sched>
__device__ int run_segment(const EvFixArgs &a, const Sched &sc, int s, SegWork &w, bool chase, bool full,
                           unsigned long long &execs, int &failed) {
  const int lane = threadIdx.x & 31;
  int got = 0;
  if (lane == 0) got = atomicCAS(a.seg_busy + s, 0, 1) == 0;
  got = __shfl_sync(0xFFFFFFFFu, got, 0);
  if (!got) {  // another warp runs it: it runs again next round
    if (lane == 0) sc.list_unit(~s);
    return 0;
  }
  const int p0 = __ldg(a.seg_pptr + s), np = __ldg(a.seg_pptr + s + 1) - p0;
  const int v0 = __ldg(a.seg_vptr + s), nl = __ldg(a.seg_vptr + s + 1) - v0;
  const bool snap = !full && __ldcg(a.seg_valid + s);
  unsigned long long start = 0ull;
  for (int i = lane; i < nl; i += 32) {
    const unsigned gv = __ldg(a.seg_var + v0 + i);
    const int2 t = __ldcg(a.store + (int)(gv & ~SEG_BOUNDARY));
    const unsigned long long um = __ldg(a.seg_umask + v0 + i);
    w.var[i] = gv;
    w.iv[i] = t;
    w.orig[i] = t;
    w.umask[i] = um;
    if (snap) {
      const int2 l = __ldcg(a.seg_last + v0 + i);
      if (l.x != t.x || l.y != t.y) start |= um;
    }
  }
  bool add_only = true;  // every propagator ADD over three distinct slots
  for (int k = lane; k < np; k += 32) {
    const int c = __ldg(a.seg_code + p0 + k);
    w.code[k] = c;
    const int sx = (c >> 8) & 0xFF, sy = (c >> 16) & 0xFF, sz = (int)((unsigned)c >> 24);
    add_only = add_only && (c & 0xFF) == OP_ADD && sx != sy && sx != sz && sy != sz;
  }
  add_only = __all_sync(0xFFFFFFFFu, add_only);
  if (snap) {
    const unsigned lo = __reduce_or_sync(0xFFFFFFFFu, (unsigned)start);
    const unsigned hi = __reduce_or_sync(0xFFFFFFFFu, (unsigned)(start >> 32));
    start = (unsigned long long)hi << 32 | lo;
  } else {
    start = np >= 64 ? ~0ull : ((1ull << np) - 1ull);
  }
  __syncwarp();
  int fl = 0, conv = 1;
  // a path of ADD links with constants is solved in closed form by the warp
  // (each link counted as one execution); anything else is swept by a lane
  const bool solved = add_only && seg_solve_path(w, np, fl);
  if (lane == 0) {
    if (solved) {
      execs += (unsigned long long)np;
    } else {
      SegStore st{w.iv, w.umask, start};
      const unsigned long long ex = add_only ? seg_sweep<true>(w, st, fl) : seg_sweep<false>(w, st, fl);
      conv = st.dirty == 0ull;
      execs += ex;
    }
  }
  __syncwarp();
  fl = __shfl_sync(0xFFFFFFFFu, fl, 0);
  conv = __shfl_sync(0xFFFFFFFFu, conv, 0);
  int changed = 0;
  for (int i = lane; i < nl; i += 32) {
    const int2 o = w.orig[i], t = w.iv[i];
    const bool lo = t.x > o.x, hi = t.y < o.y;
    if (!lo && !hi) continue;
    const unsigned gv = w.var[i];
    const int v = (int)(gv & ~SEG_BOUNDARY);
    if (lo) asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&a.store[v].x), "r"(t.x) : "memory");
    if (hi) asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&a.store[v].y), "r"(t.y) : "memory");
    changed += (int)lo + (int)hi;
    if (!(gv & SEG_BOUNDARY) || fl) continue;
    if (Sched::kDense) {
      sc.note(v);
      continue;
    }
    const int2 r = make_int2(__ldg(a.adj_ptr + v), __ldg(a.adj_ptr + v + 1));
    if (r.y - r.x == 2) {
      // a link variable: the one other unit
      const int u0 = __ldg(a.adj + r.x), u1 = __ldg(a.adj + r.x + 1);
      const int other = u0 == ~s ? u1 : u0;
      if (chase && other < 0) {
        const int k = atomicAdd(&w.sp, 1);
        if (k < SEG_STACK) {
          w.stack[k] = ~other;
          continue;
        }
      }
      sc.list_unit(other);
    } else {
      sc.schedule_but(v, r, ~s);
    }
  }
  // the snapshot of this run's own fixpoint (none when it stopped short)
  if (conv && !fl)
    for (int i = lane; i < nl; i += 32) a.seg_last[v0 + i] = w.iv[i];
  __syncwarp();
  if (lane == 0) {
    a.seg_valid[s] = conv && !fl;
    __threadfence();
    atomicExch(a.seg_busy + s, 0);
    if (!conv && !fl) sc.list_unit(~s);  // sweeps left over: the rest next round
  }
  failed |= fl;
  return changed;
}

// Runs segment s and the segments it chases (SEG_CHASE per entry, none
// when chasing is off) on the calling warp.
template <class Sched>
__device__ int run_segment_chain(const EvFixArgs &a, const Sched &sc, int s, SegWork &w, bool full,
                                 unsigned long long &execs, int &failed) {
  const int lane = threadIdx.x & 31;
  int budget = a.chase > 0 ? SEG_CHASE : 0, changed = 0;
  if (lane == 0) w.sp = 0;
  __syncwarp();
  for (;;) {
    changed += run_segment(a, sc, s, w, budget > 0, full, execs, failed);
    full = false;  // chased segments start from what changed
    __syncwarp();
    const int sp = min(w.sp, SEG_STACK);
    if (sp == 0 || failed) break;
    if (budget <= 0) {
      for (int i = lane; i < sp; i += 32) sc.list_unit(~w.stack[i]);
      break;
    }
    --budget;
    s = w.stack[sp - 1];
    __syncwarp();
    if (lane == 0) w.sp = sp - 1;
    __syncwarp();
  }
  return changed;
}

// The warp phase of an event round: the segments its CTA queued.
template <class Sched>
__device__ int run_segment_phase(const EvFixArgs &a, const Sched &sc, SegQueue &q, SegWork *work,
                                 unsigned long long &execs, int &failed) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  SegWork &w = work[warp];
  int changed = 0;
  // the lanes' own failures (from their propagators) made warp-uniform: the
  // segment code below runs on whole warps
  failed = __any_sync(0xFFFFFFFFu, failed) ? 1 : 0;
  const int items = min(q.n, SEG_QUEUE);
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(&q.head, 1);
    k = __shfl_sync(0xFFFFFFFFu, k, 0);
    if (k >= items || failed) break;
    changed += run_segment_chain(a, sc, q.q[k], w, false, execs, failed);
  }
  return changed;
}

// A frontier entry that is a segment: queued for the CTA's warps this round,
// or, with the queue full, listed for the next.
template <class Sched>
__device__ __forceinline__ void queue_segment(int u, SegQueue &q, const Sched &sc) {
  const int k = atomicAdd(&q.n, 1);
  if (k < SEG_QUEUE)
    q.q[k] = ~u;
  else
    sc.list_unit(u);
}

__device__ __forceinline__ bool in_segment(const EvFixArgs &a, long long p) {
  return a.nseg && ((__ldg(a.in_seg + (p >> 5)) >> (p & 31)) & 1u);
}

// Runs the frontier entries i = first, first + stride, ... < items of event
// round `round` (segments go to the queue).  Returns the bounds narrowed.
__device__ __forceinline__ int run_frontier(const EvFixArgs &a, long long round, long long items, long long first,
                                            long long stride, int *stack, int *defer, SegQueue &sq,
                                            unsigned long long &execs, int &failed) {
  const EvSched sc = ev_sched(a, round);
  const int *cur = (round & 1) ? a.list1 : a.list0;
  int changed = 0;
  for (long long i = first; i < items && !failed; i += stride) {
    const int u = __ldcg(cur + i);
    if (u < 0)
      queue_segment(u, sq, sc);
    else
      changed += run_entry(u, a, sc, stack, defer, a.chase, execs, failed);
  }
  return changed;
}

// ---------------------------------------------------------- dense rounds ----
//
// Early rounds narrow a large share of the variables, and listing each
// narrowed variable's units (a stamp atomic per unit) then costs more than
// running every unit.  A dense round runs every propagator once (threads,
// grid-strided, as an AC-1 sweep) and every segment (warps, all of it), and
// only notes which variables it narrowed: the first narrowing of a variable
// in the round appends it to the round's list (one atomic per variable).  The
// next round is dense again while the noted variables' units number at least
// n / dense_div and the list keeps shrinking (by an eighth over DENSE_WINDOW
// dense rounds: deep propagation that narrows about the same variables round after
// round, a long chain, moves faster in event rounds, whose chases dense
// rounds lack);
// otherwise an expansion phase lists the units of the noted variables and
// event rounds go on.  A dense round ran every unit, so one that narrows nothing ends the
// run at a fixpoint: the first round and the certifying sweep are dense
// rounds.
constexpr int DENSE_WINDOW = 16;

struct DenseSched {
  static constexpr bool kDense = true;
  const int *adj_ptr;
  unsigned *cstamp;
  int *cvl;
  unsigned *ccnt, *dsum, *dflag;
  unsigned tag;
  __device__ __forceinline__ void note(int v) const {
    if (atomicMax(cstamp + v, tag) < tag) {
      cvl[atomicAdd(ccnt, 1u)] = v;
      atomicAdd(dsum, (unsigned)(__ldg(adj_ptr + v + 1) - __ldg(adj_ptr + v)));
    }
  }
  // a segment left with sweeps to do: the next round is dense again
  __device__ __forceinline__ void list_unit(int) const { atomicOr(dflag, 1u); }
  __device__ __forceinline__ void schedule_but(int v, int2, int) const { note(v); }
};

__device__ __forceinline__ DenseSched dense_sched(const EvFixArgs &a, long long round) {
  DenseSched d;
  d.adj_ptr = a.adj_ptr;
  d.cstamp = a.cstamp;
  d.cvl = (round & 1) ? a.cvl1 : a.cvl0;
  d.ccnt = a.ccnt + (round % 3) * CNT_STRIDE;
  d.dsum = a.dsum + (round % 3) * CNT_STRIDE;
  d.dflag = a.dflag + (round % 3) * CNT_STRIDE;
  d.tag = (unsigned)(round + 1);
  return d;
}

// RedStore's joins, noting the narrowed variables.
struct DenseStore {
  int2 *s;
  const DenseSched *sc;
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + v);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int c = 0;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&s[v].x), "r"(r.l) : "memory");
      ++c;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&s[v].y), "r"(r.u) : "memory");
      ++c;
    }
    if (c) {
      sc->note(v);
      if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    }
    return c;
  }
};

// The threads' part of a dense round: every propagator outside the segments.
__device__ __forceinline__ int run_dense(const EvFixArgs &a, const DenseSched &ds, long long first, long long stride,
                                         unsigned long long &execs, int &failed) {
  DenseStore st{a.store, &ds};
  int changed = 0;
  for (long long i = first; i < a.n && !failed; i += stride) {
    if (in_segment(a, i)) continue;
    const int4 b = __ldg(a.bc + i);
    const Itv o0 = st.load(b.y), o1 = st.load(b.z), o2 = st.load(b.w);
    changed += deduce_loaded(b.x, b.y, b.z, b.w, o0, o1, o2, st, failed);
    ++execs;
  }
  return changed;
}

// Rounds run by CTA 0 alone keep their bookkeeping in shared memory: the
// frontier's first LOCAL_CAP entries, the list counters, and the round's
// sets of expanded variables and listed units (open addressing, at most
// L_PROBE probes).  Every listed unit also goes to the global list (a store
// nobody waits on), so a round whose frontier outgrows local_max hands over
// to the grid as it is.  A key that finds no free slot in its probe window
// falls back to the global round stamps; since slots only fill during a
// round, every thread that meets that key takes the same route, and each
// unit is still listed at most once per round.  The stamps hold round
// numbers, which only grow, so the rounds run here leave them valid for later
// rounds.
constexpr int LOCAL_CAP = 256, LV_LOG = 10, LP_LOG = 11, L_PROBE = 16;

struct LocalShared {
  int q[2][LOCAL_CAP];       // frontier, by round parity
  int vset[2][1 << LV_LOG];  // variables expanded, by round parity
  int pset[2][1 << LP_LOG];  // units listed, by round parity
  unsigned cnt[3], bits[3];  // list sizes and changed | failed bits, round % 3
};

// 1 inserted, 0 already there, -1 no free slot within L_PROBE probes.
template <int LOG>
__device__ __forceinline__ int local_insert(int *tab, int key) {
  unsigned h = ((unsigned)key * 2654435761u) >> (32 - LOG);
  for (int i = 0; i < L_PROBE; ++i) {
    const int prev = atomicCAS(tab + h, -1, key);
    if (prev == -1) return 1;
    if (prev == key) return 0;
    h = (h + 1) & ((1u << LOG) - 1u);
  }
  return -1;
}

// Listing policy of the local rounds: EvSched's, with the round's sets and
// the list head in shared memory.
struct LocalSched {
  static constexpr bool kDense = false;
  __device__ __forceinline__ void note(int) const {}
  const int *adj;
  unsigned *pstamp, *sstamp, *vstamp;
  int *next;           // global list of the next round
  int *next_q;         // its first LOCAL_CAP entries (shared)
  unsigned *next_cnt;  // shared
  int *vset, *pset;    // this round's sets (shared)
  unsigned next_round;
  int n;               // propagators: segment s has the set key n + s
  __device__ __forceinline__ bool claim(int u) const {
    const int t = local_insert<LP_LOG>(pset, u >= 0 ? u : n + ~u);
    return t > 0 || (t < 0 && atomicMax(u >= 0 ? pstamp + u : sstamp + ~u, next_round) < next_round);
  }
  __device__ __forceinline__ void append(int u, unsigned slot) const {
    next[slot] = u;
    if (slot < (unsigned)LOCAL_CAP) next_q[slot] = u;
  }
  __device__ __forceinline__ void list_unit(int u) const {
    if (claim(u)) append(u, atomicAdd(next_cnt, 1u));
  }
  __device__ __forceinline__ void list_batch(const int *buf, int cnt, int stride) const {
    for (int j = 0; j < cnt; ++j) list_unit(buf[j * stride]);
  }
  __device__ __forceinline__ void expand(int2 r, int skip) const {
    for (int k0 = r.x; k0 < r.y; k0 += EXPAND) {
      int q[EXPAND];
#pragma unroll
      for (int j = 0; j < EXPAND; ++j) q[j] = k0 + j < r.y ? __ldg(adj + k0 + j) : NO_UNIT;
      unsigned take = 0;
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (q[j] != NO_UNIT && q[j] != skip && claim(q[j])) take |= 1u << j;
      if (!take) continue;
      unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (take & (1u << j)) append(q[j], slot++);
    }
  }
  __device__ __forceinline__ void schedule(int v, int2 r) const {
    const int fresh = local_insert<LV_LOG>(vset, v);
    if (fresh == 0) return;
    if (fresh < 0 && atomicMax(vstamp + v, next_round) >= next_round) return;
    expand(r, NO_UNIT);
  }
  __device__ __forceinline__ void schedule_but(int v, int2 r, int skip) const { expand(r, skip); }
};

// CTA 0 alone: rounds separated by one __syncthreads each while the frontier
// stays at most local_max (shared state rotates so that what a round clears
// was last read before the previous barrier).  Writes the round reached and
// the outcome to the control block, and on a hand-over the frontier size to
// the global counter (thread 0; the writes precede its release at the next
// grid barrier).
__device__ void run_local(const EvFixArgs &a, long long round, int *stack, int *defer, SegQueue *sq, SegWork *work,
                          unsigned long long &execs, unsigned long long &narrowed) {
  __shared__ LocalShared sh;
  const int tid = threadIdx.x;
  for (int i = tid; i < (1 << LV_LOG); i += blockDim.x) sh.vset[0][i] = sh.vset[1][i] = -1;
  for (int i = tid; i < (1 << LP_LOG); i += blockDim.x) sh.pset[0][i] = sh.pset[1][i] = -1;
  if (tid == 0) {
    sh.cnt[round % 3] = ld_relaxed(a.cnt + (round % 3) * CNT_STRIDE);
    sh.cnt[(round + 1) % 3] = 0u;
    sh.bits[round % 3] = 0u;
  }
  // (the first round clears what the second appends to and ors into)
  __syncthreads();
  {
    const unsigned items = sh.cnt[round % 3];
    const int *cur = (round & 1) ? a.list1 : a.list0;
    for (unsigned i = tid; i < items && i < (unsigned)LOCAL_CAP; i += blockDim.x)
      sh.q[round & 1][i] = __ldcg(cur + i);
  }
  __syncthreads();
  int state = EV_CONTINUE;
  for (;;) {
    const int p = (int)(round & 1), r3 = (int)(round % 3), n3 = (int)((round + 1) % 3), c3 = (int)((round + 2) % 3);
    const unsigned items = sh.cnt[r3];
    if (items > a.local_max) break;
    // the parity p ^ 1 sets and segment queue served round - 1; counter c3
    // was read before the last barrier, bits n3 (round - 2's) right after the
    // one before it
    for (int i = tid; i < (1 << LV_LOG); i += blockDim.x) sh.vset[p ^ 1][i] = -1;
    for (int i = tid; i < (1 << LP_LOG); i += blockDim.x) sh.pset[p ^ 1][i] = -1;
    if (tid == 0) {
      sh.cnt[c3] = 0u;
      sh.bits[n3] = 0u;
      sq[p ^ 1].n = sq[p ^ 1].head = 0;
    }
    LocalSched sc;
    sc.adj = a.adj;
    sc.pstamp = a.pstamp;
    sc.sstamp = a.sstamp;
    sc.vstamp = a.vstamp;
    sc.next = ((round + 1) & 1) ? a.list1 : a.list0;
    sc.next_q = sh.q[p ^ 1];
    sc.next_cnt = &sh.cnt[n3];
    sc.vset = sh.vset[p];
    sc.pset = sh.pset[p];
    sc.next_round = (unsigned)(round + 1);
    sc.n = (int)a.n;
    const int *cur = p ? a.list1 : a.list0;
    int failed = 0, changed = 0;
    for (unsigned i = tid; i < items && !failed; i += blockDim.x) {
      const int u = i < (unsigned)LOCAL_CAP ? sh.q[p][i] : __ldcg(cur + i);
      if (u < 0)
        queue_segment(u, sq[p], sc);
      else
        changed += run_entry(u, a, sc, stack, defer, a.chase, execs, failed);
    }
    if (a.nseg) {
      __syncthreads();
      changed += run_segment_phase(a, sc, sq[p], work, execs, failed);
    }
    narrowed += changed;
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((tid & 31) == 0 && bits) atomicOr(&sh.bits[r3], bits);
    __syncthreads();
    const unsigned b = sh.bits[r3];
    if (tid == 0 && (round & 15) == 0) atomicExch(&a.ctl->hb, (unsigned long long)round);
    ++round;
    if (b & 2u) {
      state = EV_FAILED;
      break;
    }
    if (!(b & 1u)) {
      state = EV_FIXPOINT;
      break;
    }
    if (a.max_rounds > 0 && round >= a.max_rounds) {
      state = EV_CAP;
      break;
    }
  }
  if (tid == 0) {
    // the grid runs round `round` from the global list (or, after a fixpoint,
    // the dense certifying round); it lists into the counter of round + 1
    if (state == EV_CONTINUE) a.cnt[(round % 3) * CNT_STRIDE] = sh.cnt[round % 3];
    a.cnt[((round + 1) % 3) * CNT_STRIDE] = 0u;
    // a dense round (the certifying one) may come next
    for (int k = 0; k < 3; ++k) a.ccnt[k * CNT_STRIDE] = a.dsum[k * CNT_STRIDE] = a.dflag[k * CNT_STRIDE] = 0u;
    a.ctl->ev_round = round;
    a.ctl->ev_state = state;
  }
}

// Dynamic shared memory: one segment workspace per warp (only when the
// bytecode has segments).
__global__ void __launch_bounds__(EV_BLOCK, 2) k_fixpoint_events(EvFixArgs a) {
  __shared__ unsigned s_bits[2], s_word[2];
  __shared__ int s_stack[CHASE_CAP * EV_BLOCK], s_defer[DEFER_CAP * EV_BLOCK];
  __shared__ SegQueue s_sq[2];
  extern __shared__ unsigned long long s_dyn_ev[];
  SegWork *work = reinterpret_cast<SegWork *>(s_dyn_ev);
  const int tid = threadIdx.x;
  const long long gtid = blockIdx.x * (long long)blockDim.x + tid;
  const long long gstride = (long long)gridDim.x * blockDim.x;
  const long long gwarp = gtid >> 5, nwarps = gstride >> 5;
  unsigned long long execs = 0, narrowed = 0, cert_execs = 0, cert_narrowed = 0;
  long long round = 0, nbar = 0;
  // Rounds are dense (round 0, the certifying sweep, and while many
  // variables narrow) or event rounds; an event round after a dense one first
  // expands the dense round's noted variables into its list.  Certifying
  // sweep: when an event round changes nothing, a dense round runs every
  // unit once, whatever the lists, stamps, chases and segment snapshots
  // recorded; if it narrows nothing the store is a fixpoint of every
  // propagator, and if it narrows the rounds go on.
  bool dense = true, expand = false, certifying = false;
  // variables noted by the last DENSE_WINDOW dense rounds of this stretch of dense rounds
  long long hist[DENSE_WINDOW];
  int stretch = 0;
  int state = EV_CONTINUE;
  if (tid == 0) {
    s_bits[0] = s_bits[1] = 0u;
    s_sq[0].n = s_sq[0].head = s_sq[1].n = s_sq[1].head = 0;
  }
  __syncthreads();
  for (;;) {
    const int p = (int)(nbar & 1), rp = (int)(round & 1);
    if (dense) {
      // counters: this round's noted variables and flag were cleared before
      // it; the event lists of the next two rounds (an expansion lists into
      // round + 1's) are cleared here, nobody reads them in a dense round
      if (blockIdx.x == 0 && tid == 0) {
        a.cnt[((round + 1) % 3) * CNT_STRIDE] = 0u;
        a.cnt[((round + 2) % 3) * CNT_STRIDE] = 0u;
        a.ccnt[((round + 1) % 3) * CNT_STRIDE] = 0u;
        a.dsum[((round + 1) % 3) * CNT_STRIDE] = 0u;
        a.dflag[((round + 1) % 3) * CNT_STRIDE] = 0u;
      }
      if (tid == 0) s_sq[0].n = s_sq[0].head = s_sq[1].n = s_sq[1].head = 0;
      const DenseSched ds = dense_sched(a, round);
      int failed = 0;
      const unsigned long long execs0 = execs;
      int changed = run_dense(a, ds, gtid, gstride, execs, failed);
      if (a.nseg) {
        SegWork &w = work[tid >> 5];
        failed = __any_sync(0xFFFFFFFFu, failed) ? 1 : 0;
        for (long long sg = gwarp; sg < a.nseg && !failed; sg += nwarps)
          changed += run_segment(a, ds, (int)sg, w, false, true, execs, failed);
      }
      narrowed += changed;
      if (certifying) {
        cert_execs += execs - execs0;
        cert_narrowed += changed;
      }
      const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
      if ((tid & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
      __syncthreads();
      if (tid == 0) {
        const unsigned b = s_bits[p];
        s_bits[p] = 0u;
        s_word[p] = grid_sync_rot(a.ctl, gridDim.x, nbar, b & 1u, b & 2u, a.timeout_ns);
      }
      __syncthreads();
      const unsigned w = s_word[p];
      ++nbar;
      const long long noted = (long long)ld_relaxed(a.ccnt + (round % 3) * CNT_STRIDE);
      const long long degs = (long long)ld_relaxed(a.dsum + (round % 3) * CNT_STRIDE);
      const unsigned again = ld_relaxed(a.dflag + (round % 3) * CNT_STRIDE);
      ++round;
      const bool was_certifying = certifying;
      certifying = false;
      if (w & BIT_ERROR) {
        state = EV_ERROR;
        break;
      }
      if (w & BIT_FAILED) {
        state = EV_FAILED;
        break;
      }
      if (!(w & BIT_CHANGED)) {
        // every unit ran and nothing narrowed: this round certified the fixpoint
        if (!was_certifying) cert_execs += execs - execs0;
        state = EV_FIXPOINT;
        break;
      }
      if (a.max_rounds > 0 && round >= a.max_rounds) {
        state = EV_CAP;
        break;
      }
      dense = again || (a.dense_div > 0 && degs * a.dense_div >= a.n &&
                        (stretch < DENSE_WINDOW || noted * 8 <= hist[stretch % DENSE_WINDOW] * 7));
      hist[stretch % DENSE_WINDOW] = noted;
      stretch = dense ? stretch + 1 : 0;
      expand = !dense;
      continue;
    }
    if (expand) {
      // the units of the variables dense round - 1 noted, listed for this round
      const EvSched sc = ev_sched(a, round - 1);
      const int *cl = ((round - 1) & 1) ? a.cvl1 : a.cvl0;
      const long long noted = (long long)ld_relaxed(a.ccnt + ((round - 1) % 3) * CNT_STRIDE);
      for (long long j = gtid; j < noted; j += gstride) {
        const int v = __ldcg(cl + j);
        sc.schedule(v, make_int2(__ldg(a.adj_ptr + v), __ldg(a.adj_ptr + v + 1)));
      }
      __syncthreads();
      if (tid == 0) s_word[p] = grid_sync_rot(a.ctl, gridDim.x, nbar, 0, 0, a.timeout_ns);
      __syncthreads();
      ++nbar;
      if (s_word[p] & BIT_ERROR) {
        state = EV_ERROR;
        break;
      }
      expand = false;
      continue;
    }
    const long long items = (long long)ld_relaxed(a.cnt + (round % 3) * CNT_STRIDE);
    if (items <= (long long)a.local_max) {
      // small frontier: CTA 0 runs the rounds, everyone meets at the next grid barrier
      if (blockIdx.x == 0) run_local(a, round, s_stack + tid, s_defer + tid, s_sq, work, execs, narrowed);
      __syncthreads();
      if (tid == 0) {
        // whatever round comes next starts with empty segment queues
        s_sq[0].n = s_sq[0].head = s_sq[1].n = s_sq[1].head = 0;
        s_word[p] = grid_sync_rot(a.ctl, gridDim.x, nbar, 0, 0, a.timeout_ns, &a.ctl->hb);
      }
      __syncthreads();
      ++nbar;
      if (s_word[p] & BIT_ERROR) {
        state = EV_ERROR;
        break;
      }
      round = __ldcg(&a.ctl->ev_round);
      state = __ldcg(&a.ctl->ev_state);
      if (state == EV_FIXPOINT && a.certify) {
        if (a.max_rounds > 0 && round >= a.max_rounds) {
          state = EV_CAP;  // no round left for the certifying one
          break;
        }
        dense = certifying = true;
        state = EV_CONTINUE;
        continue;
      }
      if (state != EV_CONTINUE) break;
      continue;
    }
    // the counter of round + 2 was last read in round - 1, the noted-variable
    // counter of round + 1 in the expansion before round - 1; the other
    // segment queue was last used in round - 1
    if (blockIdx.x == 0 && tid == 0) {
      a.cnt[((round + 2) % 3) * CNT_STRIDE] = 0u;
      a.ccnt[((round + 1) % 3) * CNT_STRIDE] = 0u;
      a.dsum[((round + 1) % 3) * CNT_STRIDE] = 0u;
      a.dflag[((round + 1) % 3) * CNT_STRIDE] = 0u;
    }
    if (tid == 0) s_sq[rp ^ 1].n = s_sq[rp ^ 1].head = 0;
    int failed = 0;
    int changed = run_frontier(a, round, items, gtid, gstride, s_stack + tid, s_defer + tid, s_sq[rp], execs, failed);
    if (a.nseg) {
      __syncthreads();
      changed += run_segment_phase(a, ev_sched(a, round), s_sq[rp], work, execs, failed);
    }
    narrowed += changed;
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((tid & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
    __syncthreads();
    if (tid == 0) {
      // read and clear: the next grid round with this parity may come after
      // a local phase, which advances nbar without a grid round of the other
      // parity (a stale changed bit would then report a change that did not
      // happen)
      const unsigned b = s_bits[p];
      s_bits[p] = 0u;
      s_word[p] = grid_sync_rot(a.ctl, gridDim.x, nbar, b & 1u, b & 2u, a.timeout_ns);
    }
    __syncthreads();
    const unsigned w = s_word[p];
    ++nbar;
    ++round;
    if (w & BIT_ERROR) {
      state = EV_ERROR;
      break;
    }
    if (w & BIT_FAILED) {
      state = EV_FAILED;
      break;
    }
    if (a.max_rounds > 0 && round >= a.max_rounds && (w & BIT_CHANGED || a.certify)) {
      state = EV_CAP;  // still changing, or no round left for the certifying one
      break;
    }
    if (!(w & BIT_CHANGED)) {
      if (a.certify) {
        dense = certifying = true;
        continue;
      }
      state = EV_FIXPOINT;
      break;
    }
  }
  execs = warp_sum64(execs);
  narrowed = warp_sum64(narrowed);
  cert_execs = warp_sum64(cert_execs);
  cert_narrowed = warp_sum64(cert_narrowed);
  if ((tid & 31) == 0) {
    if (execs) atomicAdd(&a.ctl->executions, execs);
    if (narrowed) atomicAdd(&a.ctl->narrowed, narrowed);
    if (cert_execs) atomicAdd(&a.ctl->cert_execs, cert_execs);
    if (cert_narrowed) atomicAdd(&a.ctl->cert_narrowed, cert_narrowed);
  }
  if (blockIdx.x == 0 && tid == 0) {
    a.ctl->rounds = round;
    if (state == EV_FAILED) a.ctl->failed = 1;
    if (state == EV_CAP) a.ctl->changed[0] = 1;
  }
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int fixpoint_events(pirgpu_ctx *ctx, const pir_opts &opts, pir_stats *stats) {
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  EventsGraph g;
  int r;
  // AC-1 rounds of the persistent kernel first, while a round still narrows
  // something in many of its CTAs: a dense round of this kernel (every unit,
  // noting the narrowed variables) costs several AC-1 rounds on an instance
  // that narrows everywhere
  pir_stats lead;
  std::memset(&lead, 0, sizeof(lead));
  if (opts.lead >= 0 && opts.max_rounds <= 0) {
    bool done = false;
    if ((r = ac1_lead(ctx, opts, opts.lead > 0 ? opts.lead : 8, &lead, &done))) return r;
    if (done) {
      if (lead.status == PIR_FAILED) ctx->failed = true;
      ctx->at_fixpoint = lead.status == PIR_OK;
      if (stats) *stats = lead;
      if (lead.status == PIR_BARRIER_TIMEOUT) set_err(ctx, lead.status, "grid barrier wait exceeded");
      return lead.status;
    }
  }
  if ((r = events_graph(ctx, &g, opts.segments >= 0))) return r;
  const size_t n = (size_t)ctx->n, nv = (size_t)ctx->nvars, ns = (size_t)g.nseg;
  // scratch: pstamp | sstamp | busy | valid | vstamp | cstamp | counters
  // (3 x list, noted, flag, degree sum; all cleared each run) | list 0 | list 1 | noted
  // 0 | noted 1 | segment snapshots
  const size_t o_s = align256(n * 4), o_b = o_s + align256(ns * 4), o_sv = o_b + align256(ns * 4),
               o_v = o_sv + align256(ns * 4), o_cs = o_v + align256(nv * 4), o_c = o_cs + align256(nv * 4),
               o_l0 = o_c + 12 * CNT_STRIDE * 4, o_l1 = o_l0 + align256(n * 4), o_n0 = o_l1 + align256(n * 4),
               o_n1 = o_n0 + align256(nv * 4), o_last = o_n1 + align256(nv * 4),
               bytes = o_last + align256((size_t)g.seg_nvar * 8);
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, bytes))) return r;
  char *base = (char *)ctx->d_scratch;
  PIR_CK(cudaMemsetAsync(base, 0, o_l0, ctx->stream));
  if ((r = reset_control(ctx))) return r;
  EvFixArgs a;
  a.bc = g.bc;
  a.adj_ptr = g.uptr;
  a.adj = g.uadj;
  a.store = ctx->d_store;
  a.pstamp = (unsigned *)base;
  a.sstamp = (unsigned *)(base + o_s);
  a.seg_busy = (int *)(base + o_b);
  a.seg_valid = (int *)(base + o_sv);
  a.seg_last = (int2 *)(base + o_last);
  a.vstamp = (unsigned *)(base + o_v);
  a.cnt = (unsigned *)(base + o_c);
  a.ccnt = a.cnt + 3 * CNT_STRIDE;
  a.dflag = a.cnt + 6 * CNT_STRIDE;
  a.dsum = a.cnt + 9 * CNT_STRIDE;
  a.cstamp = (unsigned *)(base + o_cs);
  a.list0 = (int *)(base + o_l0);
  a.list1 = (int *)(base + o_l1);
  a.cvl0 = (int *)(base + o_n0);
  a.cvl1 = (int *)(base + o_n1);
  a.nvars = ctx->nvars;
  a.dense_div = opts.dense > 0 ? opts.dense : (opts.dense < 0 ? 0 : 32);
  a.ctl = ctx->d_ctl;
  a.n = ctx->n;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.timeout_ns = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  a.local_max = opts.local_frontier > 0 ? (unsigned)opts.local_frontier : 256u;
  a.chase = opts.chase > 0 ? std::min(opts.chase, CHASE_MAX) : (opts.chase < 0 ? 0 : CHASE_DEFAULT);
  a.certify = opts.certify >= 0;
  a.nseg = g.nseg;
  a.seg_pptr = g.seg_pptr;
  a.seg_code = g.seg_code;
  a.seg_vptr = g.seg_vptr;
  a.seg_var = g.seg_var;
  a.in_seg = g.in_seg;
  a.seg_umask = g.seg_umask;
  const size_t dyn = g.nseg ? (size_t)EV_WARPS * sizeof(SegWork) : 0;
  if (dyn) PIR_CK(cudaFuncSetAttribute(k_fixpoint_events, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fixpoint_events, EV_BLOCK, dyn));
  if (occ < 1) return set_err(ctx, PIR_ECUDA, "event kernel does not fit on an SM");
  const int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ;
  const int grid =
      std::max(1, std::min(ctx->num_sms * per_sm, (int)std::min<size_t>((n + EV_BLOCK - 1) / EV_BLOCK, 1 << 20)));
  void *args[] = {&a};
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  PIR_CK(cudaLaunchCooperativeKernel((const void *)k_fixpoint_events, dim3(grid), dim3(EV_BLOCK), args, dyn,
                                     ctx->stream));
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  st.device_ms += lead.device_ms;
  st.rounds = h.rounds + lead.rounds;
  st.executions = (int64_t)h.executions + lead.executions;
  st.narrowed = (int64_t)h.narrowed + lead.narrowed;
  st.certify_executions = (int64_t)h.cert_execs;
  st.certify_narrowed = (int64_t)h.cert_narrowed;
  int status;
  if (h.status) status = h.status;
  else if (h.failed) status = PIR_FAILED;
  else if (h.changed[0]) status = PIR_TIMEOUT;
  else status = PIR_OK;
  if (status == PIR_FAILED) ctx->failed = true;
  ctx->at_fixpoint = status == PIR_OK;
  ctx->last_grid = grid;
  st.status = status;
  if (stats) *stats = st;
  if (status == PIR_BARRIER_TIMEOUT) set_err(ctx, status, "grid barrier wait exceeded %lld ns", a.timeout_ns);
  return status;
}

}  // namespace pirgpu
