// Event-driven fixpoint of one instance: pir_fixpoint with
// opts.sched = PIR_SCHED_EVENTS.
//
// lala-pc's driver sweeps every propagator until a sweep changes nothing
// (GaussSeidelIteration around PIR::deduce(int), tests/pir_test.cpp:60-62);
// the AC-1 kernels do the same, one sweep per round.  Here a round runs only
// the propagators that have a variable narrowed in the previous round (the
// first round runs all of them), found through the variable -> propagator
// adjacency.  Every propagator of pir.hpp:721-817 reads only its three
// intervals, so one whose intervals did not change since its last run (which
// changed nothing) cannot change anything: the run ends at the same fixpoint,
// or the same failure, as the sweeps, bit for bit (propagators are monotone,
// so the order of the runs does not matter).
//
// Rounds with a large frontier run on the whole grid, separated by the grid
// barrier.  A round whose frontier has at most `local_max` propagators runs
// on CTA 0 alone, separated by __syncthreads, while the other CTAs wait at
// the next grid barrier; CTA 0 hands back when the frontier grows or the run
// ends.  Deep, narrow propagation (a long chain) then costs a block barrier
// per round instead of a grid barrier.  Within a round, a thread that
// narrows a variable with few propagators runs them itself at once (see
// "Chasing" below), so a chain of such variables advances many links per
// round: on 1M vars / 4M propagators plus a 20,000-link chain whose upper
// bounds ripple back one link per round, ~20,000 rounds become a few hundred.
#include <algorithm>
#include <cstring>

#include "pir_engine.h"
#include "pir_kernels.cuh"

namespace pirgpu {

// Engine-order AoS bytecode and the variable -> propagator adjacency (CSR),
// built once per bytecode version (pir_batch.cu).
int events_graph(pirgpu_ctx *ctx, const int4 **bc, const int **adj_ptr, const int **adj);

namespace {

constexpr int EV_CONTINUE = 0, EV_FIXPOINT = 1, EV_FAILED = 2, EV_CAP = 3, EV_ERROR = 4;
constexpr int CNT_STRIDE = 32;  // counters one 128-byte line apart

struct EvFixArgs {
  const int4 *bc;  // {op, x, y, z} per propagator
  const int *adj_ptr, *adj;
  int2 *store;
  unsigned *pstamp;  // per propagator: the last round it is listed for
  unsigned *vstamp;  // per variable: the last round its propagators were listed for
  int *list0, *list1;  // frontier of round r: list0 for even r, list1 for odd r
  unsigned *cnt;     // frontier sizes: round r in cnt[(r % 3) * CNT_STRIDE]
  Control *ctl;
  long long n;
  long long max_rounds, timeout_ns;
  unsigned local_max;
  int chase;  // runs chased per frontier entry (0: none)
};

__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Chasing.  A run that narrows a variable with at most CHASE_DEG
// propagators runs them itself at once (up to `chase` runs per frontier
// entry, CHASE_CAP pending, in shared memory) instead of leaving them to the
// next round; every other narrowed variable has its propagators listed for
// the next round, and so has whatever is still pending when the runs run
// out.  A run is first repeated on its own results (up to CLOSE_RUNS runs;
// past that the propagator is listed), so the propagator that narrowed a
// variable is not chased with the variable's others.  Every propagator of a
// narrowed variable thus runs after the narrowing, at once or in the next
// round, which is all the event schedule needs (the propagators are
// monotone).  A deep chain of small variables then advances up to `chase`
// links per round instead of one.
// The budget is capped: a chase is dependent L2 round trips (a few us each,
// more when many chasers narrow the same variables), and the grid's other
// CTAs wait for the round at a barrier with a time limit.
constexpr int CHASE_DEG = 4, CHASE_CAP = 8, CLOSE_RUNS = 4, CHASE_DEFAULT = 64, CHASE_MAX = 256, DEFER_CAP = 8;

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
// round r lists its propagators for round r + 1 (the round stamps keep every
// variable expanded, and every propagator listed, at most once per round).
// The adjacency is walked EXPAND entries at a time: their loads and stamp
// atomics are independent (one memory round trip each per batch, not per
// entry), and the batch takes its list slots with one atomic.
constexpr int EXPAND = 8;

struct EvSched {
  const int *adj;
  unsigned *pstamp, *vstamp;
  int *next;
  unsigned *next_cnt;
  unsigned next_round;
  __device__ __forceinline__ void list_prop(int q) const {
    if (atomicMax(pstamp + q, next_round) < next_round) next[atomicAdd(next_cnt, 1u)] = q;
  }
  // Lists the cnt (<= DEFER_CAP) propagators buf[0], buf[stride], ...
  __device__ __forceinline__ void list_batch(const int *buf, int cnt, int stride) const {
    int q[DEFER_CAP];
    unsigned take = 0;
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j) q[j] = j < cnt ? buf[j * stride] : -1;
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j)
      if (q[j] >= 0 && atomicMax(pstamp + q[j], next_round) < next_round) take |= 1u << j;
    if (!take) return;
    unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
    for (int j = 0; j < DEFER_CAP; ++j)
      if (take & (1u << j)) next[slot++] = q[j];
  }
  // Lists v's propagators (adjacency range r) for the next round.
  __device__ __forceinline__ void schedule(int v, int2 r) const {
    if (atomicMax(vstamp + v, next_round) >= next_round) return;
    for (int k0 = r.x; k0 < r.y; k0 += EXPAND) {
      int q[EXPAND];
#pragma unroll
      for (int j = 0; j < EXPAND; ++j) q[j] = k0 + j < r.y ? __ldg(adj + k0 + j) : -1;
      unsigned take = 0;
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (q[j] >= 0 && atomicMax(pstamp + q[j], next_round) < next_round) take |= 1u << j;
      if (!take) continue;
      unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (take & (1u << j)) next[slot++] = q[j];
    }
  }
};

__device__ __forceinline__ EvSched ev_sched(const EvFixArgs &a, long long round) {
  EvSched sc;
  sc.adj = a.adj;
  sc.pstamp = a.pstamp;
  sc.vstamp = a.vstamp;
  sc.next = ((round + 1) & 1) ? a.list1 : a.list0;
  sc.next_cnt = a.cnt + ((round + 1) % 3) * CNT_STRIDE;
  sc.next_round = (unsigned)(round + 1);
  return sc;
}

// Runs frontier entry q and what it chases (stack: this thread's CHASE_CAP
// slots, blockDim.x apart; defer: its DEFER_CAP slots).  Returns the bounds
// narrowed.  A run whose variable is chased is itself listed for the next
// round: its repeat on its own results does not see what a concurrent run of
// the same propagator joined, and the next round reads the store after the
// barrier.  Those listings wait in `defer` and go out DEFER_CAP at a time
// (their stamp atomics in flight together), off the chase's critical path.
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
    if (k == close) sc.list_prop(q);
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
        for (int j = 0; j < CHASE_DEG; ++j)
          if (e[j] != q) stack[(sp++) * stride] = e[j];
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
      while (sp > 0) sc.list_prop(stack[(--sp) * stride]);
      break;
    }
    q = stack[(--sp) * stride];
    --budget;
  }
  if (dn) sc.list_batch(defer, dn, stride);
  return changed;
}

// Runs the frontier entries i = first, first + stride, ... < items of round
// `round` (round 0: every propagator).  Returns the bounds narrowed.
__device__ __forceinline__ int run_frontier(const EvFixArgs &a, long long round, long long items, long long first,
                                            long long stride, int *stack, int *defer, unsigned long long &execs,
                                            int &failed) {
  const EvSched sc = ev_sched(a, round);
  const int *cur = (round & 1) ? a.list1 : a.list0;
  int changed = 0;
  for (long long i = first; i < items && !failed; i += stride) {
    const int q = round == 0 ? (int)i : __ldcg(cur + i);
    changed += run_entry(q, a, sc, stack, defer, a.chase, execs, failed);
  }
  return changed;
}

// Rounds run by CTA 0 alone keep their bookkeeping in shared memory: the
// frontier's first LOCAL_CAP entries, the list counters, and the round's
// sets of expanded variables and listed propagators (open addressing, at
// most L_PROBE probes).  Every listed propagator's index also goes to the
// global list (a store nobody waits on), so a round whose frontier outgrows
// local_max hands over to the grid as it is.  A key that finds no free slot
// in its probe window falls back to the global round stamps; since slots
// only fill during a round, every thread that meets that key takes the same
// route, and each propagator is still listed at most once per round.  The
// stamps hold round numbers, which only grow, so the rounds run here leave
// them valid for later rounds.
constexpr int LOCAL_CAP = 256, LV_LOG = 10, LP_LOG = 11, L_PROBE = 16;

struct LocalShared {
  int q[2][LOCAL_CAP];       // frontier, by round parity
  int vset[2][1 << LV_LOG];  // variables expanded, by round parity
  int pset[2][1 << LP_LOG];  // propagators listed, by round parity
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
  const int *adj;
  unsigned *pstamp, *vstamp;
  int *next;           // global list of the next round
  int *next_q;         // its first LOCAL_CAP entries (shared)
  unsigned *next_cnt;  // shared
  int *vset, *pset;    // this round's sets (shared)
  unsigned next_round;
  __device__ __forceinline__ bool claim(int q) const {
    const int t = local_insert<LP_LOG>(pset, q);
    return t > 0 || (t < 0 && atomicMax(pstamp + q, next_round) < next_round);
  }
  __device__ __forceinline__ void append(int q, unsigned slot) const {
    next[slot] = q;
    if (slot < (unsigned)LOCAL_CAP) next_q[slot] = q;
  }
  __device__ __forceinline__ void list_prop(int q) const {
    if (claim(q)) append(q, atomicAdd(next_cnt, 1u));
  }
  __device__ __forceinline__ void list_batch(const int *buf, int cnt, int stride) const {
    for (int j = 0; j < cnt; ++j) list_prop(buf[j * stride]);
  }
  __device__ __forceinline__ void schedule(int v, int2 r) const {
    const int fresh = local_insert<LV_LOG>(vset, v);
    if (fresh == 0) return;
    if (fresh < 0 && atomicMax(vstamp + v, next_round) >= next_round) return;
    for (int k0 = r.x; k0 < r.y; k0 += EXPAND) {
      int q[EXPAND];
#pragma unroll
      for (int j = 0; j < EXPAND; ++j) q[j] = k0 + j < r.y ? __ldg(adj + k0 + j) : -1;
      unsigned take = 0;
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (q[j] >= 0 && claim(q[j])) take |= 1u << j;
      if (!take) continue;
      unsigned slot = atomicAdd(next_cnt, (unsigned)__popc(take));
#pragma unroll
      for (int j = 0; j < EXPAND; ++j)
        if (take & (1u << j)) append(q[j], slot++);
    }
  }
};

// CTA 0 alone: rounds separated by one __syncthreads each while the frontier
// stays at most local_max (shared state rotates so that what a round clears
// was last read before the previous barrier).  Writes the round reached and
// the outcome to the control block, and on a hand-over the frontier size to
// the global counter (thread 0; the writes precede its release at the next
// grid barrier).
__device__ void run_local(const EvFixArgs &a, long long round, int *stack, int *defer, unsigned long long &execs,
                          unsigned long long &narrowed) {
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
    // the parity p ^ 1 sets served round - 1; counter c3 was read before the
    // last barrier, bits n3 (round - 2's) right after the one before it
    for (int i = tid; i < (1 << LV_LOG); i += blockDim.x) sh.vset[p ^ 1][i] = -1;
    for (int i = tid; i < (1 << LP_LOG); i += blockDim.x) sh.pset[p ^ 1][i] = -1;
    if (tid == 0) {
      sh.cnt[c3] = 0u;
      sh.bits[n3] = 0u;
    }
    LocalSched sc;
    sc.adj = a.adj;
    sc.pstamp = a.pstamp;
    sc.vstamp = a.vstamp;
    sc.next = ((round + 1) & 1) ? a.list1 : a.list0;
    sc.next_q = sh.q[p ^ 1];
    sc.next_cnt = &sh.cnt[n3];
    sc.vset = sh.vset[p];
    sc.pset = sh.pset[p];
    sc.next_round = (unsigned)(round + 1);
    const int *cur = p ? a.list1 : a.list0;
    int failed = 0, changed = 0;
    for (unsigned i = tid; i < items && !failed; i += blockDim.x) {
      const int q = i < (unsigned)LOCAL_CAP ? sh.q[p][i] : __ldcg(cur + i);
      changed += run_entry(q, a, sc, stack, defer, a.chase, execs, failed);
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
    if (state == EV_CONTINUE) {
      // the grid runs round `round` from the global list
      a.cnt[(round % 3) * CNT_STRIDE] = sh.cnt[round % 3];
      a.cnt[((round + 1) % 3) * CNT_STRIDE] = 0u;
    }
    a.ctl->ev_round = round;
    a.ctl->ev_state = state;
  }
}

__global__ void __launch_bounds__(256, 2) k_fixpoint_events(EvFixArgs a) {
  __shared__ unsigned s_bits[2], s_word[2];
  __shared__ int s_stack[CHASE_CAP * 256], s_defer[DEFER_CAP * 256];
  const int tid = threadIdx.x;
  const long long gtid = blockIdx.x * (long long)blockDim.x + tid;
  const long long gstride = (long long)gridDim.x * blockDim.x;
  unsigned long long execs = 0, narrowed = 0;
  long long round = 0, nbar = 0;
  int state = EV_CONTINUE;
  if (tid == 0) s_bits[0] = s_bits[1] = 0u;
  __syncthreads();
  for (;;) {
    const long long items = round == 0 ? a.n : (long long)ld_relaxed(a.cnt + (round % 3) * CNT_STRIDE);
    const int p = (int)(nbar & 1);
    if (round > 0 && items <= (long long)a.local_max) {
      // small frontier: CTA 0 runs the rounds, everyone meets at the next grid barrier
      if (blockIdx.x == 0) run_local(a, round, s_stack + tid, s_defer + tid, execs, narrowed);
      __syncthreads();
      if (tid == 0) s_word[p] = grid_sync_rot(a.ctl, gridDim.x, nbar, 0, 0, a.timeout_ns, &a.ctl->hb);
      __syncthreads();
      ++nbar;
      if (s_word[p] & BIT_ERROR) {
        state = EV_ERROR;
        break;
      }
      round = __ldcg(&a.ctl->ev_round);
      state = __ldcg(&a.ctl->ev_state);
      if (state != EV_CONTINUE) break;
      continue;
    }
    // the counter of round + 2 was last read in round - 1
    if (blockIdx.x == 0 && tid == 0) a.cnt[((round + 2) % 3) * CNT_STRIDE] = 0u;
    int failed = 0;
    const int changed = run_frontier(a, round, items, gtid, gstride, s_stack + tid, s_defer + tid, execs, failed);
    narrowed += changed;
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((tid & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
    __syncthreads();
    if (tid == 0) {
      const unsigned b = s_bits[p];
      s_bits[p ^ 1] = 0u;
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
    if (!(w & BIT_CHANGED)) {
      state = EV_FIXPOINT;
      break;
    }
    if (a.max_rounds > 0 && round >= a.max_rounds) {
      state = EV_CAP;
      break;
    }
  }
  execs = warp_sum64(execs);
  narrowed = warp_sum64(narrowed);
  if ((tid & 31) == 0) {
    if (execs) atomicAdd(&a.ctl->executions, execs);
    if (narrowed) atomicAdd(&a.ctl->narrowed, narrowed);
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
  const int4 *bc = nullptr;
  const int *adj_ptr = nullptr, *adj = nullptr;
  int r;
  if ((r = events_graph(ctx, &bc, &adj_ptr, &adj))) return r;
  const size_t n = (size_t)ctx->n, nv = (size_t)ctx->nvars;
  // scratch: pstamp | vstamp | counters (cleared each run) | list 0 | list 1
  const size_t o_v = align256(n * 4), o_c = o_v + align256(nv * 4), o_l0 = o_c + 3 * CNT_STRIDE * 4,
               o_l1 = o_l0 + align256(n * 4), bytes = o_l1 + align256(n * 4);
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, bytes))) return r;
  char *base = (char *)ctx->d_scratch;
  PIR_CK(cudaMemsetAsync(base, 0, o_l0, ctx->stream));
  if ((r = reset_control(ctx))) return r;
  EvFixArgs a;
  a.bc = bc;
  a.adj_ptr = adj_ptr;
  a.adj = adj;
  a.store = ctx->d_store;
  a.pstamp = (unsigned *)base;
  a.vstamp = (unsigned *)(base + o_v);
  a.cnt = (unsigned *)(base + o_c);
  a.list0 = (int *)(base + o_l0);
  a.list1 = (int *)(base + o_l1);
  a.ctl = ctx->d_ctl;
  a.n = ctx->n;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.timeout_ns = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  a.local_max = opts.local_frontier > 0 ? (unsigned)opts.local_frontier : 256u;
  a.chase = opts.chase > 0 ? std::min(opts.chase, CHASE_MAX) : (opts.chase < 0 ? 0 : CHASE_DEFAULT);
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fixpoint_events, 256, 0));
  if (occ < 1) return set_err(ctx, PIR_ECUDA, "event kernel does not fit on an SM");
  const int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ;
  const int grid = std::max(1, std::min(ctx->num_sms * per_sm, (int)std::min<size_t>((n + 255) / 256, 1 << 20)));
  void *args[] = {&a};
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  PIR_CK(cudaLaunchCooperativeKernel((const void *)k_fixpoint_events, dim3(grid), dim3(256), args, 0, ctx->stream));
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  st.rounds = h.rounds;
  st.executions = (int64_t)h.executions;
  st.narrowed = (int64_t)h.narrowed;
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
