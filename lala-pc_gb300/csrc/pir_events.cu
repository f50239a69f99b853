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
// per round instead of a grid barrier.
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
};

__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Store policy: joins as RedStore does; the first narrowing of a variable in
// round r lists its propagators for round r + 1 (the round stamps keep every
// variable expanded, and every propagator listed, at most once per round).
// The adjacency is walked EXPAND entries at a time: their loads and stamp
// atomics are independent (one memory round trip each per batch, not per
// entry), and the batch takes its list slots with one atomic.
constexpr int EXPAND = 8;

struct EvStore {
  int2 *s;
  const int *adj_ptr, *adj;
  unsigned *pstamp, *vstamp;
  int *next;
  unsigned *next_cnt;
  unsigned next_round;
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + v);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ void schedule(int v) const {
    if (atomicMax(vstamp + v, next_round) >= next_round) return;
    const int b = __ldg(adj_ptr + v), e = __ldg(adj_ptr + v + 1);
    for (int k0 = b; k0 < e; k0 += EXPAND) {
      int q[EXPAND];
#pragma unroll
      for (int j = 0; j < EXPAND; ++j) q[j] = k0 + j < e ? __ldg(adj + k0 + j) : -1;
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
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&s[v].x), "r"(r.l) : "memory");
      ++n;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&s[v].y), "r"(r.u) : "memory");
      ++n;
    }
    if (n) {
      if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
      schedule(v);
    }
    return n;
  }
};

__device__ __forceinline__ EvStore ev_store(const EvFixArgs &a, long long round) {
  EvStore st;
  st.s = a.store;
  st.adj_ptr = a.adj_ptr;
  st.adj = a.adj;
  st.pstamp = a.pstamp;
  st.vstamp = a.vstamp;
  st.next = ((round + 1) & 1) ? a.list1 : a.list0;
  st.next_cnt = a.cnt + ((round + 1) % 3) * CNT_STRIDE;
  st.next_round = (unsigned)(round + 1);
  return st;
}

// Runs the frontier entries i = first, first + stride, ... < items of round
// `round` (round 0: every propagator).  Returns the bounds narrowed.
__device__ __forceinline__ int run_frontier(const EvFixArgs &a, long long round, long long items, long long first,
                                            long long stride, unsigned long long &execs, int &failed) {
  const EvStore st = ev_store(a, round);
  const int *cur = (round & 1) ? a.list1 : a.list0;
  int changed = 0;
  for (long long i = first; i < items; i += stride) {
    const int q = round == 0 ? (int)i : __ldcg(cur + i);
    const int4 b = __ldg(a.bc + q);
    const Itv ia = st.load(b.y), ib = st.load(b.z), ic = st.load(b.w);
    changed += deduce_loaded(b.x, b.y, b.z, b.w, ia, ib, ic, st, failed);
    ++execs;
  }
  return changed;
}

// CTA 0 alone: rounds separated by __syncthreads while the frontier stays at
// most local_max.  Writes the round reached and the outcome to the control
// block (thread 0; the write precedes its release at the next grid barrier).
__device__ void run_local(const EvFixArgs &a, long long round, unsigned long long &execs,
                          unsigned long long &narrowed) {
  __shared__ unsigned s_lb[2];
  __shared__ unsigned s_items;
  const int tid = threadIdx.x;
  if (tid == 0) s_lb[0] = s_lb[1] = 0u;
  int state = EV_CONTINUE;
  for (;;) {
    if (tid == 0) {
      s_items = ld_relaxed(a.cnt + (round % 3) * CNT_STRIDE);
      a.cnt[((round + 2) % 3) * CNT_STRIDE] = 0u;
    }
    __syncthreads();
    const unsigned items = s_items;
    if (items > a.local_max) break;
    const int p = (int)(round & 1);
    int failed = 0;
    const int changed = run_frontier(a, round, items, tid, blockDim.x, execs, failed);
    narrowed += changed;
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((tid & 31) == 0 && bits) atomicOr(&s_lb[p], bits);
    __syncthreads();
    const unsigned b = s_lb[p];
    if (tid == 0) {
      s_lb[p ^ 1] = 0u;
      if ((round & 15) == 0) atomicExch(&a.ctl->hb, (unsigned long long)round);
    }
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
    a.ctl->ev_round = round;
    a.ctl->ev_state = state;
  }
}

__global__ void __launch_bounds__(256, 2) k_fixpoint_events(EvFixArgs a) {
  __shared__ unsigned s_bits[2], s_word[2];
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
      if (blockIdx.x == 0) run_local(a, round, execs, narrowed);
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
    const int changed = run_frontier(a, round, items, gtid, gstride, execs, failed);
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
