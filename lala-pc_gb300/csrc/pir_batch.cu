// Batched fixpoints for sm_103a.
//
// * Uneven independent instances (pir_fixpoint_instances): a persistent grid of
//   CTAs steals instances, largest first; one CTA runs one instance's AC-1
//   rounds separated by __syncthreads.  The instance's store is staged in
//   shared memory when it fits (with its bytecode too when that also fits),
//   otherwise it stays in the L2-resident global store.
// * Search nodes (pir_fixpoint_nodes): the per-block store copies sharing one
//   bytecode of pir.hpp:182-195, batched 32 nodes per warp.  The node stores
//   are interleaved by node ([var][32 nodes] int2 per group), so one warp
//   applying one propagator to its 32 nodes reads each interval with one
//   coalesced 256-byte access and all lanes run the same opcode.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include <cooperative_groups.h>

#include "pir_csr.h"
#include "pir_engine.h"
#include "pir_segments.h"

namespace cg = cooperative_groups;

namespace pirgpu {

struct InstOut {
  int status;
  int rounds;
  unsigned long long ns;
  unsigned long long narrowed;
  unsigned long long execs;  // executions of the event-filtered rounds
};

struct NodeOut {
  int status;
  int rounds;
};

struct BatchState {
  int4 *d_bc = nullptr;
  size_t cap_bc = 0;
  long long *d_off = nullptr;  // chunk offsets | var offsets
  size_t cap_off = 0;
  int2 *d_store = nullptr;
  size_t cap_store = 0;
  int *d_aux = nullptr;  // order | next counter | lb/ub staging
  size_t cap_aux = 0;
  InstOut *d_iout = nullptr;
  size_t cap_iout = 0;
  int2 *d_nstore = nullptr;  // node groups
  size_t cap_nstore = 0;
  int *d_tight = nullptr;  // node tightenings: off | var | lb | ub
  size_t cap_tight = 0;
  NodeOut *d_nout = nullptr;
  size_t cap_nout = 0;
  int *d_nio = nullptr;  // per-node output staging
  size_t cap_nio = 0;
  // event-driven nodes: AoS bytecode, variable -> propagator adjacency, per-CTA scratch
  long long ev_version = -1;
  int ev_graph_nvars = -1;
  int4 *d_bc4 = nullptr;
  int *d_adj_ptr = nullptr, *d_adj = nullptr;
  std::vector<int> h_adj_ptr, h_adj;  // host copy of the adjacency (the segment builder reads it)
  // path segments of the single-instance event schedule (pir_segments.h)
  long long seg_version = -1;
  int seg_nvars = -1;
  int nseg = 0;
  long long seg_nvar = 0;
  int *d_uptr = nullptr, *d_uadj = nullptr, *d_seg_pptr = nullptr, *d_seg_code = nullptr, *d_seg_vptr = nullptr;
  unsigned *d_seg_var = nullptr, *d_in_seg = nullptr;
  unsigned long long *d_seg_umask = nullptr;
  int ev_slots = 0, ev_nvars = 0;  // per-CTA scratch slots allocated (grid <= slots)
  long long ev_n = 0;
  void *d_ev = nullptr;  // per-CTA scratch block
  size_t cap_ev = 0;
  int node_variant = 0;            // event node kernel variant chosen by pir_autotune_nodes (0: default)
  int *d_watch = nullptr;  // watched variables | their bounds per node
  size_t cap_watch = 0;
  int *h_stage = nullptr;  // pinned host staging of the installed instance bytecode
  size_t cap_stage = 0;
  unsigned char *d_ent = nullptr;  // entailed-at-base flags per propagator
  size_t cap_ent = 0;
  long long ent_store_version = -1, ent_bc_version = -1;
  // staged node batches (the search driver): pinned input / output staging,
  // their device images, and the graph of one batch (clear the counters,
  // copy in, node kernel, copy out), rebuilt when a buffer moves or the
  // kernel variant changes, else updated in place
  int32_t *h_sin = nullptr;
  size_t cap_sin = 0;
  char *h_sout = nullptr;
  size_t cap_sout = 0;
  void *d_sin = nullptr, *d_sout = nullptr;
  size_t cap_dsin = 0, cap_dsout = 0;
  cudaGraph_t sg = nullptr;
  cudaGraphExec_t sgx = nullptr;
  cudaGraphNode_t sg_in = nullptr, sg_kernel = nullptr, sg_out = nullptr;
  const void *sg_kfn = nullptr;
  const void *sg_bufs[4] = {nullptr, nullptr, nullptr, nullptr};
};

void destroy_batch_state(pirgpu_ctx *ctx) {
  BatchState *b = ctx->batch;
  if (!b) return;
  if (b->h_stage) cudaFreeHost(b->h_stage);
  if (b->sgx) cudaGraphExecDestroy(b->sgx);
  if (b->sg) cudaGraphDestroy(b->sg);
  if (b->h_sin) cudaFreeHost(b->h_sin);
  if (b->h_sout) cudaFreeHost(b->h_sout);
  void *ptrs[] = {b->d_bc,    b->d_off,    b->d_store, b->d_aux,     b->d_iout, b->d_nstore, b->d_tight,
                  b->d_nout, b->d_nio, b->d_bc4, b->d_adj_ptr, b->d_adj, b->d_ev, b->d_ent, b->d_watch,
                  b->d_sin, b->d_sout, b->d_uptr, b->d_uadj, b->d_seg_pptr, b->d_seg_code, b->d_seg_vptr,
                  b->d_seg_var, b->d_in_seg, b->d_seg_umask};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete b;
  ctx->batch = nullptr;
}

// ------------------------------------------------------ instance kernel -----

struct InstArgs {
  const int4 *op, *x, *y, *z;  // padded chunks; instance j owns [coff[j], coff[j+1])
  const long long *coff, *voff;
  int2 *store;
  const int *order;
  int ninst;
  int *next;
  InstOut *out;
  long long max_rounds;
  int smem_cap;
};

// pir.hpp:333-335 on the device: reified targets are met with [0, 1].
template <class S>
__device__ __forceinline__ void install_chunks(const Bytecode &bc, S &st) {
  int dummy = 0;
  for (int c = threadIdx.x; c < bc.nchunks; c += blockDim.x) {
    const int4 o = bc.op[c], X = bc.x[c];
    const int ops[4] = {o.x, o.y, o.z, o.w}, xs[4] = {X.x, X.y, X.z, X.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (ops[k] == OP_EQ || ops[k] == OP_LEQ) {
        const Itv seen = st.load(xs[k]);
        st.embed(xs[k], seen, mk(0, 1), dummy);
      }
  }
}

// GBC: the bytecode is in global memory (else it may be staged in shared memory).
template <bool GBC, class S>
__device__ __forceinline__ void cta_rounds(const Bytecode &bc, S &st, long long max_rounds, long long &rounds,
                                           int &failed, int &changed, unsigned long long &narrowed) {
  rounds = 0;
  for (;;) {
    int ch = 0, f = 0;
    // one propagator per thread and step (63 registers: two CTAs of 512 per SM)
    for (int c = threadIdx.x; c < bc.nchunks * 4; c += blockDim.x) ch += sweep_step<1, S, GBC>(bc, c, st, f);
    narrowed += ch;
    const int any_ch = __syncthreads_or(ch);
    const int any_f = __syncthreads_or(f);
    ++rounds;
    if (any_f || !any_ch || (max_rounds > 0 && rounds >= max_rounds)) {
      failed = any_f;
      changed = any_ch;
      return;
    }
  }
}

// ------------------------------------------- event-filtered instance rounds -
//
// opts.sched = PIR_SCHED_EVENTS for instances: round r runs a propagator only
// when one of its variables was narrowed in round r - 1 (round 0 runs every
// one).  A join marks its variable in round r's bitmap right after it lands,
// before the round's barrier, so a narrowing that a propagator did not see
// when it read puts that propagator into the next round.  A propagator skipped
// in round r therefore read, at its last run, the intervals it would read now,
// and a round that narrows nothing is a fixpoint, as in AC-1.  Three bitmaps
// of ceil(nvars / 32) words rotate: round r reads bitmap (r - 1) % 3, marks
// r % 3 and clears (r + 1) % 3, which no thread reads or marks in round r.
__host__ __device__ constexpr int mark_words(int nv) { return (nv + 31) >> 5; }
__host__ __device__ constexpr int mark_bytes(int nv) { return ((3 * mark_words(nv) * 4 + 15) / 16) * 16; }

__device__ __forceinline__ bool marked(const unsigned *m, int v) { return (m[v >> 5] >> (v & 31)) & 1u; }

template <class S>
struct MarkedStore {
  S s;
  unsigned *cur;  // round r's bitmap (shared memory)
  __device__ __forceinline__ Itv load(int v) const { return s.load(v); }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    const int n = s.embed(v, seen, r, failed);
    if (n) {
      const unsigned bit = 1u << (v & 31);
      if (!(*(volatile unsigned *)(cur + (v >> 5)) & bit)) atomicOr(cur + (v >> 5), bit);
    }
    return n;
  }
};

// Propagator i, if round r's filter lets it run (prev: bitmap of round r - 1,
// null in round 0); `ran` counts the executions.
template <bool GBC, class S>
__device__ __forceinline__ int marked_step(const Bytecode &bc, int i, S &st, const unsigned *prev, int &failed,
                                           int &ran) {
  const int o = bc_load<GBC>(reinterpret_cast<const int *>(bc.op) + i);
  if (o == OP_NOP) return 0;
  const int X = bc_load<GBC>(reinterpret_cast<const int *>(bc.x) + i);
  const int Y = bc_load<GBC>(reinterpret_cast<const int *>(bc.y) + i);
  const int Z = bc_load<GBC>(reinterpret_cast<const int *>(bc.z) + i);
  if (prev && !(marked(prev, X) | marked(prev, Y) | marked(prev, Z))) return 0;
  ++ran;
  const Itv a = st.load(X), b = st.load(Y), d = st.load(Z);
  return deduce_loaded(o, X, Y, Z, a, b, d, st, failed);
}

// One CTA's event-filtered rounds; marks: the three bitmaps in shared memory.
template <bool GBC, class S>
__device__ __forceinline__ void cta_rounds_marked(const Bytecode &bc, S &st, unsigned *marks, int nv,
                                                  long long max_rounds, long long &rounds, int &failed, int &changed,
                                                  unsigned long long &narrowed, unsigned long long &execs) {
  const int words = mark_words(nv);
  for (int w = threadIdx.x; w < words; w += blockDim.x) marks[w] = 0;
  __syncthreads();
  rounds = 0;
  for (;;) {
    const int r = (int)(rounds % 3);
    const unsigned *prev = rounds ? marks + ((r + 2) % 3) * words : nullptr;
    unsigned *nxt = marks + ((r + 1) % 3) * words;
    for (int w = threadIdx.x; w < words; w += blockDim.x) nxt[w] = 0;
    MarkedStore<S> ms{st, marks + r * words};
    int ch = 0, f = 0, ran = 0;
    for (int i = threadIdx.x; i < bc.nchunks * 4; i += blockDim.x) ch += marked_step<GBC>(bc, i, ms, prev, f, ran);
    narrowed += ch;
    execs += ran;
    const int any_ch = __syncthreads_or(ch);
    const int any_f = __syncthreads_or(f);
    ++rounds;
    if (any_f || !any_ch || (max_rounds > 0 && rounds >= max_rounds)) {
      failed = any_f;
      changed = any_ch;
      return;
    }
  }
}

template <bool MARKS>
__global__ void __launch_bounds__(512, 2) k_instances(InstArgs a) {
  extern __shared__ int4 sm[];
  __shared__ int s_k;
  for (;;) {
    if (threadIdx.x == 0) s_k = atomicAdd(a.next, 1);
    __syncthreads();
    const int k = s_k;
    __syncthreads();
    if (k >= a.ninst) return;
    const int j = a.order[k];
    const long long c0 = a.coff[j];
    const int nch = (int)(a.coff[j + 1] - c0);
    const long long v0 = a.voff[j];
    const int nv = (int)(a.voff[j + 1] - v0);
    const unsigned long long t0 = globaltimer();
    int2 *gs = a.store + v0;
    Bytecode bc;
    bc.op = a.op + c0;
    bc.x = a.x + c0;
    bc.y = a.y + c0;
    bc.z = a.z + c0;
    bc.nchunks = nch;
    long long rounds = 0;
    int failed = 0, changed = 0;
    unsigned long long narrowed = 0;
    unsigned long long execs = 0;
    const int store_bytes = ((nv * 8 + 15) / 16) * 16;
    // the three round bitmaps of the event-filtered rounds follow the store
    const int mbytes = MARKS ? mark_bytes(nv) : 0;
    if (store_bytes + mbytes <= a.smem_cap) {
      int2 *ss = reinterpret_cast<int2 *>(sm);
      unsigned *marks = reinterpret_cast<unsigned *>(sm + store_bytes / 16);
      for (int v = threadIdx.x; v < nv; v += blockDim.x) ss[v] = gs[v];
      Bytecode sb = bc;
      const bool bc_in_smem = store_bytes + mbytes + nch * 64 <= a.smem_cap;
      if (bc_in_smem) {
        int4 *b4 = sm + (store_bytes + mbytes) / 16;
        int4 *sop = b4, *sx = b4 + nch, *sy = b4 + 2 * nch, *sz = b4 + 3 * nch;
        for (int c = threadIdx.x; c < nch; c += blockDim.x) {
          sop[c] = bc.op[c];
          sx[c] = bc.x[c];
          sy[c] = bc.y[c];
          sz[c] = bc.z[c];
        }
        sb.op = sop;
        sb.x = sx;
        sb.y = sy;
        sb.z = sz;
      }
      __syncthreads();
      SmemStore st{ss};
      install_chunks(sb, st);
      __syncthreads();
      if constexpr (MARKS) {
        if (bc_in_smem)
          cta_rounds_marked<false>(sb, st, marks, nv, a.max_rounds, rounds, failed, changed, narrowed, execs);
        else
          cta_rounds_marked<true>(sb, st, marks, nv, a.max_rounds, rounds, failed, changed, narrowed, execs);
      } else {
        if (bc_in_smem)
          cta_rounds<false>(sb, st, a.max_rounds, rounds, failed, changed, narrowed);
        else
          cta_rounds<true>(sb, st, a.max_rounds, rounds, failed, changed, narrowed);
      }
      for (int v = threadIdx.x; v < nv; v += blockDim.x) gs[v] = ss[v];
    } else {
      GlobalStore gst{gs};
      install_chunks(bc, gst);
      __syncthreads();
      RedStore st{gs};
      if (MARKS && mbytes <= a.smem_cap)
        cta_rounds_marked<true>(bc, st, reinterpret_cast<unsigned *>(sm), nv, a.max_rounds, rounds, failed, changed,
                                narrowed, execs);
      else
        cta_rounds<true>(bc, st, a.max_rounds, rounds, failed, changed, narrowed);
    }
    narrowed = warp_sum64(narrowed);
    if ((threadIdx.x & 31) == 0 && narrowed) atomicAdd(&a.out[j].narrowed, narrowed);
    if constexpr (MARKS) {
      execs = warp_sum64(execs);
      if ((threadIdx.x & 31) == 0 && execs) atomicAdd(&a.out[j].execs, execs);
    }
    if (threadIdx.x == 0) {
      a.out[j].status = failed ? PIR_FAILED : (changed ? PIR_TIMEOUT : PIR_OK);
      a.out[j].rounds = (int)rounds;
      a.out[j].ns = globaltimer() - t0;
    }
    __syncthreads();
  }
}

// ------------------------------------------------ cluster instance kernel ---
//
// Instances whose store does not fit one CTA's shared memory run on a
// cluster of CLU CTAs: variable v lives in the shared memory of CTA
// (v % CLU) at slot v / CLU, and every CTA reads and joins remote slots
// through distributed shared memory.  The cluster's threads split the
// propagators; rounds end with a hardware cluster barrier, and the round's
// change / failure bits are OR-ed into rank 0's shared memory.  All CTAs of a
// cluster take the same branches, so every one runs the same barriers, and
// they leave together after a barrier that follows the last remote read.
constexpr int CLU = 8;

// The store of a large instance spread over the shared memory of its cluster
// (variable v in CTA v % CLU).  An interval is one 64-bit load of distributed
// shared memory (the cluster barrier between rounds orders them); joins are
// fire-and-forget cluster-scope reductions counted against the value read,
// as RedStore does in HBM (a concurrent tighter join can make that an
// over-count, which costs at most one more round).
constexpr int CLU_BLOCK = 1024;  // threads per CTA of the cluster kernel

struct DsmStore {
  int2 *mine;  // this CTA's slot array (generic address)
  // v's slot: slot v / CLU of CTA v % CLU, the same offset in that CTA's
  // shared memory (mapa)
  __device__ __forceinline__ int2 *slot(int v) const {
    unsigned long long a;
    asm("mapa.u64 %0, %1, %2;" : "=l"(a) : "l"(mine + (v >> 3)), "r"(v & (CLU - 1)));
    return reinterpret_cast<int2 *>(a);
  }
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = *slot(v);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0;
    int2 *p = slot(v);
    if (r.l > seen.l) {
      asm volatile("red.relaxed.cluster.max.s32 [%0], %1;" ::"l"(&p->x), "r"(r.l) : "memory");
      ++n;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.cluster.min.s32 [%0], %1;" ::"l"(&p->y), "r"(r.u) : "memory");
      ++n;
    }
    if (n && is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    return n;
  }
};

// The store of DsmStore with the round bitmaps of the event-filtered rounds:
// every CTA holds a full copy of each bitmap (at the same shared-memory offset
// in every CTA), so the filter reads only its own; a join marks its variable
// in all CLU copies of round r's bitmap with cluster-scope reductions, unless
// this CTA's copy already has it (then another join marked, or is marking,
// every copy before the round's cluster barrier).
struct MarkedDsm {
  DsmStore s;
  unsigned *cur;  // this CTA's copy of round r's bitmap (generic address)
  __device__ __forceinline__ Itv load(int v) const { return s.load(v); }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    const int n = s.embed(v, seen, r, failed);
    if (n) {
      const unsigned bit = 1u << (v & 31);
      unsigned *w = cur + (v >> 5);
      if (!(*(volatile unsigned *)w & bit)) {
#pragma unroll
        for (int q = 0; q < CLU; ++q) {
          unsigned long long pa;
          asm("mapa.u64 %0, %1, %2;" : "=l"(pa) : "l"(w), "r"(q));
          asm volatile("red.relaxed.cluster.or.b32 [%0], %1;" ::"l"(pa), "r"(bit) : "memory");
        }
      }
    }
    return n;
  }
};

struct CluArgs {
  const int4 *op, *x, *y, *z;
  const long long *coff, *voff;
  int2 *store;
  const int *order;  // the instances this kernel runs, largest first
  int ninst;
  int *next;
  InstOut *out;
  long long max_rounds;
  int smem_cap;  // dynamic shared memory per CTA
};

template <bool MARKS>
__global__ void __launch_bounds__(CLU_BLOCK, 1) k_instances_cluster(CluArgs a) {
  extern __shared__ int4 sm[];
  __shared__ int s_inst;
  __shared__ unsigned s_flags[3][2];  // rank 0's: [round % 3][changed, failed]
  __shared__ unsigned long long s_t0;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  int2 *mine = reinterpret_cast<int2 *>(sm);
  DsmStore st;
  st.mine = mine;
  unsigned *flags0 = cluster.map_shared_rank(&s_flags[0][0], 0);
  int *inst0 = cluster.map_shared_rank(&s_inst, 0);
  const int ctid = rank * blockDim.x + threadIdx.x, cstride = CLU * blockDim.x;
  for (;;) {
    cluster.sync();
    if (rank == 0 && threadIdx.x == 0) {
      s_inst = atomicAdd(a.next, 1);
      for (int q = 0; q < 3; ++q) s_flags[q][0] = s_flags[q][1] = 0;
    }
    cluster.sync();
    const int k = *inst0;
    // Every CTA has read rank 0's slot before any CTA may leave: a CTA must
    // not exit while another can still access its shared memory.
    cluster.sync();
    if (k >= a.ninst) break;
    const int j = a.order[k];
    const long long c0 = a.coff[j];
    const int nch = (int)(a.coff[j + 1] - c0);
    const long long v0 = a.voff[j];
    const int nv = (int)(a.voff[j + 1] - v0);
    int2 *gs = a.store + v0;
    if (rank == 0 && threadIdx.x == 0) s_t0 = globaltimer();
    // this CTA's slots: variables v = CLU * i + rank
    for (int i = threadIdx.x; CLU * i + rank < nv; i += blockDim.x) mine[i] = gs[CLU * i + rank];
    // event-filtered rounds: this CTA's copies of the three round bitmaps
    // follow its slots; round 0's starts clear
    const int slot_bytes = (((nv + CLU - 1) / CLU) * 8 + 15) / 16 * 16;
    const bool use_marks = MARKS && slot_bytes + mark_bytes(nv) <= a.smem_cap;
    const int words = mark_words(nv);
    unsigned *marks = reinterpret_cast<unsigned *>(sm + slot_bytes / 16);
    if (MARKS && use_marks)
      for (int w = threadIdx.x; w < words; w += blockDim.x) marks[w] = 0;
    Bytecode bc;
    bc.op = a.op + c0;
    bc.x = a.x + c0;
    bc.y = a.y + c0;
    bc.z = a.z + c0;
    bc.nchunks = nch;
    cluster.sync();
    int dummy = 0;
    for (int c = ctid; c < nch; c += cstride) {  // install: reified targets met with [0, 1]
      const int4 o = bc.op[c], X = bc.x[c];
      const int ops[4] = {o.x, o.y, o.z, o.w}, xs[4] = {X.x, X.y, X.z, X.w};
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ops[q] == OP_EQ || ops[q] == OP_LEQ) st.embed(xs[q], st.load(xs[q]), mk(0, 1), dummy);
    }
    cluster.sync();
    long long round = 0;
    unsigned changed_any = 0, failed_any = 0;
    unsigned long long narrowed = 0, execs = 0;
    for (;;) {
      const int par = (int)(round % 3);
      if (rank == 0 && threadIdx.x == 0) s_flags[(round + 1) % 3][0] = s_flags[(round + 1) % 3][1] = 0;
      int ch = 0, f = 0;
      if (MARKS && use_marks) {
        const unsigned *prev = round ? marks + ((par + 2) % 3) * words : nullptr;
        unsigned *nxt = marks + ((par + 1) % 3) * words;
        for (int w = threadIdx.x; w < words; w += blockDim.x) nxt[w] = 0;
        MarkedDsm ms{st, marks + par * words};
        int ran = 0;
        for (int i = ctid; i < nch * 4; i += cstride) ch += marked_step<true>(bc, i, ms, prev, f, ran);
        execs += ran;
      } else {
        // one propagator per thread and step: 1,024 threads of 64 registers
        // keep twice the warps of 512 x 4-wide steps resident
        for (int c = ctid; c < nch * 4; c += cstride) ch += sweep_step<1>(bc, c, st, f);
      }
      narrowed += ch;
      const int any_ch = __syncthreads_or(ch), any_f = __syncthreads_or(f);
      if (threadIdx.x == 0) {
        if (any_ch) atomicOr(flags0 + 2 * par, 1u);
        if (any_f) atomicOr(flags0 + 2 * par + 1, 1u);
      }
      cluster.sync();
      changed_any = *(volatile unsigned *)(flags0 + 2 * par);
      failed_any = *(volatile unsigned *)(flags0 + 2 * par + 1);
      ++round;
      if (failed_any || !changed_any || (a.max_rounds > 0 && round >= a.max_rounds)) break;
    }
    for (int i = threadIdx.x; CLU * i + rank < nv; i += blockDim.x) gs[CLU * i + rank] = mine[i];
    narrowed = warp_sum64(narrowed);
    if ((threadIdx.x & 31) == 0 && narrowed) atomicAdd(&a.out[j].narrowed, narrowed);
    if constexpr (MARKS) {
      execs = warp_sum64(execs);
      if ((threadIdx.x & 31) == 0 && execs) atomicAdd(&a.out[j].execs, execs);
    }
    if (rank == 0 && threadIdx.x == 0) {
      a.out[j].status = failed_any ? PIR_FAILED : (changed_any ? PIR_TIMEOUT : PIR_OK);
      a.out[j].rounds = (int)round;
      a.out[j].ns = globaltimer() - s_t0;
    }
  }
}

// ---------------------------------------------------------- node kernel -----

// One node's column of a node group: var v of the node of lane `lane` lives at
// s[v * 32 + lane].  Several warps update the same node, so joins are
// device-scope reductions.
struct NodeStore {
  int2 *s;  // already offset by the lane
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + (size_t)v * 32);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0;
    int2 *p = s + (size_t)v * 32;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&p->x), "r"(r.l) : "memory");
      ++n;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&p->y), "r"(r.u) : "memory");
      ++n;
    }
    if (n && is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    return n;
  }
};

struct NodeArgs {
  Bytecode bc;
  int nvars;
  const int2 *base;
  int2 *nstore;
  const int *off, *var, *lb, *ub;
  int nnodes, ngroups;
  int *next;
  NodeOut *out;
  unsigned long long *narrowed;
  long long max_rounds;
};

__global__ void __launch_bounds__(512) k_nodes(NodeArgs a) {
  __shared__ int s_g;
  __shared__ unsigned s_changed[2], s_failed[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_g = atomicAdd(a.next, 1);
    __syncthreads();
    const int g = s_g;
    __syncthreads();
    if (g >= a.ngroups) return;
    const int node = g * 32 + lane;
    const bool valid = node < a.nnodes;
    int2 *S = a.nstore + (size_t)g * a.nvars * 32;
    for (int v = warp; v < a.nvars; v += nwarps) S[(size_t)v * 32 + lane] = a.base[v];
    if (threadIdx.x < 2) {
      s_changed[threadIdx.x] = 0;
      s_failed[threadIdx.x] = 0;
    }
    __syncthreads();
    unsigned failed_mask = 0;
    if (warp == 0) {
      int f = 0;
      if (valid) {
        for (int k = a.off[node]; k < a.off[node + 1]; ++k) {
          int2 *p = S + (size_t)a.var[k] * 32 + lane;
          int2 t = *p;
          t.x = max(t.x, a.lb[k]);
          t.y = min(t.y, a.ub[k]);
          *p = t;
          f |= is_bot(mk(t.x, t.y));
        }
      }
      failed_mask = __ballot_sync(0xFFFFFFFFu, f);
      if (lane == 0) s_failed[1] = failed_mask;
    }
    __syncthreads();
    failed_mask = s_failed[1];
    const unsigned valid_mask = (g * 32 + 32 <= a.nnodes) ? 0xFFFFFFFFu : ((1u << (a.nnodes - g * 32)) - 1u);
    unsigned active = valid_mask & ~failed_mask;
    unsigned timeout_mask = 0;
    int node_rounds = 0;  // meaningful in warp 0
    long long round = 0;
    unsigned long long narrowed = 0;
    NodeStore st{S + lane};
    __syncthreads();
    while (active) {
      const int par = (int)(round & 1);
      if (threadIdx.x == 0) {
        s_changed[par ^ 1] = 0;
        s_failed[par ^ 1] = 0;
      }
      const bool me = (active >> lane) & 1u;
      int ch = 0, f = 0;
      for (int c = warp; c < a.bc.nchunks; c += nwarps) {
        const int4 o = __ldg(a.bc.op + c), X = __ldg(a.bc.x + c), Y = __ldg(a.bc.y + c), Z = __ldg(a.bc.z + c);
        if (!me) continue;
        const Itv a0 = st.load(X.x), b0 = st.load(Y.x), c0 = st.load(Z.x);
        const Itv a1 = st.load(X.y), b1 = st.load(Y.y), c1 = st.load(Z.y);
        const Itv a2 = st.load(X.z), b2 = st.load(Y.z), c2 = st.load(Z.z);
        const Itv a3 = st.load(X.w), b3 = st.load(Y.w), c3 = st.load(Z.w);
        ch += deduce_loaded(o.x, X.x, Y.x, Z.x, a0, b0, c0, st, f);
        ch += deduce_loaded(o.y, X.y, Y.y, Z.y, a1, b1, c1, st, f);
        ch += deduce_loaded(o.z, X.z, Y.z, Z.z, a2, b2, c2, st, f);
        ch += deduce_loaded(o.w, X.w, Y.w, Z.w, a3, b3, c3, st, f);
      }
      narrowed += ch;
      const unsigned cb = __ballot_sync(0xFFFFFFFFu, ch != 0), fb = __ballot_sync(0xFFFFFFFFu, f != 0);
      if (lane == 0) {
        if (cb) atomicOr(&s_changed[par], cb);
        if (fb) atomicOr(&s_failed[par], fb);
      }
      __syncthreads();
      const unsigned changed = s_changed[par] & active, failed = s_failed[par] & active;
      ++round;
      if ((active >> lane) & 1u) node_rounds = (int)round;
      failed_mask |= failed;
      active &= changed & ~failed;
      if (active && a.max_rounds > 0 && round >= a.max_rounds) {
        timeout_mask = active;
        active = 0;
      }
      __syncthreads();
    }
    narrowed = warp_sum64(narrowed);
    if (lane == 0 && narrowed) atomicAdd(a.narrowed, narrowed);
    if (warp == 0 && valid) {
      const unsigned bit = 1u << lane;
      a.out[node].status = (failed_mask & bit) ? PIR_FAILED : ((timeout_mask & bit) ? PIR_TIMEOUT : PIR_OK);
      a.out[node].rounds = node_rounds;
    }
    __syncthreads();
  }
}

// ------------------------------------------------- event-driven nodes -----
//
// One CTA per node, nodes stolen from a counter.  The base store is a fixpoint
// of the bytecode, so after the node's tightenings only propagators of a
// variable that changed in the previous round can change anything: round r
// runs exactly the propagators adjacent (variable -> propagator adjacency) to
// the variables that narrowed in round r - 1 (first round: the tightened
// variables).  A propagator none of whose variables changed since its last
// run is at its fixpoint, so when a round leaves no variable changed the
// store is the node's fixpoint, the one AC-1 rounds reach.
//
// Propagators entailed at the base store (ask, pir.hpp:417-438) are skipped:
// entailment survives narrowing and an entailed propagator narrows nothing
// (both checked exhaustively against the oracle), so they cannot change a
// node's fixpoint -- lala-pc's FixpointSubset idea (pir.hpp:874-884).
//
// A node's store is an overlay on the base store: each CTA keeps a working
// array that holds only the node's own narrowings (the whole integer range
// where it narrowed nothing, reset there after every node), and a read meets
// it with the base, which every CTA reads and nobody writes during the launch
// (L2 / L1 resident).  A shared-memory bitmap marks the variables the node
// narrowed, so reads of the others touch the base alone.  The base can change
// between launches without anything being reloaded.  Within a round, the
// expansion of the changed variables' adjacency is spread over the whole CTA
// (block scan of the degrees), and candidates, changed variables and touched
// variables are deduplicated in shared-memory hash sets; a set whose probe
// window is full falls back to epoch stamps in global memory for that key (a
// key takes the same path for as long as its set is not cleared).

constexpr int CAND_LOG = 11, CHG_LOG = 10, TOUCH_LOG = 11, MAX_PROBE = 16;

struct EvArgs {
  const int4 *bc;  // (op, x, y, z) per propagator, engine order
  long long n;
  int nvars;
  const int *adj_ptr, *adj;
  const unsigned char *ent;  // per propagator: entailed at the base store (skipped)
  const int2 *base;  // read-only during the launch
  int bitmap_words;  // words of the shared-memory bitmap of narrowed variables (0: none, every read meets both)
  int2 *out_store;  // node-major nnodes x nvars, or nullptr
  const int *watch;  // nwatch variables whose final bounds every node reports
  int nwatch;
  int2 *out_watch;   // nnodes x nwatch
  const int *off, *var, *lb, *ub;
  int nnodes;
  int *next;
  int2 *ws;          // grid x nvars: the node's narrowings, [INT_MIN, INT_MAX] elsewhere
  unsigned *vmark;   // grid x nvars: epoch a variable last entered a changed list (fallback)
  unsigned *tmark;   // grid x nvars: node tag a variable last entered the touched list (fallback)
  int *lists;        // grid x 3 x nvars: changed lists (2) and the touched list
  unsigned *pstamp;  // grid x n: epoch a propagator last became a candidate (fallback)
  int *cand;         // grid x n
  unsigned *epochs;  // grid
  NodeOut *out;
  unsigned long long *execs, *narrowed;
  unsigned long long *cert;  // certifying sweeps: [0] executions, [1] bounds narrowed
  long long max_rounds;
  int certify;  // end every node with a certifying sweep
};

// Insert `key` into the shared-memory set tab[1 << LOG] (-1 = free): 1 newly
// inserted, 0 already there, -1 no free slot within MAX_PROBE (Fibonacci
// hashing, linear probing).
template <int LOG>
__device__ __forceinline__ int set_insert(int *tab, int key) {
  unsigned h = ((unsigned)key * 2654435761u) >> (32 - LOG);
  for (int i = 0; i < MAX_PROBE; ++i) {
    const int prev = atomicCAS(tab + h, -1, key);
    if (prev == -1) return 1;
    if (prev == key) return 0;
    h = (h + 1) & ((1u << LOG) - 1u);
  }
  return -1;
}

template <int LOG>
__device__ __forceinline__ void set_clear(int *tab) {
  for (int i = threadIdx.x; i < (1 << LOG); i += blockDim.x) tab[i] = -1;
}

struct NodeEvStore {
  int2 *ws;              // the node's narrowings (overlay)
  const int2 *base;      // the base store
  unsigned *bits;        // shared-memory bitmap of the variables the node narrowed (null: none)
  unsigned *vmark, *tmark;
  int *dnext, *touched;
  int *nd, *nt;              // shared-memory counters
  int *chg_set, *touch_set;  // shared-memory sets (touch_set: only without the bitmap)
  unsigned epoch, tag;
  // base meet overlay; the overlay is read only for variables the node narrowed
  __device__ __forceinline__ Itv load(int v) const {
    const int2 b = __ldg(base + v);
    if (bits && !(bits[v >> 5] & (1u << (v & 31)))) return mk(b.x, b.y);
    const int2 t = __ldcg(ws + v);
    return mk(max(b.x, t.x), min(b.y, t.y));
  }
  // v narrowed: first time this round -> next changed list; first time this
  // node -> touched list (first: from the bitmap, -1 without it)
  __device__ __forceinline__ void note(int v, int first) const {
    int c = set_insert<CHG_LOG>(chg_set, v);
    if (c < 0) c = atomicMax(vmark + v, epoch) < epoch ? 1 : 0;
    if (c > 0) dnext[atomicAdd(nd, 1)] = v;
    int t = first;
    if (t < 0 && c > 0) {
      t = set_insert<TOUCH_LOG>(touch_set, v);
      if (t < 0) t = atomicExch(tmark + v, tag) != tag ? 1 : 0;
    }
    if (t > 0) touched[atomicAdd(nt, 1)] = v;
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&ws[v].x), "r"(r.l) : "memory");
      ++n;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&ws[v].y), "r"(r.u) : "memory");
      ++n;
    }
    if (n) {
      int first = -1;
      if (bits) {
        const unsigned m = 1u << (v & 31);
        first = (atomicOr(bits + (v >> 5), m) & m) ? 0 : 1;
      }
      note(v, first);
      if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    }
    return n;
  }
};

// Inclusive prefix sum of `x` over the CTA (blockDim.x a multiple of 32,
// at most 1024); s_warp holds 32 ints.
__device__ __forceinline__ int block_scan_incl(int x, int *s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  const int r = x + (warp ? s_warp[warp - 1] : 0);
  __syncthreads();
  return r;
}

// NB threads per CTA (one node per CTA); MINB: resident CTAs per SM the
// register budget is sized for (more nodes in flight against fewer registers
// per thread).
template <int NB, int MINB>
__global__ void __launch_bounds__(NB, MINB) k_nodes_events(EvArgs a) {
  __shared__ int s_node, s_ncand, s_nd[2], s_nt;
  __shared__ int s_cand_set[1 << CAND_LOG], s_chg_set[1 << CHG_LOG];
  __shared__ int s_beg[NB], s_end[NB], s_warp[32];
  // dynamic: the bitmap of narrowed variables (bitmap_words words), or else
  // the touched-variable set
  extern __shared__ unsigned s_dyn[];
  unsigned *bits = a.bitmap_words ? s_dyn : nullptr;
  int *s_touch_set = a.bitmap_words ? nullptr : reinterpret_cast<int *>(s_dyn);
  const size_t nv = (size_t)a.nvars;
  const int tid = threadIdx.x;
  int2 *ws = a.ws + blockIdx.x * nv;
  unsigned *vmark = a.vmark + blockIdx.x * nv, *tmark = a.tmark + blockIdx.x * nv;
  int *const dl0 = a.lists + blockIdx.x * 3 * nv, *const dl1 = dl0 + nv;  // changed lists
  int *touched = a.lists + blockIdx.x * 3 * nv + 2 * nv;
  unsigned *pstamp = a.pstamp + blockIdx.x * (size_t)a.n;
  int *cand = a.cand + blockIdx.x * (size_t)a.n;
  unsigned epoch = a.epochs[blockIdx.x];
  unsigned long long execs = 0, narrowed = 0, cert_execs = 0, cert_narrowed = 0;
  for (int i = tid; i < a.bitmap_words; i += blockDim.x) s_dyn[i] = 0u;  // then cleared word by word
  __syncthreads();
  for (;;) {
    if (tid == 0) {
      s_node = atomicAdd(a.next, 1);
      s_nd[0] = s_nd[1] = 0;
      s_nt = 0;
    }
    set_clear<CHG_LOG>(s_chg_set);
    if (!bits) set_clear<TOUCH_LOG>(s_touch_set);
    __syncthreads();
    const int node = s_node;
    if (node >= a.nnodes) break;
    ++epoch;
    const unsigned tag = epoch;
    NodeEvStore st{ws, a.base, bits, vmark, tmark, dl0, touched, &s_nd[0], &s_nt, s_chg_set, s_touch_set,
                   epoch, tag};
    // tightenings: meets, the changed ones start the first changed list
    int f = 0;
    const int k0 = a.off[node], k1 = a.off[node + 1];
    for (int k = k0 + tid; k < k1; k += blockDim.x) {
      const int v = a.var[k];
      int dummy = 0;
      st.embed(v, st.load(v), mk(a.lb[k], a.ub[k]), dummy);
    }
    __syncthreads();
    for (int k = k0 + tid; k < k1; k += blockDim.x) f |= is_bot(st.load(a.var[k]));
    int failed = __syncthreads_or(f);
    int cur = 0;
    long long round = 0;
    int status = PIR_OK;
    // Certifying sweep: when a round lists nothing, one more round runs every
    // non-entailed propagator of every variable the node narrowed (the touched
    // list), whatever the wake lists, stamps and sets recorded.  A propagator
    // none of whose variables the node narrowed reads the base store, which is
    // a fixpoint, so a sweep without narrowing proves the node's store a
    // fixpoint; a sweep that narrows lists as any round does and the rounds go
    // on (and end with another sweep).
    bool certified = !a.certify;
    while (!failed) {
      const bool certifying = s_nd[cur] == 0;
      if (certifying && certified) break;
      if (a.max_rounds > 0 && round >= a.max_rounds) {
        status = PIR_TIMEOUT;
        break;
      }
      ++round;
      ++epoch;
      if (tid == 0) {
        s_ncand = 0;
        s_nd[cur ^ 1] = 0;
      }
      set_clear<CAND_LOG>(s_cand_set);
      set_clear<CHG_LOG>(s_chg_set);
      __syncthreads();
      // candidates: the non-entailed propagators adjacent to the variables
      // changed last round (certifying: to every variable the node narrowed),
      // the adjacency spread over the CTA
      const int nd = certifying ? s_nt : s_nd[cur];
      const int *src = certifying ? touched : (cur ? dl1 : dl0);
      for (int c0 = 0; c0 < nd; c0 += blockDim.x) {
        const int i = c0 + tid;
        int beg = 0, deg = 0;
        if (i < nd) {
          const int v = src[i];
          beg = __ldg(a.adj_ptr + v);
          deg = __ldg(a.adj_ptr + v + 1) - beg;
        }
        const int incl = block_scan_incl(deg, s_warp);
        s_beg[tid] = beg;
        s_end[tid] = incl;
        __syncthreads();
        const int total = s_end[blockDim.x - 1];
        for (int j = tid; j < total; j += blockDim.x) {
          int lo = 0, hi = (int)blockDim.x - 1;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (s_end[mid] > j) hi = mid;
            else lo = mid + 1;
          }
          const int first = lo ? s_end[lo - 1] : 0;
          const int p = __ldg(a.adj + s_beg[lo] + (j - first));
          if (a.ent && a.ent[p]) continue;
          int c = set_insert<CAND_LOG>(s_cand_set, p);
          if (c < 0) c = atomicMax(pstamp + p, epoch) < epoch ? 1 : 0;
          if (c > 0) cand[atomicAdd(&s_ncand, 1)] = p;
        }
        __syncthreads();
      }
      NodeEvStore rs{ws, a.base, bits, vmark, tmark, cur ? dl0 : dl1, touched, &s_nd[cur ^ 1], &s_nt, s_chg_set,
                     s_touch_set, epoch, tag};
      const int nc = s_ncand;
      int f2 = 0, ch = 0;
      for (int i = tid; i < nc; i += blockDim.x) {
        const int4 b = __ldg(a.bc + cand[i]);
        const Itv ia = rs.load(b.y), ib = rs.load(b.z), ic = rs.load(b.w);
        ch += deduce_loaded(b.x, b.y, b.z, b.w, ia, ib, ic, rs, f2);
        ++execs;
      }
      narrowed += ch;
      if (certifying) {
        cert_narrowed += ch;
        if (tid == 0) cert_execs += nc;
      }
      failed = __syncthreads_or(f2);
      cur ^= 1;
      // a sweep that narrowed nothing certifies; one that narrowed resumes the rounds
      if (certifying) certified = s_nd[cur] == 0;
    }
    if (failed) status = PIR_FAILED;
    if (tid == 0) {
      a.out[node].status = status;
      a.out[node].rounds = (int)round;
    }
    if (a.out_store) {
      int2 *dst = a.out_store + (size_t)node * nv;
      for (size_t v = tid; v < nv; v += blockDim.x) {
        const Itv t = st.load((int)v);
        dst[v] = make_int2(t.l, t.u);
      }
    }
    for (int k = tid; k < a.nwatch; k += blockDim.x) {
      const Itv t = st.load(a.watch[k]);
      a.out_watch[(size_t)node * a.nwatch + k] = make_int2(t.l, t.u);
    }
    __syncthreads();
    // the overlay back to the whole range where this node narrowed
    // (every bit set during the node belongs to a touched variable)
    const int nt = s_nt;
    for (int i = tid; i < nt; i += blockDim.x) {
      const int v = touched[i];
      ws[v] = make_int2(INT_MIN, INT_MAX);
      if (bits) bits[v >> 5] = 0u;
    }
    __syncthreads();
  }
  if (tid == 0) a.epochs[blockIdx.x] = epoch;
  execs = warp_sum64(execs);
  narrowed = warp_sum64(narrowed);
  cert_narrowed = warp_sum64(cert_narrowed);
  if ((tid & 31) == 0) {
    if (execs) atomicAdd(a.execs, execs);
    if (narrowed) atomicAdd(a.narrowed, narrowed);
    if (cert_narrowed) atomicAdd(a.cert + 1, cert_narrowed);
  }
  if (tid == 0 && cert_execs) atomicAdd(a.cert, cert_execs);
}

// ------------------------------------------------- one warp per node -------
//
// The same node rounds as k_nodes_events on one warp instead of one CTA:
// __syncwarp instead of block barriers, a warp scan of the degrees for the
// adjacency expansion, and about 6 KB of shared memory per node in flight,
// so an SM holds several times more nodes (a node's frontier is a few hundred
// propagators: a CTA's warps spent most of each round at its barriers).  The
// narrowed-variable bitmap is hashed (variable v sets bit v mod WBITS): a
// false positive only costs a read of the overlay, and the touched list takes
// each variable once through its global stamp (tmark), not through the bit.
constexpr int WCAND_LOG = 10, WCHG_LOG = 9, WBITS_LOG = 13;

struct WarpNodeShared {
  int cand_set[1 << WCAND_LOG];
  int chg_set[1 << WCHG_LOG];
  unsigned bits[(1 << WBITS_LOG) / 32];
  int beg[32], end[32];
  int ncand, nd[2], nt;
};

template <int LOG>
__device__ __forceinline__ void warp_set_clear(int *tab) {
  for (int i = threadIdx.x & 31; i < (1 << LOG); i += 32) tab[i] = -1;
}

// The node store of a warp: base meet overlay, the overlay read only where
// the hashed bitmap says the node may have narrowed.
struct WarpNodeStore {
  int2 *ws;
  const int2 *base;
  unsigned *bits;
  unsigned *vmark, *tmark;
  int *dnext, *touched;
  int *nd, *nt;
  int *chg_set;
  unsigned epoch, tag;
  __device__ __forceinline__ bool maybe(int v) const {
    const unsigned h = (unsigned)v & ((1u << WBITS_LOG) - 1u);
    return (bits[h >> 5] >> (h & 31)) & 1u;
  }
  __device__ __forceinline__ Itv load(int v) const {
    const int2 b = __ldg(base + v);
    if (!maybe(v)) return mk(b.x, b.y);
    const int2 t = __ldcg(ws + v);
    return mk(max(b.x, t.x), min(b.y, t.y));
  }
  __device__ __forceinline__ void note(int v) const {
    int c = set_insert<WCHG_LOG>(chg_set, v);
    if (c < 0) c = atomicMax(vmark + v, epoch) < epoch ? 1 : 0;
    if (c > 0) dnext[atomicAdd(nd, 1)] = v;
    if (atomicExch(tmark + v, tag) != tag) touched[atomicAdd(nt, 1)] = v;
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0;
    if (r.l > seen.l) {
      asm volatile("red.relaxed.gpu.global.max.s32 [%0], %1;" ::"l"(&ws[v].x), "r"(r.l) : "memory");
      ++n;
    }
    if (r.u < seen.u) {
      asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(&ws[v].y), "r"(r.u) : "memory");
      ++n;
    }
    if (n) {
      const unsigned h = (unsigned)v & ((1u << WBITS_LOG) - 1u);
      atomicOr(bits + (h >> 5), 1u << (h & 31));
      note(v);
      if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    }
    return n;
  }
};

// WPB warps per CTA, each running nodes one after the other (work stealing);
// per-node scratch slots are per warp (slot = CTA * WPB + warp).
template <int WPB, int MINB>
__global__ void __launch_bounds__(WPB * 32, MINB) k_nodes_warp(EvArgs a) {
  extern __shared__ unsigned long long s_dyn_w[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpNodeShared &sh = reinterpret_cast<WarpNodeShared *>(s_dyn_w)[warp];
  const size_t nv = (size_t)a.nvars;
  const size_t slot = (size_t)blockIdx.x * WPB + warp;
  int2 *ws = a.ws + slot * nv;
  unsigned *vmark = a.vmark + slot * nv, *tmark = a.tmark + slot * nv;
  int *const dl0 = a.lists + slot * 3 * nv, *const dl1 = dl0 + nv;  // changed lists
  int *touched = dl0 + 2 * nv;
  unsigned *pstamp = a.pstamp + slot * (size_t)a.n;
  int *cand = a.cand + slot * (size_t)a.n;
  unsigned epoch = a.epochs[slot];
  unsigned long long execs = 0, narrowed = 0, cert_execs = 0, cert_narrowed = 0;
  for (int i = lane; i < (1 << WBITS_LOG) / 32; i += 32) sh.bits[i] = 0u;
  __syncwarp();
  for (;;) {
    int node = 0;
    if (lane == 0) node = atomicAdd(a.next, 1);
    node = __shfl_sync(0xFFFFFFFFu, node, 0);
    if (node >= a.nnodes) break;
    if (lane == 0) {
      sh.nd[0] = sh.nd[1] = 0;
      sh.nt = 0;
    }
    warp_set_clear<WCHG_LOG>(sh.chg_set);
    __syncwarp();
    ++epoch;
    const unsigned tag = epoch;
    WarpNodeStore st{ws, a.base, sh.bits, vmark, tmark, dl0, touched, &sh.nd[0], &sh.nt, sh.chg_set, epoch, tag};
    const int k0 = a.off[node], k1 = a.off[node + 1];
    for (int k = k0 + lane; k < k1; k += 32) {
      const int v = a.var[k];
      int dummy = 0;
      st.embed(v, st.load(v), mk(a.lb[k], a.ub[k]), dummy);
    }
    __syncwarp();
    int f = 0;
    for (int k = k0 + lane; k < k1; k += 32) f |= is_bot(st.load(a.var[k]));
    int failed = __any_sync(0xFFFFFFFFu, f) ? 1 : 0;
    int cur = 0;
    long long round = 0;
    int status = PIR_OK;
    // the certifying sweep of k_nodes_events: when a round lists nothing, one
    // more round over the propagators of every variable the node narrowed
    bool certified = !a.certify;
    while (!failed) {
      __syncwarp();
      const bool certifying = sh.nd[cur] == 0;
      if (certifying && certified) break;
      if (a.max_rounds > 0 && round >= a.max_rounds) {
        status = PIR_TIMEOUT;
        break;
      }
      ++round;
      ++epoch;
      const int nd = certifying ? sh.nt : sh.nd[cur];
      const int *src = certifying ? touched : (cur ? dl1 : dl0);
      __syncwarp();
      if (lane == 0) {
        sh.ncand = 0;
        sh.nd[cur ^ 1] = 0;
      }
      warp_set_clear<WCAND_LOG>(sh.cand_set);
      warp_set_clear<WCHG_LOG>(sh.chg_set);
      __syncwarp();
      for (int c0 = 0; c0 < nd; c0 += 32) {
        const int i = c0 + lane;
        int beg = 0, deg = 0;
        if (i < nd) {
          const int v = src[i];
          beg = __ldg(a.adj_ptr + v);
          deg = __ldg(a.adj_ptr + v + 1) - beg;
        }
        int incl = deg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
          if (lane >= o) incl += y;
        }
        sh.beg[lane] = beg;
        sh.end[lane] = incl;
        __syncwarp();
        const int total = sh.end[31];
        for (int j = lane; j < total; j += 32) {
          int lo = 0, hi = 31;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sh.end[mid] > j) hi = mid;
            else lo = mid + 1;
          }
          const int first = lo ? sh.end[lo - 1] : 0;
          const int p = __ldg(a.adj + sh.beg[lo] + (j - first));
          if (a.ent && a.ent[p]) continue;
          int c = set_insert<WCAND_LOG>(sh.cand_set, p);
          if (c < 0) c = atomicMax(pstamp + p, epoch) < epoch ? 1 : 0;
          if (c > 0) cand[atomicAdd(&sh.ncand, 1)] = p;
        }
        __syncwarp();
      }
      WarpNodeStore rs{ws, a.base, sh.bits, vmark, tmark, cur ? dl0 : dl1, touched, &sh.nd[cur ^ 1], &sh.nt,
                       sh.chg_set, epoch, tag};
      const int nc = sh.ncand;
      int f2 = 0, ch = 0;
      for (int i = lane; i < nc; i += 32) {
        const int4 b = __ldg(a.bc + cand[i]);
        const Itv ia = rs.load(b.y), ib = rs.load(b.z), ic = rs.load(b.w);
        ch += deduce_loaded(b.x, b.y, b.z, b.w, ia, ib, ic, rs, f2);
        ++execs;
      }
      narrowed += ch;
      if (certifying) {
        cert_narrowed += ch;
        if (lane == 0) cert_execs += nc;
      }
      failed = __any_sync(0xFFFFFFFFu, f2) ? 1 : 0;
      __syncwarp();
      cur ^= 1;
      if (certifying) certified = sh.nd[cur] == 0;
    }
    if (failed) status = PIR_FAILED;
    if (lane == 0) {
      a.out[node].status = status;
      a.out[node].rounds = (int)round;
    }
    if (a.out_store) {
      int2 *dst = a.out_store + (size_t)node * nv;
      for (size_t v = lane; v < nv; v += 32) {
        const Itv t = st.load((int)v);
        dst[v] = make_int2(t.l, t.u);
      }
    }
    for (int k = lane; k < a.nwatch; k += 32) {
      const Itv t = st.load(a.watch[k]);
      a.out_watch[(size_t)node * a.nwatch + k] = make_int2(t.l, t.u);
    }
    __syncwarp();
    // the overlay back to the whole range where this node narrowed, the bitmap cleared
    const int nt = sh.nt;
    for (int i = lane; i < nt; i += 32) ws[touched[i]] = make_int2(INT_MIN, INT_MAX);
    for (int i = lane; i < (1 << WBITS_LOG) / 32; i += 32) sh.bits[i] = 0u;
    __syncwarp();
  }
  if (lane == 0) a.epochs[slot] = epoch;
  execs = warp_sum64(execs);
  narrowed = warp_sum64(narrowed);
  cert_narrowed = warp_sum64(cert_narrowed);
  if (lane == 0) {
    if (execs) atomicAdd(a.execs, execs);
    if (narrowed) atomicAdd(a.narrowed, narrowed);
    if (cert_narrowed) atomicAdd(a.cert + 1, cert_narrowed);
    if (cert_execs) atomicAdd(a.cert, cert_execs);
  }
}

// Entailment of every propagator at the base store (engine-order AoS bytecode).
__global__ void k_entailed(const int4 *bc, long long n, const int2 *store, unsigned char *ent) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int4 b = __ldg(bc + p);
    const int2 x = store[b.y], y = store[b.z], z = store[b.w];
    ent[p] = b.x != OP_NOP && ask(b.x, mk(x.x, x.y), mk(y.x, y.y), mk(z.x, z.y)) ? 1 : 0;
  }
}

// Node-major output: out[node][v] = group store[v][lane].
__global__ void k_nodes_unpack(const int2 *nstore, int nvars, int nnodes, int *out_lb, int *out_ub) {
  const long long total = (long long)nnodes * nvars;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int node = (int)(i / nvars), v = (int)(i % nvars);
    const int2 t = nstore[((size_t)(node >> 5) * nvars + v) * 32 + (node & 31)];
    out_lb[i] = t.x;
    out_ub[i] = t.y;
  }
}

__global__ void k_fill_top(int2 *a, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = make_int2(INT_MIN, INT_MAX);
}

__global__ void k_pack_int2(const int *lb, const int *ub, long long n, int2 *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_int2(lb[i], ub[i]);
}

__global__ void k_unpack_int2(const int2 *in, long long n, int *lb, int *ub) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int2 t = in[i];
    lb[i] = t.x;
    ub[i] = t.y;
  }
}

BatchState *batch(pirgpu_ctx *ctx) {
  if (!ctx->batch) ctx->batch = new BatchState();
  return ctx->batch;
}

// AoS bytecode and the variable -> propagator adjacency of the context's
// bytecode (engine order), rebuilt when the bytecode changes.
int ensure_events_graph(pirgpu_ctx *ctx, BatchState *b) {
  if (b->ev_version == ctx->bytecode_version && b->ev_graph_nvars == ctx->nvars && b->d_bc4) return PIR_OK;
  const long long n = ctx->n;
  const int nv = ctx->nvars;
  if (!adjacency_fits(3 * n))
    return set_err(ctx, PIR_EINVAL, "event schedule: %lld propagators need more than 2^31 - 1 adjacency entries", n);
  std::vector<int> ptr((size_t)nv + 1, 0), adj((size_t)n * 3);
  void *ptrs[] = {b->d_bc4, b->d_adj_ptr, b->d_adj};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  b->d_bc4 = nullptr;
  b->d_adj_ptr = b->d_adj = nullptr;
  if (cudaMalloc(&b->d_bc4, std::max<size_t>(1, (size_t)n) * sizeof(int4)) != cudaSuccess ||
      cudaMalloc(&b->d_adj_ptr, ((size_t)nv + 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&b->d_adj, std::max<size_t>(1, (size_t)n * 3) * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "event graph");
  }
  if (n >= DEVICE_INSTALL_MIN) {
    // on the device (pir_install.cu); the host copy of the adjacency for the segment builder
    int r;
    if ((r = device_events_graph(ctx, b->d_bc4, b->d_adj_ptr, b->d_adj))) return r;
    PIR_CK(cudaMemcpyAsync(ptr.data(), b->d_adj_ptr, ptr.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PIR_CK(cudaMemcpyAsync(adj.data(), b->d_adj, adj.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PIR_CK(cudaStreamSynchronize(ctx->stream));
  } else {
    // on the host's threads
    std::vector<int4> bc4((size_t)n);
    const int T = adjacency_threads(n, 0, nv);
    run_threads(T, [&](int t) {
      for (long long p = n * t / T; p < n * (t + 1) / T; ++p)
        bc4[(size_t)p] =
            make_int4(ctx->h_op[(size_t)p], ctx->h_x[(size_t)p], ctx->h_y[(size_t)p], ctx->h_z[(size_t)p]);
    });
    if (!build_adjacency(n, nv, ctx->h_x.data(), ctx->h_y.data(), ctx->h_z.data(), ptr.data(), adj.data(), T))
      return set_err(ctx, PIR_EINVAL, "event schedule: adjacency does not fit int32 offsets");
    PIR_CK(cudaMemcpyAsync(b->d_bc4, bc4.data(), (size_t)n * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(b->d_adj_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(b->d_adj, adj.data(), adj.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaStreamSynchronize(ctx->stream));
  }
  b->h_adj_ptr.swap(ptr);
  b->h_adj.swap(adj);
  b->ev_version = ctx->bytecode_version;
  b->ev_graph_nvars = nv;
  return PIR_OK;
}

// Path segments and the variable -> unit adjacency of the context's
// bytecode, rebuilt with the adjacency.
static int ensure_segments(pirgpu_ctx *ctx, BatchState *b) {
  int r;
  if ((r = ensure_events_graph(ctx, b))) return r;
  if (b->seg_version == ctx->bytecode_version && b->seg_nvars == ctx->nvars) return PIR_OK;
  const long long n = ctx->n;
  const int nv = ctx->nvars;
  Segments S;
  if (!build_segments(n, nv, ctx->h_op.data(), ctx->h_x.data(), ctx->h_y.data(), ctx->h_z.data(),
                      b->h_adj_ptr.data(), b->h_adj.data(), adjacency_threads(n, 0, nv), S))
    return set_err(ctx, PIR_EINVAL, "event schedule: unit adjacency does not fit int32 offsets");
  void *old[] = {b->d_uptr, b->d_uadj, b->d_seg_pptr, b->d_seg_code, b->d_seg_vptr, b->d_seg_var, b->d_in_seg,
                 b->d_seg_umask};
  for (void *q : old)
    if (q) cudaFree(q);
  b->d_uptr = b->d_uadj = b->d_seg_pptr = b->d_seg_code = b->d_seg_vptr = nullptr;
  b->d_seg_var = b->d_in_seg = nullptr;
  b->d_seg_umask = nullptr;
  b->nseg = 0;
  if (S.nseg > 0) {
    auto up = [&](void **dst, const void *src, size_t bytes) -> int {
      if (cudaMalloc(dst, std::max<size_t>(bytes, 4)) != cudaSuccess) {
        cudaGetLastError();
        *dst = nullptr;
        return set_err(ctx, PIR_ENOMEM, "event segments");
      }
      if (bytes) PIR_CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
      return PIR_OK;
    };
    if ((r = up((void **)&b->d_uptr, S.uptr.data(), S.uptr.size() * 4)) ||
        (r = up((void **)&b->d_uadj, S.uadj.data(), S.uadj.size() * 4)) ||
        (r = up((void **)&b->d_seg_pptr, S.pptr.data(), S.pptr.size() * 4)) ||
        (r = up((void **)&b->d_seg_code, S.code.data(), S.code.size() * 4)) ||
        (r = up((void **)&b->d_seg_vptr, S.vptr.data(), S.vptr.size() * 4)) ||
        (r = up((void **)&b->d_seg_var, S.var.data(), S.var.size() * 4)) ||
        (r = up((void **)&b->d_in_seg, S.in_seg.data(), S.in_seg.size() * 4)) ||
        (r = up((void **)&b->d_seg_umask, S.umask.data(), S.umask.size() * 8)))
      return r;
    PIR_CK(cudaStreamSynchronize(ctx->stream));
    b->nseg = S.nseg;
    b->seg_nvar = (long long)S.var.size();
  }
  b->seg_version = ctx->bytecode_version;
  b->seg_nvars = nv;
  return PIR_OK;
}

int events_graph(pirgpu_ctx *ctx, EventsGraph *g, bool segments) {
  BatchState *b = batch(ctx);
  const int r = segments ? ensure_segments(ctx, b) : ensure_events_graph(ctx, b);
  if (r) return r;
  *g = EventsGraph();
  g->bc = b->d_bc4;
  g->adj_ptr = b->d_adj_ptr;
  g->adj = b->d_adj;
  g->uptr = b->d_adj_ptr;
  g->uadj = b->d_adj;
  if (segments && b->nseg > 0) {
    g->nseg = b->nseg;
    g->seg_nvar = b->seg_nvar;
    g->uptr = b->d_uptr;
    g->uadj = b->d_uadj;
    g->seg_pptr = b->d_seg_pptr;
    g->seg_code = b->d_seg_code;
    g->seg_vptr = b->d_seg_vptr;
    g->seg_var = b->d_seg_var;
    g->in_seg = b->d_seg_umask ? b->d_in_seg : nullptr;
    g->seg_umask = b->d_seg_umask;
  }
  return PIR_OK;
}

// A launch of the event node kernel for nnodes nodes, all but the nodes' own
// arrays: the variant, the grid, the per-CTA scratch and the propagators
// entailed at the base store (recomputed when the store or bytecode changed).
struct NodePlan {
  const void *kfn;
  int grid, block;
  size_t dyn_smem;
  bool need_ent;
  EvArgs a;
};

static int plan_nodes(pirgpu_ctx *ctx, BatchState *b, int32_t nnodes, const pir_opts &opts, NodePlan *plan) {
  int r;
  if ((r = ensure_events_graph(ctx, b))) return r;
  // variants 1..10: (threads per CTA, nodes per CTA -- 1: one node per CTA,
  // else one per warp --, resident CTAs per SM the registers are sized for)
  struct NodeVariant {
    int block, wpb;
    const void *fn;
  };
  static const NodeVariant kNodeVariants[] = {
      {256, 1, (const void *)k_nodes_events<256, 2>}, {256, 1, (const void *)k_nodes_events<256, 3>},
      {256, 1, (const void *)k_nodes_events<256, 4>}, {256, 1, (const void *)k_nodes_events<256, 6>},
      {256, 1, (const void *)k_nodes_events<256, 8>}, {128, 1, (const void *)k_nodes_events<128, 8>},
      {128, 1, (const void *)k_nodes_events<128, 10>}, {256, 8, (const void *)k_nodes_warp<8, 2>},
      {256, 8, (const void *)k_nodes_warp<8, 3>},      {128, 4, (const void *)k_nodes_warp<4, 6>}};
  static_assert(sizeof(kNodeVariants) / sizeof(kNodeVariants[0]) == PIR_NODE_VARIANTS, "node variant count");
  const int nvar = opts.variant >= 1 && opts.variant <= PIR_NODE_VARIANTS ? opts.variant
                   : (b->node_variant > 0 ? b->node_variant : 6);
  const int block = kNodeVariants[nvar - 1].block, wpb = kNodeVariants[nvar - 1].wpb;
  const void *kfn = kNodeVariants[nvar - 1].fn;
  // CTA per node: the bitmap of narrowed variables, in shared memory while it
  // takes at most 32 KB; warp per node: its shared state
  const int words = (ctx->nvars + 31) / 32;
  const int bitmap_words = wpb == 1 && words * 4 <= 32 * 1024 ? words : 0;
  const size_t dyn_smem = wpb > 1 ? (size_t)wpb * sizeof(WarpNodeShared)
                          : bitmap_words ? (size_t)bitmap_words * 4 : ((size_t)1 << TOUCH_LOG) * sizeof(int);
  if (dyn_smem > 48 * 1024)
    PIR_CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem));
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, block, dyn_smem));
  occ = std::max(occ, 1);
  const int grid = std::max(1, std::min((nnodes + wpb - 1) / wpb,
                                        ctx->num_sms * (opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ)));
  const size_t nv = (size_t)ctx->nvars, n = (size_t)std::max<long long>(ctx->n, 1);
  // per-node-in-flight scratch slots (a CTA's, or a warp's): ws | vmark |
  // tmark | lists(3) | pstamp | cand | epochs
  const size_t per_cta = nv * 8 + nv * 4 * 2 + nv * 4 * 3 + n * 4 * 2;
  const int need_slots = grid * wpb;
  if (b->ev_slots < need_slots || b->ev_nvars != ctx->nvars || b->ev_n != ctx->n) {
    const int slots = std::max(need_slots, ctx->num_sms * occ * wpb);
    const size_t need = per_cta * (size_t)slots + 64 * (size_t)slots + 256;
    if (b->d_ev) cudaFree(b->d_ev);
    b->d_ev = nullptr;
    b->cap_ev = 0;
    b->ev_slots = 0;
    if (cudaMalloc(&b->d_ev, need) != cudaSuccess) {
      cudaGetLastError();
      return set_err(ctx, PIR_ENOMEM, "event scratch (%zu bytes)", need);
    }
    b->cap_ev = need;
    b->ev_slots = slots;
    b->ev_nvars = ctx->nvars;
    b->ev_n = ctx->n;
    PIR_CK(cudaMemsetAsync(b->d_ev, 0, need, ctx->stream));  // stamps and epochs start at 0
    // the overlays start at the whole integer range (the first slots * nvars int2)
    const long long cells = (long long)slots * ctx->nvars;
    k_fill_top<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(reinterpret_cast<int2 *>(b->d_ev), cells);
    PIR_CK(cudaGetLastError());
  }
  const size_t slots = (size_t)b->ev_slots;
  char *base = (char *)b->d_ev;
  EvArgs a;
  a.bc = b->d_bc4;
  a.n = ctx->n;
  a.nvars = ctx->nvars;
  a.adj_ptr = b->d_adj_ptr;
  a.adj = b->d_adj;
  a.base = ctx->d_store;
  a.bitmap_words = bitmap_words;
  a.ws = (int2 *)base;
  base += slots * nv * 8;
  a.vmark = (unsigned *)base;
  base += slots * nv * 4;
  a.tmark = (unsigned *)base;
  base += slots * nv * 4;
  a.lists = (int *)base;
  base += slots * nv * 12;
  a.pstamp = (unsigned *)base;
  base += slots * n * 4;
  a.cand = (int *)base;
  base += slots * n * 4;
  a.epochs = (unsigned *)base;
  // propagators entailed at the base store
  if ((r = ensure(ctx, (void **)&b->d_ent, &b->cap_ent, n))) return r;
  const bool need_ent = b->ent_store_version != ctx->store_version || b->ent_bc_version != ctx->bytecode_version;
  a.ent = b->d_ent;
  plan->kfn = kfn;
  plan->grid = grid;
  plan->block = block;
  plan->dyn_smem = dyn_smem;
  plan->need_ent = need_ent;
  plan->a = a;
  return PIR_OK;
}

int fixpoint_nodes_events(pirgpu_ctx *ctx, BatchState *b, int32_t nnodes, const int32_t *off, const int32_t *var,
                          const int32_t *lb, const int32_t *ub, const pir_opts &opts, int32_t *out_lb,
                          int32_t *out_ub, int32_t *out_status, int32_t *out_rounds, pir_stats *stats,
                          int32_t nwatch = 0, const int32_t *watch = nullptr, int32_t *out_wlb = nullptr,
                          int32_t *out_wub = nullptr) {
  int r;
  NodePlan plan;
  if ((r = plan_nodes(ctx, b, nnodes, opts, &plan))) return r;
  EvArgs a = plan.a;
  const void *kfn = plan.kfn;
  const int grid = plan.grid, block = plan.block;
  const size_t dyn_smem = plan.dyn_smem;
  const bool need_ent = plan.need_ent;
  const size_t nv = (size_t)ctx->nvars;
  // tightenings, counters, outputs
  const int ntight = off[nnodes];
  if ((r = ensure(ctx, (void **)&b->d_tight, &b->cap_tight, ((size_t)nnodes + 1 + 3 * (size_t)ntight + 8) * sizeof(int))))
    return r;
  if ((r = ensure(ctx, (void **)&b->d_nout, &b->cap_nout, (size_t)nnodes * sizeof(NodeOut) + 64))) return r;
  int *d_off = b->d_tight, *d_var = d_off + nnodes + 1, *d_lb = d_var + ntight, *d_ub = d_lb + ntight;
  int *d_next = d_ub + ntight;
  unsigned long long *d_cnt =
      reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(b->d_nout) + (size_t)nnodes * sizeof(NodeOut));
  PIR_CK(cudaMemcpyAsync(d_off, off, (nnodes + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (ntight) {
    PIR_CK(cudaMemcpyAsync(d_var, var, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(d_lb, lb, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(d_ub, ub, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  }
  PIR_CK(cudaMemsetAsync(d_next, 0, 4 * sizeof(int), ctx->stream));
  PIR_CK(cudaMemsetAsync(d_cnt, 0, 4 * sizeof(unsigned long long), ctx->stream));
  int2 *d_out_store = nullptr;
  if (out_lb) {
    if ((r = ensure(ctx, (void **)&b->d_nstore, &b->cap_nstore, (size_t)nnodes * nv * sizeof(int2)))) return r;
    d_out_store = b->d_nstore;
  }
  a.out_store = d_out_store;
  a.nwatch = nwatch;
  a.watch = nullptr;
  a.out_watch = nullptr;
  if (nwatch > 0) {
    const size_t wbytes = (size_t)nwatch * sizeof(int) + 16 + (size_t)nnodes * nwatch * sizeof(int2);
    if ((r = ensure(ctx, (void **)&b->d_watch, &b->cap_watch, wbytes))) return r;
    int *dw = b->d_watch;
    int2 *dwo = reinterpret_cast<int2 *>(reinterpret_cast<char *>(dw) + (((size_t)nwatch * sizeof(int) + 15) & ~(size_t)15));
    PIR_CK(cudaMemcpyAsync(dw, watch, (size_t)nwatch * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    a.watch = dw;
    a.out_watch = dwo;
  }
  a.off = d_off;
  a.var = d_var;
  a.lb = d_lb;
  a.ub = d_ub;
  a.nnodes = nnodes;
  a.next = d_next;
  a.out = b->d_nout;
  a.execs = d_cnt;
  a.narrowed = d_cnt + 1;
  a.cert = d_cnt + 2;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.certify = opts.certify >= 0;
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (need_ent) {
    k_entailed<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(b->d_bc4, ctx->n, ctx->d_store, b->d_ent);
    PIR_CK(cudaGetLastError());
  }
  {
    void *kargs[] = {&a};
    PIR_CK(cudaLaunchKernel(kfn, dim3(grid), dim3(block), kargs, dyn_smem, ctx->stream));
  }
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  std::vector<NodeOut> hout(nnodes);
  unsigned long long hcnt[4] = {0, 0, 0, 0};
  PIR_CK(cudaMemcpyAsync(hout.data(), b->d_nout, nnodes * sizeof(NodeOut), cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemcpyAsync(hcnt, d_cnt, sizeof(hcnt), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<int2> hw;
  if (nwatch > 0) {
    hw.resize((size_t)nnodes * nwatch);
    PIR_CK(cudaMemcpyAsync(hw.data(), a.out_watch, hw.size() * sizeof(int2), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (out_lb) {
    int per = (int)std::min<long long>(nnodes, (256ll << 20) / std::max<long long>(8ll * ctx->nvars, 1));
    per = std::max(per, 1);
    if ((r = ensure(ctx, (void **)&b->d_nio, &b->cap_nio, (size_t)per * nv * 2 * sizeof(int)))) return r;
    for (int j0 = 0; j0 < nnodes; j0 += per) {
      const int cnt = std::min(per, nnodes - j0);
      const long long items = (long long)cnt * (long long)nv;
      k_unpack_int2<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(b->d_nstore + (size_t)j0 * nv, items, b->d_nio,
                                                              b->d_nio + (size_t)cnt * nv);
      PIR_CK(cudaGetLastError());
      PIR_CK(cudaMemcpyAsync(out_lb + (size_t)j0 * nv, b->d_nio, (size_t)items * sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream));
      PIR_CK(cudaMemcpyAsync(out_ub + (size_t)j0 * nv, b->d_nio + (size_t)cnt * nv, (size_t)items * sizeof(int),
                             cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  b->ent_store_version = ctx->store_version;
  b->ent_bc_version = ctx->bytecode_version;
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  int worst = PIR_OK;
  for (int j = 0; j < nnodes; ++j) {
    out_status[j] = hout[j].status;
    if (out_rounds) out_rounds[j] = hout[j].rounds;
    st.rounds = std::max<int64_t>(st.rounds, hout[j].rounds);
    if (hout[j].status == PIR_TIMEOUT) worst = PIR_TIMEOUT;
  }
  for (size_t k = 0; k < hw.size(); ++k) {
    out_wlb[k] = hw[k].x;
    out_wub[k] = hw[k].y;
  }
  st.executions = (int64_t)hcnt[0];
  st.narrowed = (int64_t)hcnt[1];
  st.certify_executions = (int64_t)hcnt[2];
  st.certify_narrowed = (int64_t)hcnt[3];
  st.status = worst;
  if (stats) *stats = st;
  return PIR_OK;
}

// Pinned host buffer of at least `bytes` (a power of two, so that growing
// batches reallocate, and move the staged graph's buffers, rarely).
static int ensure_pinned(pirgpu_ctx *ctx, void **ptr, size_t *cap, size_t bytes) {
  if (*cap >= bytes && *ptr) return PIR_OK;
  size_t want = 4096;
  while (want < bytes) want <<= 1;
  if (*ptr) cudaFreeHost(*ptr);
  *ptr = nullptr;
  *cap = 0;
  if (cudaHostAlloc(ptr, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return set_err(ctx, PIR_ENOMEM, "cudaHostAlloc(%zu) failed", want);
  }
  *cap = want;
  return PIR_OK;
}

static size_t pow2_at_least(size_t bytes) {
  size_t want = 4096;
  while (want < bytes) want <<= 1;
  return want;
}

// Staged batch layout.  In (int32, host and device alike): watch (nwatch) |
// off (nnodes + 1) | var | lb | ub (ntight each).  Out (device, copied back
// whole): counters (4 x u64: executions, narrowings, and the certifying
// sweeps' executions and narrowings) | work counter (4 x int) | padding to 64
// bytes | NodeOut x nnodes | watched bounds int2 x nnodes x nwatch.
constexpr size_t STAGE_HDR = 64;
static size_t stage_in_bytes(int32_t nnodes, int32_t ntight, int32_t nwatch) {
  return ((size_t)nwatch + (size_t)nnodes + 1 + 3 * (size_t)ntight) * sizeof(int32_t);
}
static size_t stage_out_bytes(int32_t nnodes, int32_t nwatch) {
  return STAGE_HDR + (size_t)nnodes * sizeof(NodeOut) + (size_t)nnodes * (size_t)nwatch * sizeof(int2);
}

int nodes_stage(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, int32_t **in) {
  BatchState *b = batch(ctx);
  int r;
  if ((r = ensure_pinned(ctx, (void **)&b->h_sin, &b->cap_sin, stage_in_bytes(nnodes, ntight, nwatch)))) return r;
  *in = b->h_sin;
  return PIR_OK;
}

static int build_stage_graph(pirgpu_ctx *ctx, BatchState *b, size_t bytes_in, size_t bytes_out,
                             const cudaKernelNodeParams &kp) {
  if (b->sgx) cudaGraphExecDestroy(b->sgx);
  if (b->sg) cudaGraphDestroy(b->sg);
  b->sgx = nullptr;
  b->sg = nullptr;
  b->sg_kfn = nullptr;
  PIR_CK(cudaGraphCreate(&b->sg, 0));
  cudaMemsetParams ms;
  std::memset(&ms, 0, sizeof(ms));
  ms.dst = b->d_sout;
  ms.value = 0;
  ms.elementSize = 4;
  ms.width = STAGE_HDR / 4;  // the counters
  ms.height = 1;
  cudaGraphNode_t clear, e0, e1;
  PIR_CK(cudaGraphAddMemsetNode(&clear, b->sg, nullptr, 0, &ms));
  PIR_CK(cudaGraphAddMemcpyNode1D(&b->sg_in, b->sg, &clear, 1, b->d_sin, b->h_sin, bytes_in, cudaMemcpyHostToDevice));
  PIR_CK(cudaGraphAddEventRecordNode(&e0, b->sg, &b->sg_in, 1, ctx->ev0));
  PIR_CK(cudaGraphAddKernelNode(&b->sg_kernel, b->sg, &e0, 1, &kp));
  PIR_CK(cudaGraphAddEventRecordNode(&e1, b->sg, &b->sg_kernel, 1, ctx->ev1));
  PIR_CK(cudaGraphAddMemcpyNode1D(&b->sg_out, b->sg, &e1, 1, b->h_sout, b->d_sout, bytes_out, cudaMemcpyDeviceToHost));
  PIR_CK(cudaGraphInstantiate(&b->sgx, b->sg, 0));
  b->sg_kfn = kp.func;
  b->sg_bufs[0] = b->h_sin;
  b->sg_bufs[1] = b->h_sout;
  b->sg_bufs[2] = b->d_sin;
  b->sg_bufs[3] = b->d_sout;
  return PIR_OK;
}

int nodes_run_staged(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, const pir_opts &opts,
                     int32_t *out_status, int32_t *out_rounds, const int2 **wout, pir_stats *stats) {
  BatchState *b = batch(ctx);
  int r;
  NodePlan plan;
  if ((r = plan_nodes(ctx, b, nnodes, opts, &plan))) return r;
  const size_t bytes_in = stage_in_bytes(nnodes, ntight, nwatch), bytes_out = stage_out_bytes(nnodes, nwatch);
  if ((r = ensure(ctx, &b->d_sin, &b->cap_dsin, pow2_at_least(bytes_in)))) return r;
  if ((r = ensure(ctx, &b->d_sout, &b->cap_dsout, pow2_at_least(bytes_out)))) return r;
  if ((r = ensure_pinned(ctx, (void **)&b->h_sout, &b->cap_sout, bytes_out))) return r;
  EvArgs a = plan.a;
  int32_t *din = static_cast<int32_t *>(b->d_sin);
  char *dout = static_cast<char *>(b->d_sout);
  a.nwatch = nwatch;
  a.watch = nwatch > 0 ? din : nullptr;
  a.off = din + nwatch;
  a.var = a.off + nnodes + 1;
  a.lb = a.var + ntight;
  a.ub = a.lb + ntight;
  a.nnodes = nnodes;
  a.execs = reinterpret_cast<unsigned long long *>(dout);
  a.narrowed = a.execs + 1;
  a.cert = a.execs + 2;
  a.next = reinterpret_cast<int *>(dout + 32);
  a.out = reinterpret_cast<NodeOut *>(dout + STAGE_HDR);
  a.out_watch = nwatch > 0 ? reinterpret_cast<int2 *>(dout + STAGE_HDR + (size_t)nnodes * sizeof(NodeOut)) : nullptr;
  a.out_store = nullptr;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.certify = opts.certify >= 0;
  void *kargs[] = {&a};
  cudaKernelNodeParams kp{};
  kp.func = const_cast<void *>(plan.kfn);
  kp.gridDim = dim3(plan.grid);
  kp.blockDim = dim3(plan.block);
  kp.sharedMemBytes = (unsigned)plan.dyn_smem;
  kp.kernelParams = kargs;
  if (plan.need_ent) {
    k_entailed<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(b->d_bc4, ctx->n, ctx->d_store, b->d_ent);
    PIR_CK(cudaGetLastError());
  }
  const bool moved = b->sg_bufs[0] != b->h_sin || b->sg_bufs[1] != b->h_sout || b->sg_bufs[2] != b->d_sin ||
                     b->sg_bufs[3] != b->d_sout;
  if (!b->sgx || moved || b->sg_kfn != plan.kfn) {
    if ((r = build_stage_graph(ctx, b, bytes_in, bytes_out, kp))) return r;
  } else {
    PIR_CK(cudaGraphExecMemcpyNodeSetParams1D(b->sgx, b->sg_in, b->d_sin, b->h_sin, bytes_in, cudaMemcpyHostToDevice));
    PIR_CK(cudaGraphExecKernelNodeSetParams(b->sgx, b->sg_kernel, &kp));
    PIR_CK(cudaGraphExecMemcpyNodeSetParams1D(b->sgx, b->sg_out, b->h_sout, b->d_sout, bytes_out,
                                              cudaMemcpyDeviceToHost));
  }
  PIR_CK(cudaGraphLaunch(b->sgx, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  b->ent_store_version = ctx->store_version;
  b->ent_bc_version = ctx->bytecode_version;
  const unsigned long long *cnt = reinterpret_cast<const unsigned long long *>(b->h_sout);
  const NodeOut *no = reinterpret_cast<const NodeOut *>(b->h_sout + STAGE_HDR);
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  int worst = PIR_OK;
  for (int j = 0; j < nnodes; ++j) {
    out_status[j] = no[j].status;
    if (out_rounds) out_rounds[j] = no[j].rounds;
    st.rounds = std::max<int64_t>(st.rounds, no[j].rounds);
    if (no[j].status == PIR_TIMEOUT) worst = PIR_TIMEOUT;
  }
  st.executions = (int64_t)cnt[0];
  st.narrowed = (int64_t)cnt[1];
  st.certify_executions = (int64_t)cnt[2];
  st.certify_narrowed = (int64_t)cnt[3];
  st.status = worst;
  if (stats) *stats = st;
  *wout = reinterpret_cast<const int2 *>(b->h_sout + STAGE_HDR + (size_t)nnodes * sizeof(NodeOut));
  return PIR_OK;
}

}  // namespace pirgpu

using namespace pirgpu;

// fn(j) for j = 0 .. count-1 on the host's threads (dynamic assignment).
template <class F>
static void host_parallel(int count, F fn) {
  const int nt = (int)std::max(1u, std::min({16u, std::thread::hardware_concurrency(), (unsigned)std::max(count, 1)}));
  if (nt <= 1 || count < 2) {
    for (int j = 0; j < count; ++j) fn(j);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (int j; (j = next.fetch_add(1)) < count;) fn(j);
    });
  for (auto &th : pool) th.join();
}

extern "C" int pir_fixpoint_instances(pirgpu_ctx *ctx, int32_t ninst, const int64_t *prop_off, const int64_t *var_off,
                                      const int32_t *op, const int32_t *x, const int32_t *y, const int32_t *z,
                                      int32_t *lb, int32_t *ub, const pir_opts *opts_in, int32_t *out_status,
                                      int32_t *out_rounds, float *out_device_ms, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  if (ninst < 0 || (ninst > 0 && (!prop_off || !var_off || !lb || !ub || !out_status)))
    return set_err(ctx, PIR_EINVAL, "bad arguments");
  if (ninst == 0) return PIR_OK;
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  if (prop_off[0] != 0 || var_off[0] != 0) return set_err(ctx, PIR_EINVAL, "offsets must start at 0");
  if (opts.sched != PIR_SCHED_AC1 && opts.sched != PIR_SCHED_EVENTS)
    return set_err(ctx, PIR_EINVAL, "instances run AC-1 or event-filtered rounds (sched %d)", opts.sched);
  const int marks = opts.sched == PIR_SCHED_EVENTS;
  for (int j = 0; j < ninst; ++j) {
    if (prop_off[j + 1] < prop_off[j] || var_off[j + 1] < var_off[j])
      return set_err(ctx, PIR_EINVAL, "offsets of instance %d decrease", j);
    if (var_off[j + 1] - var_off[j] > INT32_MAX / 64) return set_err(ctx, PIR_EINVAL, "instance %d too large", j);
  }
  const long long nprops = prop_off[ninst], nvars = var_off[ninst];
  if (nprops > 0 && (!op || !x || !y || !z)) return set_err(ctx, PIR_EINVAL, "null bytecode");
  // validation on the host's threads: the first bad instance is reported
  std::atomic<int> bad_inst{INT32_MAX}, bad_kind{0};
  host_parallel(ninst, [&](int j) {
    const long long nv = var_off[j + 1] - var_off[j];
    for (long long i = prop_off[j]; i < prop_off[j + 1]; ++i) {
      const int kind = (op[i] < 0 || op[i] >= OP_COUNT) ? 1
                       : (x[i] < 0 || x[i] >= nv || y[i] < 0 || y[i] >= nv || z[i] < 0 || z[i] >= nv) ? 2
                                                                                                         : 0;
      if (kind) {
        int cur = bad_inst.load();
        while (j < cur && !bad_inst.compare_exchange_weak(cur, j)) {
        }
        if (bad_inst.load() == j) bad_kind.store(kind);
        return;
      }
    }
  });
  if (bad_inst.load() != INT32_MAX)
    return set_err(ctx, PIR_EINVAL, bad_kind.load() == 1 ? "instance %d: bad opcode" : "instance %d: var index out of range",
                   bad_inst.load());
  PIR_CK(cudaSetDevice(ctx->device));
  BatchState *b = batch(ctx);
  // Padded chunk layout: instance j owns chunks coff[j] .. coff[j+1]-1.
  std::vector<long long> off(2 * (size_t)(ninst + 1));
  long long *coff = off.data(), *voff = off.data() + ninst + 1;
  coff[0] = 0;
  for (int j = 0; j < ninst; ++j) {
    coff[j + 1] = coff[j] + (prop_off[j + 1] - prop_off[j] + 3) / 4;
    voff[j] = var_off[j];
  }
  voff[ninst] = var_off[ninst];
  const long long nchunks = coff[ninst];
  // pinned staging (every slot below is written: no clearing)
  const size_t stage_ints = (size_t)std::max<long long>(nchunks, 1) * 16;
  if (b->cap_stage < stage_ints) {
    if (b->h_stage) cudaFreeHost(b->h_stage);
    b->h_stage = nullptr;
    b->cap_stage = 0;
    if (cudaMallocHost(&b->h_stage, stage_ints * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return set_err(ctx, PIR_ENOMEM, "pinned staging (%zu bytes)", stage_ints * sizeof(int));
    }
    b->cap_stage = stage_ints;
  }
  int *hop = b->h_stage, *hx = hop + 4 * nchunks, *hy = hx + 4 * nchunks, *hz = hy + 4 * nchunks;
  // Install order: each instance's propagators grouped by opcode with a
  // stable counting sort (the order the reference's GPU path sorts by,
  // pir.hpp:339-341), so that warps run one opcode at a time; instances on
  // the host's threads (disjoint output ranges).
  host_parallel(ninst, [&](int j) {
    const long long p0 = prop_off[j], p1 = prop_off[j + 1], d0 = coff[j] * 4, d1 = coff[j + 1] * 4;
    long long start[OP_COUNT + 1] = {0};
    for (long long i = p0; i < p1; ++i) ++start[op[i] + 1];
    for (int o = 0; o < OP_COUNT; ++o) start[o + 1] += start[o];
    for (long long i = p0; i < p1; ++i) {
      const long long d = d0 + start[op[i]]++;
      hop[d] = op[i];
      hx[d] = x[i];
      hy[d] = y[i];
      hz[d] = z[i];
    }
    for (long long d = d0 + (p1 - p0); d < d1; ++d) {
      hop[d] = OP_NOP;
      hx[d] = hy[d] = hz[d] = 0;
    }
  });
  std::vector<int> order(ninst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
    return prop_off[p + 1] - prop_off[p] > prop_off[q + 1] - prop_off[q];
  });
  // Instances whose store does not fit one CTA's shared memory (at two CTAs
  // per SM) but fits a cluster's go to the cluster kernel, the rest to the
  // one-CTA-per-instance kernel; `order` lists the cluster ones first.
  const int small_cap = (std::min(ctx->smem_optin, (int)((228 * 1024) / 2) - 2048) / 16) * 16;
  void (*kinst)(InstArgs) = marks ? k_instances<true> : k_instances<false>;
  void (*kclu)(CluArgs) = marks ? k_instances_cluster<true> : k_instances_cluster<false>;
  // the cluster kernel's dynamic shared memory: what its static arrays leave
  cudaFuncAttributes clu_attr{};
  PIR_CK(cudaFuncGetAttributes(&clu_attr, (const void *)kclu));
  const int clu_cap = ((ctx->smem_optin - (int)clu_attr.sharedSizeBytes) / 16) * 16 - 1024;
  int nbig = 0;
  if (opts.mode != PIR_MODE_SMEM) {
    std::vector<int> big, rest;
    for (int j : order) {
      const long long nv = var_off[j + 1] - var_off[j];
      const long long slot_bytes = ((nv + CLU - 1) / CLU) * 8;
      const long long mb = marks ? mark_bytes((int)nv) : 0;  // the round bitmaps beside the store
      if (nv * 8 + mb > small_cap && slot_bytes <= clu_cap) big.push_back(j);
      else rest.push_back(j);
    }
    nbig = (int)big.size();
    order = big;
    order.insert(order.end(), rest.begin(), rest.end());
  }
  int r;
  if ((r = ensure(ctx, (void **)&b->d_bc, &b->cap_bc, (size_t)std::max<long long>(nchunks, 1) * 64))) return r;
  if ((r = ensure(ctx, (void **)&b->d_off, &b->cap_off, off.size() * sizeof(long long)))) return r;
  if ((r = ensure(ctx, (void **)&b->d_store, &b->cap_store, (size_t)std::max<long long>(nvars, 1) * 8))) return r;
  const size_t aux_ints = (size_t)ninst + 4 + 2 * (size_t)nvars;
  if ((r = ensure(ctx, (void **)&b->d_aux, &b->cap_aux, aux_ints * sizeof(int)))) return r;
  if ((r = ensure(ctx, (void **)&b->d_iout, &b->cap_iout, (size_t)ninst * sizeof(InstOut)))) return r;
  int *d_order = b->d_aux, *d_next = d_order + ninst, *d_lb = d_next + 4, *d_ub = d_lb + nvars;
  PIR_CK(cudaMemcpyAsync(b->d_bc, b->h_stage, (size_t)nchunks * 64, cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(b->d_off, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(d_order, order.data(), ninst * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemsetAsync(d_next, 0, 4 * sizeof(int), ctx->stream));
  PIR_CK(cudaMemsetAsync(b->d_iout, 0, (size_t)ninst * sizeof(InstOut), ctx->stream));
  if (nvars) {
    PIR_CK(cudaMemcpyAsync(d_lb, lb, nvars * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(d_ub, ub, nvars * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    k_pack_int2<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(d_lb, d_ub, nvars, b->d_store);
    PIR_CK(cudaGetLastError());
  }
  const int block = opts.block > 0 ? std::min(opts.block, 512) : 512;
  // CTAs per SM: as asked (default 2), lowered until registers and shared
  // memory let that many stay resident; each gets an equal share of the SM's
  // shared memory.
  int per_sm = opts.ctas_per_sm > 0 ? opts.ctas_per_sm : 2;
  int smem = 0;
  for (;;) {
    smem = std::min(ctx->smem_optin, (int)((228 * 1024) / per_sm) - 2048);
    smem = (smem / 16) * 16;
    PIR_CK(cudaFuncSetAttribute(kinst, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int occ = 0;
    PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kinst, block, smem));
    if (occ >= per_sm || per_sm == 1) break;
    per_sm = std::max(1, occ);
  }
  InstArgs a;
  a.op = b->d_bc;
  a.x = b->d_bc + nchunks;
  a.y = b->d_bc + 2 * nchunks;
  a.z = b->d_bc + 3 * nchunks;
  a.coff = b->d_off;
  a.voff = b->d_off + ninst + 1;
  a.store = b->d_store;
  a.order = d_order;
  a.ninst = ninst;
  a.next = d_next;
  a.out = b->d_iout;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.smem_cap = smem;
  const int grid = std::max(1, std::min(ninst, ctx->num_sms * per_sm));
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (nbig > 0) {
    // phase 1: the large instances on clusters of CLU CTAs (whole GPU)
    CluArgs ca;
    ca.op = a.op;
    ca.x = a.x;
    ca.y = a.y;
    ca.z = a.z;
    ca.coff = a.coff;
    ca.voff = a.voff;
    ca.store = a.store;
    ca.order = d_order;
    ca.ninst = nbig;
    ca.next = d_next + 1;
    ca.out = b->d_iout;
    ca.max_rounds = a.max_rounds;
    ca.smem_cap = clu_cap;
    PIR_CK(cudaFuncSetAttribute(kclu, cudaFuncAttributeMaxDynamicSharedMemorySize, clu_cap));
    cudaLaunchConfig_t cfg{};
    const int nclusters = std::max(1, std::min(nbig, ctx->num_sms / CLU));
    cfg.gridDim = dim3(nclusters * CLU);
    cfg.blockDim = dim3(CLU_BLOCK);
    cfg.dynamicSmemBytes = clu_cap;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CLU;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PIR_CK(cudaLaunchKernelEx(&cfg, kclu, ca));
  }
  if (nbig < ninst) {
    // phase 2: the rest, one CTA per instance
    a.order = d_order + nbig;
    a.ninst = ninst - nbig;
    const int grid2 = std::max(1, std::min(ninst - nbig, ctx->num_sms * per_sm));
    kinst<<<grid2, block, smem, ctx->stream>>>(a);
  }
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if (nvars) {
    k_unpack_int2<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(b->d_store, nvars, d_lb, d_ub);
    PIR_CK(cudaMemcpyAsync(lb, d_lb, nvars * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PIR_CK(cudaMemcpyAsync(ub, d_ub, nvars * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  }
  std::vector<InstOut> hout(ninst);
  PIR_CK(cudaMemcpyAsync(hout.data(), b->d_iout, ninst * sizeof(InstOut), cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  int worst = PIR_OK;
  for (int j = 0; j < ninst; ++j) {
    out_status[j] = hout[j].status;
    if (out_rounds) out_rounds[j] = hout[j].rounds;
    if (out_device_ms) out_device_ms[j] = (float)(hout[j].ns * 1e-6);
    st.rounds = std::max<int64_t>(st.rounds, hout[j].rounds);
    st.executions += marks ? (int64_t)hout[j].execs : (int64_t)hout[j].rounds * (prop_off[j + 1] - prop_off[j]);
    st.narrowed += (int64_t)hout[j].narrowed;
    if (hout[j].status == PIR_TIMEOUT) worst = PIR_TIMEOUT;
  }
  st.status = worst;
  if (stats) *stats = st;
  return PIR_OK;
}

extern "C" int pir_fixpoint_nodes(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                                  const int32_t *lb, const int32_t *ub, const pir_opts *opts_in, int32_t *out_lb,
                                  int32_t *out_ub, int32_t *out_status, int32_t *out_rounds, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  if (nnodes < 0 || (nnodes > 0 && (!off || !out_status))) return set_err(ctx, PIR_EINVAL, "bad arguments");
  if ((out_lb == nullptr) != (out_ub == nullptr)) return set_err(ctx, PIR_EINVAL, "out_lb and out_ub go together");
  if (nnodes == 0) return PIR_OK;
  if (off[0] != 0) return set_err(ctx, PIR_EINVAL, "off[0] must be 0");
  for (int j = 0; j < nnodes; ++j)
    if (off[j + 1] < off[j]) return set_err(ctx, PIR_EINVAL, "node %d: offsets decrease", j);
  const int ntight = off[nnodes];
  if (ntight > 0 && (!var || !lb || !ub)) return set_err(ctx, PIR_EINVAL, "null tightenings");
  for (int k = 0; k < ntight; ++k)
    if (var[k] < 0 || var[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "tightening %d: var out of range", k);
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  PIR_CK(cudaSetDevice(ctx->device));
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  if (ctx->failed || ctx->n == 0) {
    // every node inherits the empty store, or there is nothing to propagate
    std::vector<int32_t> blb(ctx->nvars), bub(ctx->nvars);
    int r = pir_read_store(ctx, blb.data(), bub.data());
    if (r) return r;
    for (int j = 0; j < nnodes; ++j) {
      bool f = ctx->failed;
      std::vector<int32_t> nl(blb), nu(bub);
      for (int k = off[j]; k < off[j + 1]; ++k) {
        nl[var[k]] = std::max(nl[var[k]], lb[k]);
        nu[var[k]] = std::min(nu[var[k]], ub[k]);
        f |= nl[var[k]] > nu[var[k]] || nl[var[k]] == INF || nu[var[k]] == MINF;
      }
      out_status[j] = f ? PIR_FAILED : PIR_OK;
      if (out_rounds) out_rounds[j] = 0;
      if (out_lb) {
        std::copy(nl.begin(), nl.end(), out_lb + (size_t)j * ctx->nvars);
        std::copy(nu.begin(), nu.end(), out_ub + (size_t)j * ctx->nvars);
      }
    }
    if (stats) *stats = st;
    return PIR_OK;
  }
  BatchState *b = batch(ctx);
  if (opts.sched == PIR_SCHED_EVENTS && ctx->at_fixpoint)
    return fixpoint_nodes_events(ctx, b, nnodes, off, var, lb, ub, opts, out_lb, out_ub, out_status, out_rounds,
                                 stats);
  const int ngroups = (nnodes + 31) / 32;
  const size_t group_bytes = (size_t)ctx->nvars * 32 * sizeof(int2);
  int r;
  if ((r = ensure(ctx, (void **)&b->d_nstore, &b->cap_nstore, group_bytes * ngroups))) return r;
  if ((r = ensure(ctx, (void **)&b->d_tight, &b->cap_tight, ((size_t)nnodes + 1 + 3 * (size_t)ntight + 8) * sizeof(int))))
    return r;
  if ((r = ensure(ctx, (void **)&b->d_nout, &b->cap_nout, (size_t)nnodes * sizeof(NodeOut) + 64))) return r;
  int *d_off = b->d_tight, *d_var = d_off + nnodes + 1, *d_lb = d_var + ntight, *d_ub = d_lb + ntight;
  int *d_next = d_ub + ntight;
  static_assert(sizeof(NodeOut) == 8, "NodeOut packs to 8 bytes");
  unsigned long long *d_nar =
      reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(b->d_nout) + (size_t)nnodes * sizeof(NodeOut));
  PIR_CK(cudaMemcpyAsync(d_off, off, (nnodes + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (ntight) {
    PIR_CK(cudaMemcpyAsync(d_var, var, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(d_lb, lb, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    PIR_CK(cudaMemcpyAsync(d_ub, ub, ntight * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  }
  PIR_CK(cudaMemsetAsync(d_next, 0, 4 * sizeof(int), ctx->stream));
  PIR_CK(cudaMemsetAsync(d_nar, 0, sizeof(unsigned long long), ctx->stream));
  NodeArgs a;
  a.bc = bytecode_view(ctx);
  a.nvars = ctx->nvars;
  a.base = ctx->d_store;
  a.nstore = b->d_nstore;
  a.off = d_off;
  a.var = d_var;
  a.lb = d_lb;
  a.ub = d_ub;
  a.nnodes = nnodes;
  a.ngroups = ngroups;
  a.next = d_next;
  a.out = b->d_nout;
  a.narrowed = d_nar;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  const int block = opts.block > 0 ? std::min(opts.block, 512) : 512;
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nodes, block, 0));
  const int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, std::max(occ, 1)) : std::max(occ, 1);
  const int grid = std::max(1, std::min(ngroups, ctx->num_sms * per_sm));
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  k_nodes<<<grid, block, 0, ctx->stream>>>(a);
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  std::vector<NodeOut> hout(nnodes);
  unsigned long long hnar = 0;
  PIR_CK(cudaMemcpyAsync(hout.data(), b->d_nout, nnodes * sizeof(NodeOut), cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemcpyAsync(&hnar, d_nar, sizeof(hnar), cudaMemcpyDeviceToHost, ctx->stream));
  if (out_lb) {
    // stage node-major outputs in chunks of nodes to bound the staging buffer
    int per = (int)std::min<long long>(nnodes, (256ll << 20) / std::max<long long>(8ll * ctx->nvars, 1));
    if (per < nnodes) per = std::max(32, (per / 32) * 32);
    if ((r = ensure(ctx, (void **)&b->d_nio, &b->cap_nio, (size_t)per * ctx->nvars * 2 * sizeof(int)))) return r;
    for (int j0 = 0; j0 < nnodes; j0 += per) {
      const int cnt = std::min(per, nnodes - j0);
      // the unpack kernel indexes groups from node 0; offset the store by whole groups
      const int2 *src = b->d_nstore + (size_t)(j0 / 32) * ctx->nvars * 32;
      if (j0 % 32 != 0) return set_err(ctx, PIR_EINVAL, "internal: unaligned node chunk");
      k_nodes_unpack<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(src, ctx->nvars, cnt, b->d_nio,
                                                                  b->d_nio + (size_t)cnt * ctx->nvars);
      PIR_CK(cudaGetLastError());
      PIR_CK(cudaMemcpyAsync(out_lb + (size_t)j0 * ctx->nvars, b->d_nio, (size_t)cnt * ctx->nvars * sizeof(int),
                             cudaMemcpyDeviceToHost, ctx->stream));
      PIR_CK(cudaMemcpyAsync(out_ub + (size_t)j0 * ctx->nvars, b->d_nio + (size_t)cnt * ctx->nvars,
                             (size_t)cnt * ctx->nvars * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  int worst = PIR_OK;
  for (int j = 0; j < nnodes; ++j) {
    out_status[j] = hout[j].status;
    if (out_rounds) out_rounds[j] = hout[j].rounds;
    st.rounds = std::max<int64_t>(st.rounds, hout[j].rounds);
    st.executions += (int64_t)hout[j].rounds * ctx->n;
    if (hout[j].status == PIR_TIMEOUT) worst = PIR_TIMEOUT;
  }
  st.narrowed = (int64_t)hnar;
  st.status = worst;
  if (stats) *stats = st;
  return PIR_OK;
}

extern "C" int pir_autotune_nodes(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                                  const int32_t *lb, const int32_t *ub, int32_t *out_variant, float *out_ms) {
  if (!ctx) return PIR_EINVAL;
  if (out_variant) *out_variant = 0;
  if (out_ms) *out_ms = 0.f;
  if (nnodes <= 0 || !off) return set_err(ctx, PIR_EINVAL, "no nodes to tune on");
  std::vector<int32_t> status((size_t)nnodes);
  int best = 0;
  float best_ms = 0.f;
  for (int v = 1; v <= PIR_NODE_VARIANTS; ++v) {
    pir_opts o;
    std::memset(&o, 0, sizeof(o));
    o.sched = PIR_SCHED_EVENTS;
    o.variant = v;
    float t = -1.f;
    for (int rep = 0; rep < 2; ++rep) {  // the first run may load the working stores
      pir_stats st;
      const int r = pir_fixpoint_nodes(ctx, nnodes, off, var, lb, ub, &o, nullptr, nullptr, status.data(), nullptr, &st);
      if (r != PIR_OK) return r;
      if (t < 0.f || st.device_ms < t) t = st.device_ms;
    }
    if (best == 0 || t < best_ms) {
      best = v;
      best_ms = t;
    }
  }
  batch(ctx)->node_variant = best;
  if (out_variant) *out_variant = best;
  if (out_ms) *out_ms = best_ms;
  return PIR_OK;
}
