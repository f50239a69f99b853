// Fixpoint kernels of the plain (AC-1) propagation engine for sm_103a.
//
// Round structure (the GPU form of the Gauss-Seidel driver around
// PIR::deduce(int), tests/pir_test.cpp:60-62, and of the per-block copies with
// shared bytecode of pir.hpp:182-195): every round applies every propagator
// once; bound joins are atomic and visible to later reads of the same round;
// the round's "changed" and "failed" bits are OR-reduced (CTA: a warp reduction
// and a shared-memory OR, grid: the barrier word) and the loop stops after a
// round with no change, a round that saw an empty interval, or the round cap.
#pragma once
#include "pir_device.cuh"

namespace pirgpu {

// Device-side control block of one fixpoint run (scratch memory).
struct Control {
  // grid barrier words (grid_sync_rot): arrivals | changed-count << 20 |
  // failed-count << 40, three in rotation, one 128-byte line each
  unsigned long long rot[3][16];
  int status;                 // 0, or the pir_status error a CTA raised
  int failed;                 // sticky failure flag (host loop / single-thread kernels)
  int changed[4];             // host-loop change flags, one per round parity
  long long rounds;           // rounds executed (written by CTA 0)
  unsigned long long narrowed;
  unsigned long long executions;
  // event-driven fixpoint: the CTA that runs small rounds alone publishes a
  // heartbeat (rounds done), the round it stopped at and why (EV_*)
  unsigned long long hb;
  long long ev_round;
  int ev_state;
  int pad_i;
  // certifying sweeps: their executions and the bounds they narrowed
  unsigned long long cert_execs, cert_narrowed;
  // bounds narrowed per round, three in rotation (the persistent kernel's
  // handover to the event schedule)
  unsigned long long joins[3];
  unsigned long long pad[2];
};

constexpr unsigned BIT_CHANGED = 1u << 29;
constexpr unsigned BIT_FAILED = 1u << 30;
constexpr unsigned BIT_ERROR = 1u << 31;

constexpr int ERR_BARRIER_TIMEOUT = 3;  // = PIR_BARRIER_TIMEOUT

static __device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

static __device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

static __device__ __forceinline__ unsigned long long atom_add_release(unsigned long long *p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}
static __device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier of round `round` (0, 1, 2, ...) with an OR-reduction of the
// changed / failed bits, called by thread 0 of every CTA.  Round r uses word
// rot[r % 3]: each CTA adds 1 | changed << 20 | failed << 40 with one release
// RMW and polls the same word with acquire loads until all nblocks arrived, so
// the last arrival releases everyone directly (no generation word, no second
// store).  CTA 0 zeroes the word of round r + 2 as soon as it has passed round
// r: that word was last read at barrier r - 1, which every CTA left before
// arriving at barrier r, and CTA 0's own arrival at barrier r + 1 (a release
// after the zeroing) is seen by every CTA before it can arrive at r + 2.  The
// three words start at zero (the host clears the control block).  Every wait is
// bounded by timeout_ns; on expiry the CTA records PIR_BARRIER_TIMEOUT in
// ctl->status and the result carries BIT_ERROR.  The result's low 20 bits
// are the number of CTAs that reported a change (BIT_CHANGED: at least one).  With a heartbeat word `hb`
// (a CTA working alone while the others wait), the limit runs from the last
// change of *hb, and the waiters poll less often.
static __device__ __noinline__ unsigned grid_sync_rot(Control *ctl, unsigned nblocks, long long round, int changed,
                                                      int failed, long long timeout_ns,
                                                      const unsigned long long *hb = nullptr) {
  unsigned long long *w = &ctl->rot[round % 3][0];
  const unsigned long long add =
      1ull | ((unsigned long long)(changed != 0) << 20) | ((unsigned long long)(failed != 0) << 40);
  unsigned long long v = atom_add_release(w, add) + add;
  if ((unsigned)(v & 0xFFFFFull) != nblocks) {
    unsigned long long t0 = globaltimer(), beat = hb ? *(const volatile unsigned long long *)hb : 0ull;
    for (unsigned it = 0;; ++it) {
      v = ld_acquire64(w);
      if ((unsigned)(v & 0xFFFFFull) == nblocks) break;
      if (it >= 64) __nanosleep(hb ? 1000 : (it < 512 ? 20 : 200));
      if ((it & 7u) == 0u) {
        if (*(volatile int *)&ctl->status) return BIT_ERROR;
        if (hb) {
          const unsigned long long b = *(const volatile unsigned long long *)hb;
          if (b != beat) {
            beat = b;
            t0 = globaltimer();
          }
        }
        if ((long long)(globaltimer() - t0) > timeout_ns) {
          atomicCAS(&ctl->status, 0, ERR_BARRIER_TIMEOUT);
          return BIT_ERROR;
        }
      }
    }
  }
  if (blockIdx.x == 0) ctl->rot[(round + 2) % 3][0] = 0ull;
  // low 20 bits: how many CTAs reported a change in this round
  unsigned r = (unsigned)((v >> 20) & 0xFFFFFull);
  if ((v >> 20) & 0xFFFFFull) r |= BIT_CHANGED;
  if ((v >> 40) & 0xFFFFFull) r |= BIT_FAILED;
  if (*(volatile int *)&ctl->status) r |= BIT_ERROR;
  return r;
}

// The bytecode as a structure of arrays, padded with OP_NOP to a multiple of 4
// so that one thread reads four propagators with 128-bit loads.
struct Bytecode {
  const int4 *op, *x, *y, *z;
  int nchunks;  // ceil(n / 4)
};

// Joins into the HBM store with fire-and-forget reductions (red.global): a
// bound counts as narrowed when it is tighter than the value read.  A
// concurrent tighter join can make that an over-count, which at worst costs
// one more round; a round with no join at all is a true fixpoint because every
// read in it saw the final store.
struct RedStore {
  int2 *s;
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + v);
    return mk(t.x, t.y);
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
    if (n && is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    return n;
  }
};

// Propagators c*PPI .. c*PPI+PPI-1 (PPI = 1, 2 or 4 per thread and step): all
// intervals are gathered first (reads may be stale within a round), then the
// updates are applied in order.  The bytecode arrays are read with 32-, 64- or
// 128-bit loads.
template <int PPI>
struct Vec;
template <>
struct Vec<1> {
  using T = int;
  static __device__ __forceinline__ int get(const T &v, int) { return v; }
};
template <>
struct Vec<2> {
  using T = int2;
  static __device__ __forceinline__ int get(const T &v, int k) { return k == 0 ? v.x : v.y; }
};
template <>
struct Vec<4> {
  using T = int4;
  static __device__ __forceinline__ int get(const T &v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
  }
};

// Bytecode loads: the read-only global path (ld.global.nc) when the bytecode is
// in global memory (GBC), generic loads when it may be staged in shared memory.
template <bool GBC, class V>
__device__ __forceinline__ V bc_load(const V *p) {
  if (GBC) return __ldg(p);
  return *p;
}

template <int PPI, class S, bool GBC = true>
__device__ __forceinline__ int sweep_step(const Bytecode &bc, int c, S &st, int &failed) {
  using V = typename Vec<PPI>::T;
  const V o = bc_load<GBC>(reinterpret_cast<const V *>(bc.op) + c), X = bc_load<GBC>(reinterpret_cast<const V *>(bc.x) + c);
  const V Y = bc_load<GBC>(reinterpret_cast<const V *>(bc.y) + c), Z = bc_load<GBC>(reinterpret_cast<const V *>(bc.z) + c);
  Itv a[PPI], b[PPI], d[PPI];
#pragma unroll
  for (int k = 0; k < PPI; ++k) {
    a[k] = st.load(Vec<PPI>::get(X, k));
    b[k] = st.load(Vec<PPI>::get(Y, k));
    d[k] = st.load(Vec<PPI>::get(Z, k));
  }
  int ch = 0;
#pragma unroll
  for (int k = 0; k < PPI; ++k)
    ch += deduce_loaded(Vec<PPI>::get(o, k), Vec<PPI>::get(X, k), Vec<PPI>::get(Y, k), Vec<PPI>::get(Z, k), a[k],
                        b[k], d[k], st, failed);
  return ch;
}

template <int PPI>
__device__ __forceinline__ void bc_fetch(const Bytecode &bc, int c, typename Vec<PPI>::T (&v)[4]) {
  using V = typename Vec<PPI>::T;
  v[0] = __ldg(reinterpret_cast<const V *>(bc.op) + c);
  v[1] = __ldg(reinterpret_cast<const V *>(bc.x) + c);
  v[2] = __ldg(reinterpret_cast<const V *>(bc.y) + c);
  v[3] = __ldg(reinterpret_cast<const V *>(bc.z) + c);
}

template <int PPI, class S>
__device__ __forceinline__ void gather(const typename Vec<PPI>::T (&v)[4], const S &st, Itv (&a)[PPI], Itv (&b)[PPI],
                                       Itv (&d)[PPI]) {
#pragma unroll
  for (int k = 0; k < PPI; ++k) {
    a[k] = st.load(Vec<PPI>::get(v[1], k));
    b[k] = st.load(Vec<PPI>::get(v[2], k));
    d[k] = st.load(Vec<PPI>::get(v[3], k));
  }
}

// Grid-strided sweep over the steps c, c + stride, ... below nsteps, software
// pipelined: before step i is computed, the intervals of step i+1 and the
// bytecode of step i+2 are already requested, so two L2 round trips overlap
// the arithmetic instead of following it.  Reads may therefore be up to two
// steps older than this thread's own joins; within a round every read may be
// stale anyway, and a round in which nothing changed anywhere read the store of
// its start, so the end-of-round change test stays exact.
template <int PPI, class S>
__device__ __forceinline__ int sweep_pipelined(const Bytecode &bc, int c, const int stride, const int nsteps, S &st,
                                               int &failed) {
  using V = typename Vec<PPI>::T;
  if (c >= nsteps) return 0;
  V cur[4], nxt[4];
  Itv a[PPI], b[PPI], d[PPI];
  bc_fetch<PPI>(bc, c, cur);
  gather<PPI>(cur, st, a, b, d);
  int c1 = c + stride;
  if (c1 < nsteps) bc_fetch<PPI>(bc, c1, nxt);
  int ch = 0;
  for (;;) {
    const bool has1 = c1 < nsteps;
    Itv a1[PPI], b1[PPI], d1[PPI];
    if (has1) gather<PPI>(nxt, st, a1, b1, d1);
    const int c2 = c1 + stride;
    V nn[4];
    if (c2 < nsteps) bc_fetch<PPI>(bc, c2, nn);
#pragma unroll
    for (int k = 0; k < PPI; ++k)
      ch += deduce_loaded(Vec<PPI>::get(cur[0], k), Vec<PPI>::get(cur[1], k), Vec<PPI>::get(cur[2], k),
                          Vec<PPI>::get(cur[3], k), a[k], b[k], d[k], st, failed);
    if (!has1) break;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cur[j] = nxt[j];
      nxt[j] = nn[j];
    }
#pragma unroll
    for (int k = 0; k < PPI; ++k) {
      a[k] = a1[k];
      b[k] = b1[k];
      d[k] = d1[k];
    }
    c1 = c2;
  }
  return ch;
}

// Number of PPI-wide steps covering the (4-padded) bytecode.
template <int PPI>
__device__ __forceinline__ int steps_of(const Bytecode &bc) {
  return bc.nchunks * (4 / PPI);
}

template <class S, bool GBC = true>
__device__ __forceinline__ int sweep_chunk(const Bytecode &bc, int c, S &st, int &failed) {
  return sweep_step<4, S, GBC>(bc, c, st, failed);
}

}  // namespace pirgpu
