// Learned propagator scheduler for sm_103a.
//
// A small MLP (8 -> 32 -> 32 -> 1, BF16 weights, FP32 accumulation) scores
// every propagator at the start of a round from eight features:
//   0-2  opcode class one-hot: {ADD}, {MUL, TDIV, FDIV, CDIV, EDIV}, {MIN, MAX, EQ, LEQ}
//   3-5  log2(width + 1) / 32 of x, y, z
//   6    rounds since any of x, y, z last narrowed, clamped to 64, / 64
//   7    log2(deg x + deg y + deg z) / 16 (static)
// and the round runs only the top-scored propagators (each CTA wakes a fraction
// of the propagators it scored, by a threshold on its own score histogram, so
// a learned round needs one grid barrier).  When a round of woken propagators
// changes nothing, one full AC-1
// sweep certifies the fixpoint; if it changes anything, the learned rounds
// resume.  Propagators are monotone, so any fair schedule that ends with a
// no-change full sweep reaches the same fixpoint as the plain method: the
// result is the AC-1 fixpoint bit for bit.
//
// Training data are change traces of the plain AC-1 fixpoint (features at the
// start of a round, label = the propagator narrowed a bound in that round),
// and the network is trained on the device by the kernels below (forward,
// backward with a per-CTA reduction of the weight gradients, Adam).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "pir_engine.h"

namespace pirgpu {

// Parameter layout (floats): W1[32][8], b1[32], W2[32][32], b2[32], W3[32], b3.
constexpr int NF = 8, NH = 32;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr int HIST_BINS = 2048;
constexpr float HIST_LO = -16.f, HIST_HI = 16.f;
constexpr int TRAIN_CTA = 128;

struct SchedState {
  int nvars = 0;
  long long n = 0;
  long long bc_version = -1;
  float *d_param = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr, *d_loss = nullptr;
  __nv_bfloat16 *d_wbf = nullptr;
  int adam_t = 0;
  bool trained = false;
  int *d_var_last = nullptr;  // round of the last narrowing of each variable
  int *d_deg = nullptr;       // variable degree
  unsigned char *d_pdeg = nullptr;  // per-propagator degree feature (x16 fixed point)
  float *d_score = nullptr;
  unsigned long long *d_counts = nullptr;  // woken executions, samples
  float *d_tx = nullptr, *d_ty = nullptr;  // trace samples
  long long tcap = 0, tcount = 0;
  std::vector<int> dirty;  // variables embedded since the last learned fixpoint
  // learned rounds on a frontier (k_learned_local): the store was a fixpoint
  // of bytecode version base_bc at store version base_version, and `since`
  // lists the variables embedded after it (since_ok: all of them)
  long long base_version = -1, base_bc = -1;
  std::vector<int> since;
  bool since_ok = false;
  unsigned *d_vlast = nullptr, *d_pstamp = nullptr;
  int *d_lf = nullptr, *d_cv = nullptr, *d_since = nullptr, *d_nv = nullptr;
  float *d_lscore = nullptr;
  long long loc_bc_version = -1, loc_n = -1;
  int loc_nvars = -1;
  unsigned loc_base = 65;
};

void destroy_sched_state(pirgpu_ctx *ctx) {
  SchedState *s = ctx->sched;
  if (!s) return;
  void *ptrs[] = {s->d_param, s->d_m,      s->d_v,  s->d_grad, s->d_loss, s->d_wbf,     s->d_var_last,
                  s->d_deg,   s->d_pdeg,   s->d_score, s->d_counts, s->d_tx, s->d_ty, s->d_vlast,
                  s->d_pstamp, s->d_lf,    s->d_cv, s->d_since, s->d_lscore, s->d_nv};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete s;
  ctx->sched = nullptr;
}

// --------------------------------------------------------------- device -----

__device__ __forceinline__ float log2w(Itv a) {
  if (a.l == MINF || a.u == INF) return 1.f;
  const long long w = (long long)a.u - (long long)a.l;
  return w <= 0 ? 0.f : __log2f((float)w + 1.f) * (1.f / 32.f);
}

__device__ __forceinline__ void features(int op, Itv a, Itv b, Itv c, int last, int round, unsigned char pdeg,
                                         float f[NF]) {
  const int cls = op == OP_ADD ? 0 : ((op >= OP_MUL && op <= OP_EDIV) ? 1 : 2);
  f[0] = cls == 0;
  f[1] = cls == 1;
  f[2] = cls == 2;
  f[3] = log2w(a);
  f[4] = log2w(b);
  f[5] = log2w(c);
  f[6] = (float)min(max(round - last, 0), 64) * (1.f / 64.f);
  f[7] = (float)pdeg * (1.f / 256.f);
}

// Weights staged in shared memory as FP32 (converted from BF16).
__device__ __forceinline__ void stage_weights(const __nv_bfloat16 *wbf, float *sw) {
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sw[i] = __bfloat162float(wbf[i]);
}

// ------------------------------------------- tensor-core scoring (mma) -----
// The inference MLP of 32 propagators per warp on the tensor cores
// (mma.sync, BF16 operands, FP32 accumulation): layer 1 is a 16x8x8 product
// per 16 propagators and 8 outputs, layer 2 two 16x8x16 products per 8
// outputs, and the layer-1 accumulators become layer 2's A fragments in
// registers (the m16n8 accumulator layout of two adjacent 8-column tiles is
// the m16k16 A layout).  Fragment layouts (g = lane / 4, c = lane % 4):
// A 16x8: {row g, cols 2c..2c+1}, {row g+8, same}; A 16x16 adds the same for
// cols 2c+8..2c+9; B 8x8 (k x n): {k 2c..2c+1, n g}; B 16x8 adds k 2c+8..;
// accumulators 16x8: {row g, cols 2c..2c+1}, {row g+8, cols 2c..2c+1}.

__device__ __forceinline__ void mma_k8(float (&d)[4], unsigned a0, unsigned a1, unsigned b0) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a0), "r"(a1), "r"(b0));
}
__device__ __forceinline__ void mma_k16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const unsigned *>(&v);
}

// The weights as B fragments, loaded once per thread: layer 1 per 8-output
// tile j, layer 2 per tile j and 16-input step s (two registers).
struct MmaWeights {
  unsigned w1[4];
  unsigned w2[4][2][2];
  __device__ __forceinline__ void load(const __nv_bfloat16 *wbf) {
    const int g = (threadIdx.x & 31) >> 2, c = threadIdx.x & 3;
    const unsigned *w = reinterpret_cast<const unsigned *>(wbf);  // bf16 pairs; every offset below is even
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      w1[j] = __ldg(w + (OFF_W1 + (8 * j + g) * NF + 2 * c) / 2);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        w2[j][k][0] = __ldg(w + (OFF_W2 + (8 * j + g) * NH + 16 * k + 2 * c) / 2);
        w2[j][k][1] = __ldg(w + (OFF_W2 + (8 * j + g) * NH + 16 * k + 2 * c + 8) / 2);
      }
    }
  }
};

// Scores of the warp's 32 propagators (lane i holds the features of row i);
// every lane of the warp must call it.  `tile` is the warp's 32 x 8 BF16
// staging area in shared memory; sw holds the biases and W3 in FP32.
__device__ __forceinline__ float mlp_forward_mma(const float f[NF], const MmaWeights &W, const float *sw,
                                                 __nv_bfloat16 *tile) {
  const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
  unsigned *row = reinterpret_cast<unsigned *>(tile + lane * NF);
#pragma unroll
  for (int i = 0; i < NF / 2; ++i) row[i] = pack_bf16(f[2 * i], f[2 * i + 1]);
  __syncwarp();
  const unsigned *t32 = reinterpret_cast<const unsigned *>(tile);
  float sc[2][2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const unsigned a0 = t32[((16 * t + g) * NF + 2 * c) / 2], a1 = t32[((16 * t + g + 8) * NF + 2 * c) / 2];
    float h[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float b0 = sw[OFF_B1 + 8 * j + 2 * c], b1 = sw[OFF_B1 + 8 * j + 2 * c + 1];
      h[j][0] = b0;
      h[j][1] = b1;
      h[j][2] = b0;
      h[j][3] = b1;
      mma_k8(h[j], a0, a1, W.w1[j]);
    }
    unsigned A2[2][4];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      A2[k][0] = pack_bf16(fmaxf(h[2 * k][0], 0.f), fmaxf(h[2 * k][1], 0.f));
      A2[k][1] = pack_bf16(fmaxf(h[2 * k][2], 0.f), fmaxf(h[2 * k][3], 0.f));
      A2[k][2] = pack_bf16(fmaxf(h[2 * k + 1][0], 0.f), fmaxf(h[2 * k + 1][1], 0.f));
      A2[k][3] = pack_bf16(fmaxf(h[2 * k + 1][2], 0.f), fmaxf(h[2 * k + 1][3], 0.f));
    }
    float lo = 0.f, hi = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float b0 = sw[OFF_B2 + 8 * j + 2 * c], b1 = sw[OFF_B2 + 8 * j + 2 * c + 1];
      float o[4] = {b0, b1, b0, b1};
      mma_k16(o, A2[0], W.w2[j][0][0], W.w2[j][0][1]);
      mma_k16(o, A2[1], W.w2[j][1][0], W.w2[j][1][1]);
      const float v0 = sw[OFF_W3 + 8 * j + 2 * c], v1 = sw[OFF_W3 + 8 * j + 2 * c + 1];
      lo = fmaf(fmaxf(o[0], 0.f), v0, fmaf(fmaxf(o[1], 0.f), v1, lo));
      hi = fmaf(fmaxf(o[2], 0.f), v0, fmaf(fmaxf(o[3], 0.f), v1, hi));
    }
    lo += __shfl_xor_sync(0xFFFFFFFFu, lo, 1);
    lo += __shfl_xor_sync(0xFFFFFFFFu, lo, 2);
    hi += __shfl_xor_sync(0xFFFFFFFFu, hi, 1);
    hi += __shfl_xor_sync(0xFFFFFFFFu, hi, 2);
    sc[t][0] = lo + sw[OFF_B3];
    sc[t][1] = hi + sw[OFF_B3];
  }
  __syncwarp();  // the tile is free again
  // row `lane` = tile lane / 16, row lane % 16 of it, held by the quad of lanes 4 * (lane % 8)
  const int src = (lane & 7) << 2;
  const float v00 = __shfl_sync(0xFFFFFFFFu, sc[0][0], src), v01 = __shfl_sync(0xFFFFFFFFu, sc[0][1], src);
  const float v10 = __shfl_sync(0xFFFFFFFFu, sc[1][0], src), v11 = __shfl_sync(0xFFFFFFFFu, sc[1][1], src);
  const bool high = (lane >> 3) & 1;
  return (lane >> 4) ? (high ? v11 : v10) : (high ? v01 : v00);
}

__device__ __forceinline__ int hist_bin(float z) {
  const float t = (fminf(fmaxf(z, HIST_LO), HIST_HI - 1e-3f) - HIST_LO) * ((float)HIST_BINS / (HIST_HI - HIST_LO));
  return min(HIST_BINS - 1, max(0, (int)t));
}

// Joins into the HBM store that also stamp the variable's last-change round.
struct StampStore {
  int2 *s;
  int *last;
  int round;
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
    if (n) {
      last[v] = round;
      if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    }
    return n;
  }
};

__device__ __forceinline__ int bc_get(const int *a, long long i) { return __ldg(a + i); }

// Threshold bin of this CTA's top fraction: the highest bin b such that the
// count of the CTA's scores in bins >= b reaches k = ceil(frac x the CTA's
// scored propagators) (bin 0 when it never does), from the CTA's histogram
// `sh` in shared memory, by a block-wide suffix sum: thread t owns the bins
// of segment t counted from the top.
__device__ int select_bin(const unsigned *sh, float frac) {
  __shared__ unsigned long long s_warp[32];
  __shared__ int s_bin;
  const int tid = threadIdx.x, nt = blockDim.x, per = (HIST_BINS + nt - 1) / nt;
  if (tid == 0) s_bin = 0;
  const int hi = HIST_BINS - tid * per;  // segment [hi - per, hi)
  unsigned long long seg = 0;
  for (int b = hi - 1; b >= hi - per && b >= 0; --b) seg += sh[b];
  // inclusive prefix over threads 0..tid (the bins from the top down to this segment)
  const int lane = tid & 31, warp = tid >> 5;
  unsigned long long x = seg;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < (nt >> 5) ? s_warp[lane] : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (nt >> 5)) s_warp[lane] = w;
  }
  __syncthreads();
  const unsigned long long total = s_warp[(nt >> 5) - 1];
  const unsigned long long k =
      total ? (unsigned long long)fmax(1.0, ceil((double)frac * (double)total)) : 1ull;
  const unsigned long long incl = x + (warp ? s_warp[warp - 1] : 0ull), above = incl - seg;
  if (above < k && incl >= k) {
    // the crossing is in this segment: walk it from the top
    unsigned long long acc = above;
    for (int b = hi - 1; b >= hi - per && b >= 0; --b) {
      acc += sh[b];
      if (acc >= k) {
        s_bin = b;
        break;
      }
    }
  }
  __syncthreads();
  return s_bin;
}

struct LearnedArgs {
  const int *op, *x, *y, *z;
  long long n;
  int2 *store;
  int *var_last;
  const unsigned char *pdeg;
  const __nv_bfloat16 *wbf;
  float *score;
  unsigned long long *counts;  // [0] woken executions
  Control *ctl;
  long long max_rounds;
  long long timeout_ns;
  float frac;  // fraction of each CTA's propagators woken per round
};

// Persistent learned fixpoint: per learned round, (A) each CTA scores its
// propagators into a histogram in shared memory, (B) derives the threshold of
// its top fraction, (C) runs its woken propagators; one grid barrier per
// round carries the change bit.  A learned round without change is followed
// by a certifying full sweep.
__global__ void __launch_bounds__(256) k_fixpoint_learned(LearnedArgs a) {
  __shared__ float sw[NPARAM];
  __shared__ unsigned sh[HIST_BINS];
  __shared__ unsigned s_word;
  __shared__ __align__(16) __nv_bfloat16 s_tile[256 / 32][32 * NF];
  stage_weights(a.wbf, sw);
  MmaWeights W;
  W.load(a.wbf);
  __nv_bfloat16 *tile = s_tile[threadIdx.x >> 5];
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long gstride = (long long)gridDim.x * blockDim.x;
  const long long gwarp = gtid >> 5, nwarps = gstride >> 5;
  const int lane = threadIdx.x & 31;
  unsigned long long woken = 0, narrowed = 0;
  long long round = 0, nbar = 0;  // nbar: grid barriers passed (thread 0)
  bool certify = false;
  for (;;) {
    ++round;
    const int r = (int)round;
    StampStore st{a.store, a.var_last, r};
    int changed = 0, failed = 0;
    if (!certify) {
      // (A) scores and histogram
      for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x) sh[i] = 0;
      __syncthreads();
      // 32 propagators per warp and step (the loop bound is warp-uniform:
      // the tensor-core products need every lane)
      for (long long w = gwarp; w * 32 < a.n; w += nwarps) {
        const long long p = w * 32 + lane;
        float f[NF] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (p < a.n) {
          const int o = bc_get(a.op, p), X = bc_get(a.x, p), Y = bc_get(a.y, p), Z = bc_get(a.z, p);
          const Itv ia = st.load(X), ib = st.load(Y), ic = st.load(Z);
          const int last = max(__ldcg(a.var_last + X), max(__ldcg(a.var_last + Y), __ldcg(a.var_last + Z)));
          features(o, ia, ib, ic, last, r, a.pdeg[p], f);
        }
        const float s = mlp_forward_mma(f, W, sw, tile);
        if (p < a.n) {
          a.score[p] = s;
          atomicAdd(&sh[hist_bin(s)], 1u);
        }
      }
      __syncthreads();
      // (B) this CTA's threshold: the propagators it scored are the ones it runs
      const int bin = select_bin(sh, a.frac);
      // (C) woken propagators
      for (long long p = gtid; p < a.n; p += gstride) {
        if (hist_bin(__ldcg(a.score + p)) < bin) continue;
        ++woken;
        const int o = bc_get(a.op, p), X = bc_get(a.x, p), Y = bc_get(a.y, p), Z = bc_get(a.z, p);
        const Itv ia = st.load(X), ib = st.load(Y), ic = st.load(Z);
        changed += deduce_loaded(o, X, Y, Z, ia, ib, ic, st, failed);
      }
    } else {
      // certifying full sweep
      for (long long p = gtid; p < a.n; p += gstride) {
        const int o = bc_get(a.op, p), X = bc_get(a.x, p), Y = bc_get(a.y, p), Z = bc_get(a.z, p);
        const Itv ia = st.load(X), ib = st.load(Y), ic = st.load(Z);
        changed += deduce_loaded(o, X, Y, Z, ia, ib, ic, st, failed);
      }
    }
    narrowed += changed;
    const int any_changed = __syncthreads_or(changed);
    const int any_failed = __syncthreads_or(failed);
    if (threadIdx.x == 0) s_word = grid_sync_rot(a.ctl, gridDim.x, nbar++, any_changed, any_failed, a.timeout_ns);
    __syncthreads();
    const unsigned w = s_word;
    if (w & BIT_ERROR) break;
    bool stop = false;
    if (w & BIT_FAILED) {
      stop = true;
      if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->failed = 1;
    } else if (certify) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.counts + 1, 1ull);
      if (!(w & BIT_CHANGED)) stop = true;  // certified fixpoint
      certify = false;
    } else if (!(w & BIT_CHANGED)) {
      certify = true;
    }
    if (!stop && a.max_rounds > 0 && round >= a.max_rounds) {
      if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->changed[0] = 1;
      stop = true;
    }
    if (stop) break;
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->rounds = round;
  woken = warp_sum64(woken);
  narrowed = warp_sum64(narrowed);
  if ((threadIdx.x & 31) == 0) {
    if (woken) atomicAdd(a.counts, woken);
    if (narrowed) atomicAdd(&a.ctl->narrowed, narrowed);
  }
}

// ------------------------------------------- learned rounds on a frontier ----
//
// The learned schedule for a store that was a fixpoint before a few
// embeddings (a search node: snapshot, embed the branching bounds, fixpoint).
// Only the propagators of variables narrowed since can narrow anything, so a
// round scores only its frontier -- the propagators of the variables the
// previous round narrowed, and those deferred -- and the whole run fits one
// CTA (rounds separated by __syncthreads, no grid barrier).  A round wakes the
// frontier entries the network gives a logit of at least 0, and at least the
// top `frac` of the frontier; the others are deferred to the next round (so
// every listed propagator runs at least once after its last listing, and a
// propagator listed in several rounds may run once).  The first join of a
// round that narrows a variable puts the variable on the round's list, and
// after the round the CTA lists those variables' propagators for the next
// round (expand_vars).  When the frontier is
// empty, a certifying round runs, trusting none of the bookkeeping, every
// propagator of every variable embedded or narrowed in this run (the others
// read only intervals of the fixpoint the run started from); if it narrows
// something the rounds resume, else the store is the fixpoint, the same as
// AC-1's bit for bit (propagators are monotone).  Round ids are absolute
// (base + round) so that the per-propagator and per-variable stamps need no
// clearing between runs.  A frontier or a set of narrowed variables beyond
// the lists' capacity stops the run (LOC_OVERFLOW); the host then finishes
// with the grid kernel, whose full certifying sweep does not depend on how
// the store was reached.
constexpr int LOC_BLOCK = 512;
constexpr int LOC_FCAP = 1 << 16;   // entries of one frontier list
constexpr int LOC_CVCAP = 1 << 16;  // variables embedded or narrowed in one run
constexpr int LOC_SINCE_CAP = 1 << 14;  // embedded variables the host hands over
constexpr int LOC_DONE = 1, LOC_FAILED = 2, LOC_CAP = 3, LOC_OVERFLOW = 4;

struct LocalArgs {
  const int4 *bc;                 // {op, x, y, z} per propagator
  const int *adj_ptr, *adj;       // variable -> propagator adjacency
  int2 *store;
  unsigned *vlast;                // per variable: id of the round of its last narrowing (base: embedded)
  unsigned *pstamp;               // per propagator: id of the last round it is listed for
  const unsigned char *pdeg;
  const __nv_bfloat16 *wbf;
  int *F0, *F1;                   // frontier lists of even / odd rounds
  float *score;                   // per frontier slot
  int *cv;                        // variables embedded or narrowed in this run
  int *nv;                        // variables narrowed in the current round
  const int *since;               // the embedded variables
  int nsince;
  unsigned base;                  // id of round r: base + r
  unsigned long long *counts;     // [0] executions of scored rounds, [1] of certifying rounds,
                                  // [2] certifying rounds, [3] end state (LOC_*)
  Control *ctl;
  long long max_rounds;
  float frac;
};

// Joins into the store; the first join of a round that narrows a variable
// appends the variable to the round's list of narrowed variables (their
// propagators are listed for the next round by expand_vars, by the whole CTA).
struct FrontierStore {
  int2 *s;
  unsigned *vlast;
  unsigned base, rid;  // this run, this round
  int *nv, *nnv, *cv, *ncv, *over;
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
    if (!n) return 0;
    if (is_bot(mk(max(seen.l, r.l), min(seen.u, r.u)))) failed = 1;
    const unsigned old = atomicMax(vlast + v, rid);
    if (old < base) {
      const int k = atomicAdd(ncv, 1);
      if (k < LOC_CVCAP) cv[k] = v;
      else *over = 1;
    }
    if (old < rid) {
      const int k = atomicAdd(nnv, 1);
      if (k < LOC_CVCAP) nv[k] = v;
      else *over = 1;
    }
    return n;
  }
};

// Exclusive prefix sum over the CTA (blockDim.x a multiple of 32, at most
// 1,024); *total gets the sum.  Every thread must call it.
__device__ __forceinline__ int block_excl_scan(int x, int *s_warp, int *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int incl = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < nw ? s_warp[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  *total = s_warp[nw - 1];
  const int r = incl - x + (warp ? s_warp[warp - 1] : 0);
  __syncthreads();  // s_warp is free again
  return r;
}

// The propagators of vars[0 .. count) listed as round `id`'s frontier (each
// once: the per-propagator stamp), by the whole CTA: the adjacency entries of
// up to blockDim.x variables at a time are flattened (a block scan of their
// degrees) and spread over the threads, so the stamp atomics are issued in
// parallel instead of one variable's entries after another.
__device__ void expand_vars(const LocalArgs &a, const int *vars, int count, unsigned id, int *f, int *nf,
                            int *over, int *s_off, int *s_start, int *s_warp) {
  const int tid = threadIdx.x;
  for (int c0 = 0; c0 < count; c0 += blockDim.x) {
    const int m = min(count - c0, (int)blockDim.x);
    int deg = 0, start = 0;
    if (tid < m) {
      const int v = vars[c0 + tid];
      start = __ldg(a.adj_ptr + v);
      deg = __ldg(a.adj_ptr + v + 1) - start;
    }
    int total = 0;
    const int off = block_excl_scan(deg, s_warp, &total);
    s_off[tid] = off;
    s_start[tid] = start;
    __syncthreads();
    for (int j = tid; j < total; j += blockDim.x) {
      int lo = 0, hi = m - 1;  // the last variable whose entries start at or before j
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_off[mid] <= j) lo = mid;
        else hi = mid - 1;
      }
      const int p = __ldg(a.adj + s_start[lo] + (j - s_off[lo]));
      if (atomicMax(a.pstamp + p, id) < id) {
        const int k = atomicAdd(nf, 1);
        if (k < LOC_FCAP) f[k] = p;
        else *over = 1;
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(LOC_BLOCK, 1) k_learned_local(LocalArgs a) {
  __shared__ float sw[NPARAM];
  __shared__ unsigned sh[HIST_BINS];
  __shared__ __align__(16) __nv_bfloat16 s_tile[LOC_BLOCK / 32][32 * NF];
  __shared__ int s_off[LOC_BLOCK], s_start[LOC_BLOCK], s_warp[32];
  __shared__ int s_nf[2], s_ncv, s_nnv, s_over;
  stage_weights(a.wbf, sw);
  MmaWeights W;
  W.load(a.wbf);
  __nv_bfloat16 *tile = s_tile[threadIdx.x >> 5];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_nf[0] = s_nf[1] = 0;
    s_ncv = 0;
    s_nnv = 0;
    s_over = 0;
  }
  __syncthreads();
  // the embedded variables start the run (round 0) and list round 1
  for (int i = tid; i < a.nsince; i += blockDim.x) {
    const int v = a.since[i];
    if (atomicMax(a.vlast + v, a.base) < a.base) {
      const int k = atomicAdd(&s_ncv, 1);
      if (k < LOC_CVCAP) a.cv[k] = v;
      else s_over = 1;
    }
  }
  __syncthreads();
  expand_vars(a, a.cv, min(s_ncv, LOC_CVCAP), a.base + 1u, a.F1, &s_nf[1], &s_over, s_off, s_start, s_warp);
  unsigned long long ex = 0, cex = 0, narrowed = 0;
  long long round = 0;
  int state = 0, certifying = 0, ncert = 0;
  for (;;) {
    ++round;
    const int cur = (int)(round & 1), nxt = cur ^ 1;
    int *F = cur ? a.F1 : a.F0, *Fn = cur ? a.F0 : a.F1;
    const unsigned rid = a.base + (unsigned)round, nid = rid + 1u;
    if (s_over) {
      state = LOC_OVERFLOW;
      break;
    }
    if (s_nf[cur] == 0) {
      // certifying round: every propagator of every variable of this run
      __syncthreads();
      expand_vars(a, a.cv, min(s_ncv, LOC_CVCAP), rid, F, &s_nf[cur], &s_over, s_off, s_start, s_warp);
      certifying = 1;
      ++ncert;
      if (s_over) {
        state = LOC_OVERFLOW;
        break;
      }
    }
    const int n = min(s_nf[cur], LOC_FCAP);
    for (int i = tid; i < HIST_BINS; i += blockDim.x) sh[i] = 0;
    if (tid == 0) {
      s_nf[nxt] = 0;
      s_nnv = 0;
    }
    __syncthreads();
    FrontierStore st{a.store, a.vlast, a.base, rid, a.nv, &s_nnv, a.cv, &s_ncv, &s_over};
    int changed = 0, failed = 0;
    int bin = 0;
    // (A) scores of the frontier, 32 entries per warp and step (warp-uniform bound)
    if (!certifying) {
      for (int b = warp * 32; b < n; b += blockDim.x) {
        const int i = b + lane;
        float f[NF] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (i < n) {
          const int p = F[i];
          const int4 c = __ldg(a.bc + p);
          const Itv ia = st.load(c.y), ib = st.load(c.z), ic = st.load(c.w);
          const unsigned last = max(__ldcg(a.vlast + c.y), max(__ldcg(a.vlast + c.z), __ldcg(a.vlast + c.w)));
          // rounds since a variable of the propagator last narrowed ("long ago" before this run)
          const int since = last < a.base ? 64 : (int)min(rid - last, 64u);
          features(c.x, ia, ib, ic, (int)round - since, (int)round, a.pdeg[p], f);
        }
        const float s = mlp_forward_mma(f, W, sw, tile);
        if (i < n) {
          a.score[i] = s;
          atomicAdd(&sh[hist_bin(s)], 1u);
        }
      }
      __syncthreads();
      // (B) at least the top frac, and every entry with a logit >= 0
      bin = min(select_bin(sh, a.frac), hist_bin(0.f));
    }
    // (C) the woken entries run, the others wait for the next round
    for (int i = tid; i < n; i += blockDim.x) {
      const int p = F[i];
      if (!certifying && hist_bin(a.score[i]) < bin) {
        if (atomicMax(a.pstamp + p, nid) < nid) {
          const int k = atomicAdd(&s_nf[nxt], 1);
          if (k < LOC_FCAP) Fn[k] = p;
          else s_over = 1;
        }
        continue;
      }
      const int4 c = __ldg(a.bc + p);
      const Itv ia = st.load(c.y), ib = st.load(c.z), ic = st.load(c.w);
      changed += deduce_loaded(c.x, c.y, c.z, c.w, ia, ib, ic, st, failed);
      if (certifying) ++cex;
      else ++ex;
    }
    narrowed += changed;
    const int any_ch = __syncthreads_or(changed);
    const int any_f = __syncthreads_or(failed);
    if (any_f) {
      state = LOC_FAILED;
      break;
    }
    if (certifying && !any_ch) {
      state = LOC_DONE;
      break;
    }
    certifying = 0;
    if (a.max_rounds > 0 && round >= a.max_rounds) {
      state = LOC_CAP;
      break;
    }
    // the propagators of the variables this round narrowed, for the next round
    expand_vars(a, a.nv, min(s_nnv, LOC_CVCAP), nid, Fn, &s_nf[nxt], &s_over, s_off, s_start, s_warp);
  }
  ex = warp_sum64(ex);
  cex = warp_sum64(cex);
  narrowed = warp_sum64(narrowed);
  if (lane == 0) {
    if (ex) atomicAdd(a.counts, ex);
    if (cex) atomicAdd(a.counts + 1, cex);
    if (narrowed) atomicAdd(&a.ctl->narrowed, narrowed);
  }
  if (tid == 0) {
    a.counts[2] = (unsigned long long)ncert;
    a.counts[3] = (unsigned long long)state;
    a.ctl->rounds = round;
    if (state == LOC_FAILED) a.ctl->failed = 1;
    if (state == LOC_CAP) a.ctl->changed[0] = 1;
  }
}

// One traced AC-1 round: features at the time each propagator is read, then
// the propagator; label = it narrowed a bound.  Positives are always kept,
// negatives with probability keep_neg (a hash of round and index).
__global__ void __launch_bounds__(256) k_trace_round(const int *op, const int *x, const int *y, const int *z,
                                                     long long n, int2 *store, int *var_last,
                                                     const unsigned char *pdeg, int round, float keep_neg,
                                                     unsigned seed, float *tx, float *ty, long long tcap,
                                                     unsigned long long *tcount, Control *ctl) {
  StampStore st{store, var_last, round};
  int changed = 0, failed = 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int o = op[p], X = x[p], Y = y[p], Z = z[p];
    const Itv ia = st.load(X), ib = st.load(Y), ic = st.load(Z);
    const int last = max(__ldcg(var_last + X), max(__ldcg(var_last + Y), __ldcg(var_last + Z)));
    float f[NF];
    features(o, ia, ib, ic, last, round, pdeg[p], f);
    const int ch = deduce_loaded(o, X, Y, Z, ia, ib, ic, st, failed);
    changed += ch;
    unsigned h = (unsigned)p * 0x9E3779B1u ^ ((unsigned)round * 0x85EBCA77u) ^ seed;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    const bool keep = ch > 0 || (float)(h & 0xFFFFFF) < keep_neg * 16777216.f;
    if (keep) {
      const unsigned long long slot = atomicAdd(tcount, 1ull);
      if ((long long)slot < tcap) {
#pragma unroll
        for (int i = 0; i < NF; ++i) tx[slot * NF + i] = f[i];
        ty[slot] = ch > 0 ? 1.f : 0.f;
      }
    }
  }
  const unsigned any_ch = __any_sync(0xFFFFFFFFu, changed), any_f = __any_sync(0xFFFFFFFFu, failed);
  if ((threadIdx.x & 31) == 0) {
    if (any_ch) atomicOr(&ctl->changed[0], 1);
    if (any_f) atomicOr(&ctl->failed, 1);
  }
}

// Weighted binary cross-entropy with logits: one sample per thread; weight
// gradients reduced over the CTA in shared memory, then added to `grad`.
__global__ void __launch_bounds__(TRAIN_CTA) k_mlp_grad(const float *X, const float *Y, const int *idx,
                                                       long long count, const __nv_bfloat16 *wbf, float pos_weight,
                                                       float inv_batch, float *grad, float *loss) {
  extern __shared__ float smem[];
  float *sw = smem;                                // NPARAM
  float *H1 = sw + ((NPARAM + 31) / 32) * 32;      // TRAIN_CTA x (NH+1)
  float *H2 = H1 + TRAIN_CTA * (NH + 1);
  float *D2 = H2 + TRAIN_CTA * (NH + 1);           // dL/d(pre-activation 2)
  float *D1 = D2 + TRAIN_CTA * (NH + 1);           // dL/d(pre-activation 1)
  float *XS = D1 + TRAIN_CTA * (NH + 1);           // TRAIN_CTA x NF
  float *DZ = XS + TRAIN_CTA * NF;                 // TRAIN_CTA
  __shared__ float s_loss;
  stage_weights(wbf, sw);
  if (threadIdx.x == 0) s_loss = 0.f;
  __syncthreads();
  const int t = threadIdx.x;
  const long long sidx = blockIdx.x * (long long)TRAIN_CTA + t;
  float f[NF];
  float yv = 0.f;
  const bool valid = sidx < count;
  if (valid) {
    const long long s = idx ? idx[sidx] : sidx;
#pragma unroll
    for (int i = 0; i < NF; ++i) f[i] = X[s * NF + i];
    yv = Y[s];
  } else {
#pragma unroll
    for (int i = 0; i < NF; ++i) f[i] = 0.f;
  }
#pragma unroll
  for (int i = 0; i < NF; ++i) XS[t * NF + i] = f[i];
  float h1[NH], h2[NH];
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B1 + j];
#pragma unroll
    for (int i = 0; i < NF; ++i) a = fmaf(sw[OFF_W1 + j * NF + i], f[i], a);
    h1[j] = fmaxf(a, 0.f);
    H1[t * (NH + 1) + j] = h1[j];
  }
  float z = sw[OFF_B3];
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B2 + j];
#pragma unroll
    for (int i = 0; i < NH; ++i) a = fmaf(sw[OFF_W2 + j * NH + i], h1[i], a);
    h2[j] = fmaxf(a, 0.f);
    H2[t * (NH + 1) + j] = h2[j];
    z = fmaf(sw[OFF_W3 + j], h2[j], z);
  }
  // loss = w * (softplus(z) - y z), dz = w * (sigmoid(z) - y) / batch
  const float w = valid ? (yv > 0.5f ? pos_weight : 1.f) : 0.f;
  const float sp = z > 0.f ? z + log1pf(__expf(-z)) : log1pf(__expf(z));
  const float sig = 1.f / (1.f + __expf(-z));
  const float dz = w * (sig - yv) * inv_batch;
  DZ[t] = dz;
  atomicAdd(&s_loss, w * (sp - yv * z));
#pragma unroll
  for (int j = 0; j < NH; ++j) D2[t * (NH + 1) + j] = h2[j] > 0.f ? dz * sw[OFF_W3 + j] : 0.f;
#pragma unroll
  for (int i = 0; i < NH; ++i) {
    float a = 0.f;
#pragma unroll
    for (int j = 0; j < NH; ++j) a = fmaf(sw[OFF_W2 + j * NH + i], D2[t * (NH + 1) + j], a);
    D1[t * (NH + 1) + i] = h1[i] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // weight gradients: reductions over the CTA's samples
  for (int e = t; e < NPARAM; e += TRAIN_CTA) {
    float g = 0.f;
    if (e < OFF_B1) {
      const int j = e / NF, i = e % NF;
      for (int s = 0; s < TRAIN_CTA; ++s) g = fmaf(D1[s * (NH + 1) + j], XS[s * NF + i], g);
    } else if (e < OFF_W2) {
      const int j = e - OFF_B1;
      for (int s = 0; s < TRAIN_CTA; ++s) g += D1[s * (NH + 1) + j];
    } else if (e < OFF_B2) {
      const int j = (e - OFF_W2) / NH, i = (e - OFF_W2) % NH;
      for (int s = 0; s < TRAIN_CTA; ++s) g = fmaf(D2[s * (NH + 1) + j], H1[s * (NH + 1) + i], g);
    } else if (e < OFF_W3) {
      const int j = e - OFF_B2;
      for (int s = 0; s < TRAIN_CTA; ++s) g += D2[s * (NH + 1) + j];
    } else if (e < OFF_B3) {
      const int j = e - OFF_W3;
      for (int s = 0; s < TRAIN_CTA; ++s) g = fmaf(DZ[s], H2[s * (NH + 1) + j], g);
    } else {
      for (int s = 0; s < TRAIN_CTA; ++s) g += DZ[s];
    }
    atomicAdd(grad + e, g);
  }
  if (threadIdx.x == 0) atomicAdd(loss, s_loss);
}

// Adam on the FP32 master parameters; the BF16 copy is refreshed.
__global__ void k_adam(float *param, float *grad, float *m, float *v, __nv_bfloat16 *wbf, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float p = param[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  param[i] = p;
  wbf[i] = __float2bfloat16_rn(p);
  grad[i] = 0.f;
}

__global__ void k_to_bf16(const float *param, __nv_bfloat16 *wbf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NPARAM) wbf[i] = __float2bfloat16_rn(param[i]);
}

__global__ void k_degree(const int *x, const int *y, const int *z, long long n, int *deg) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    atomicAdd(deg + x[p], 1);
    atomicAdd(deg + y[p], 1);
    atomicAdd(deg + z[p], 1);
  }
}

__global__ void k_prop_degree(const int *x, const int *y, const int *z, long long n, const int *deg,
                              unsigned char *pdeg) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float d = (float)(deg[x[p]] + deg[y[p]] + deg[z[p]]);
    pdeg[p] = (unsigned char)min(255.f, __log2f(d + 1.f) * 16.f);
  }
}

__global__ void k_fill_int(int *a, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}

__global__ void k_mark(int *a, const int *idx, int count, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) a[idx[i]] = v;
}

// ------------------------------------------------------------------ host -----

SchedState *sched(pirgpu_ctx *ctx) {
  if (!ctx->sched) ctx->sched = new SchedState();
  return ctx->sched;
}

// Parameters: allocated once per context, initialized with a fixed-seed
// He-uniform draw.
int ensure_params(pirgpu_ctx *ctx) {
  SchedState *s = sched(ctx);
  if (s->d_param) return PIR_OK;
  const size_t b = NPARAM * sizeof(float);
  if (cudaMalloc(&s->d_param, b) != cudaSuccess || cudaMalloc(&s->d_m, b) != cudaSuccess ||
      cudaMalloc(&s->d_v, b) != cudaSuccess || cudaMalloc(&s->d_grad, b) != cudaSuccess ||
      cudaMalloc(&s->d_loss, sizeof(float)) != cudaSuccess ||
      cudaMalloc(&s->d_wbf, NPARAM * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&s->d_counts, 4 * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "scheduler parameters");
  }
  std::vector<float> p(NPARAM, 0.f);
  std::mt19937 g(12345);
  auto fill = [&](int off, int cnt, int fan_in) {
    std::uniform_real_distribution<float> u(-std::sqrt(6.f / fan_in), std::sqrt(6.f / fan_in));
    for (int i = 0; i < cnt; ++i) p[off + i] = u(g);
  };
  fill(OFF_W1, NH * NF, NF);
  fill(OFF_W2, NH * NH, NH);
  fill(OFF_W3, NH, NH);
  PIR_CK(cudaMemcpyAsync(s->d_param, p.data(), b, cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_m, 0, b, ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_v, 0, b, ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_grad, 0, b, ctx->stream));
  k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(s->d_param, s->d_wbf);
  PIR_CK(cudaGetLastError());
  s->adam_t = 0;
  return PIR_OK;
}

// Per-variable and per-propagator buffers for the current bytecode.
int ensure_graph(pirgpu_ctx *ctx) {
  SchedState *s = sched(ctx);
  if (s->bc_version == ctx->bytecode_version && s->nvars == ctx->nvars && s->d_var_last) return PIR_OK;
  void *ptrs[] = {s->d_var_last, s->d_deg, s->d_pdeg, s->d_score};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  s->d_var_last = s->d_deg = nullptr;
  s->d_pdeg = nullptr;
  s->d_score = nullptr;
  const size_t nv = std::max(ctx->nvars, 1), n = (size_t)std::max<long long>(ctx->n, 1);
  if (cudaMalloc(&s->d_var_last, nv * sizeof(int)) != cudaSuccess || cudaMalloc(&s->d_deg, nv * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_pdeg, n) != cudaSuccess || cudaMalloc(&s->d_score, n * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "scheduler buffers");
  }
  PIR_CK(cudaMemsetAsync(s->d_deg, 0, nv * sizeof(int), ctx->stream));
  const int grid = ctx->num_sms * 4;
  if (ctx->n > 0) {
    k_degree<<<grid, 256, 0, ctx->stream>>>(ctx->d_x, ctx->d_y, ctx->d_z, ctx->n, s->d_deg);
    k_prop_degree<<<grid, 256, 0, ctx->stream>>>(ctx->d_x, ctx->d_y, ctx->d_z, ctx->n, s->d_deg, s->d_pdeg);
  }
  PIR_CK(cudaGetLastError());
  s->bc_version = ctx->bytecode_version;
  s->nvars = ctx->nvars;
  s->n = ctx->n;
  return PIR_OK;
}

// Start-of-fixpoint stamps: every variable "long ago", the variables embedded
// since the last fixpoint "just changed" (round 0).
int reset_stamps(pirgpu_ctx *ctx) {
  SchedState *s = sched(ctx);
  k_fill_int<<<ctx->num_sms * 2, 256, 0, ctx->stream>>>(s->d_var_last, ctx->nvars, -64);
  if (!s->dirty.empty()) {
    const int cnt = (int)s->dirty.size();
    int r;
    if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, cnt * sizeof(int)))) return r;
    PIR_CK(cudaMemcpyAsync(ctx->d_scratch, s->dirty.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    k_mark<<<(cnt + 255) / 256, 256, 0, ctx->stream>>>(s->d_var_last, (const int *)ctx->d_scratch, cnt, 0);
    s->dirty.clear();
  }
  PIR_CK(cudaGetLastError());
  return PIR_OK;
}

void note_embedded(pirgpu_ctx *ctx, const int32_t *var, int count) {
  SchedState *s = sched(ctx);
  // the embedding that follows bumps the store version once: the chain from
  // the last fixpoint goes on if nothing else changed the store in between
  if (s->since_ok && s->base_version == ctx->store_version && s->base_bc == ctx->bytecode_version &&
      s->since.size() + (size_t)count <= (size_t)LOC_SINCE_CAP) {
    s->since.insert(s->since.end(), var, var + count);
    s->base_version = ctx->store_version + 1;
  } else {
    s->since_ok = false;
  }
  if (s->dirty.size() > (size_t)1 << 22) return;
  s->dirty.insert(s->dirty.end(), var, var + count);
}

void note_fixpoint(pirgpu_ctx *ctx) {
  SchedState *s = sched(ctx);
  s->base_version = ctx->store_version;
  s->base_bc = ctx->bytecode_version;
  s->since.clear();
  s->since_ok = true;
}

// Buffers of the frontier rounds: stamps sized to the bytecode and the store
// (cleared when allocated; round ids only grow between runs), frontier lists,
// scores, the run's variables and the embedded ones.
static int ensure_local(pirgpu_ctx *ctx) {
  SchedState *s = sched(ctx);
  if (s->d_vlast && s->loc_bc_version == ctx->bytecode_version && s->loc_nvars == ctx->nvars && s->loc_n == ctx->n)
    return PIR_OK;
  void *ptrs[] = {s->d_vlast, s->d_pstamp, s->d_lf, s->d_cv, s->d_since, s->d_lscore, s->d_nv};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  s->d_vlast = s->d_pstamp = nullptr;
  s->d_lf = s->d_cv = s->d_since = s->d_nv = nullptr;
  s->d_lscore = nullptr;
  const size_t nv = (size_t)std::max(ctx->nvars, 1), n = (size_t)std::max<long long>(ctx->n, 1);
  if (cudaMalloc(&s->d_vlast, nv * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&s->d_pstamp, n * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&s->d_lf, 2 * (size_t)LOC_FCAP * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_cv, (size_t)LOC_CVCAP * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_nv, (size_t)LOC_CVCAP * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_since, (size_t)LOC_SINCE_CAP * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&s->d_lscore, (size_t)LOC_FCAP * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "learned frontier buffers");
  }
  PIR_CK(cudaMemsetAsync(s->d_vlast, 0, nv * sizeof(unsigned), ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_pstamp, 0, n * sizeof(unsigned), ctx->stream));
  s->loc_base = 65;
  s->loc_bc_version = ctx->bytecode_version;
  s->loc_nvars = ctx->nvars;
  s->loc_n = ctx->n;
  return PIR_OK;
}

// The learned rounds on a frontier (k_learned_local), from the fixpoint the
// store was at before the embeddings in `since`.  *handed_over: the lists
// overflowed, the grid kernel finishes the run (stats so far in *st).
static int fixpoint_learned_local(pirgpu_ctx *ctx, const pir_opts &opts, float frac, pir_stats *st,
                                  bool *handed_over) {
  SchedState *s = sched(ctx);
  int r;
  EventsGraph g;
  if ((r = events_graph(ctx, &g, false)) || (r = ensure_local(ctx))) return r;
  if (s->loc_base > 0xF0000000u) {
    PIR_CK(cudaMemsetAsync(s->d_vlast, 0, (size_t)std::max(ctx->nvars, 1) * sizeof(unsigned), ctx->stream));
    PIR_CK(cudaMemsetAsync(s->d_pstamp, 0, (size_t)std::max<long long>(ctx->n, 1) * sizeof(unsigned), ctx->stream));
    s->loc_base = 65;
  }
  const int nsince = (int)s->since.size();
  if (nsince)
    PIR_CK(cudaMemcpyAsync(s->d_since, s->since.data(), nsince * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if ((r = reset_control(ctx))) return r;
  PIR_CK(cudaMemsetAsync(s->d_counts, 0, 4 * sizeof(unsigned long long), ctx->stream));
  LocalArgs a;
  a.bc = g.bc;
  a.adj_ptr = g.adj_ptr;
  a.adj = g.adj;
  a.store = ctx->d_store;
  a.vlast = s->d_vlast;
  a.pstamp = s->d_pstamp;
  a.pdeg = s->d_pdeg;
  a.wbf = s->d_wbf;
  a.F0 = s->d_lf;
  a.F1 = s->d_lf + LOC_FCAP;
  a.score = s->d_lscore;
  a.cv = s->d_cv;
  a.nv = s->d_nv;
  a.since = s->d_since;
  a.nsince = nsince;
  a.base = s->loc_base;
  a.counts = s->d_counts;
  a.ctl = ctx->d_ctl;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.frac = frac;
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  k_learned_local<<<1, LOC_BLOCK, 0, ctx->stream>>>(a);
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  unsigned long long cnt[4];
  PIR_CK(cudaMemcpyAsync(cnt, s->d_counts, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
  if ((r = read_control(ctx, &h))) return r;
  std::memset(st, 0, sizeof(*st));
  PIR_CK(cudaEventElapsedTime(&st->device_ms, ctx->ev0, ctx->ev1));
  s->loc_base += (unsigned)h.rounds + 2u;
  st->rounds = h.rounds;
  st->narrowed = (int64_t)h.narrowed;
  st->executions = (int64_t)(cnt[0] + cnt[1]);
  st->certify_executions = (int64_t)cnt[1];
  *handed_over = cnt[3] == (unsigned long long)LOC_OVERFLOW;
  st->status = cnt[3] == (unsigned long long)LOC_FAILED ? PIR_FAILED
               : cnt[3] == (unsigned long long)LOC_CAP  ? PIR_TIMEOUT
                                                        : PIR_OK;
  return PIR_OK;
}

int fixpoint_learned(pirgpu_ctx *ctx, const pir_opts &opts, pir_stats *stats) {
  int r;
  if ((r = ensure_params(ctx)) || (r = ensure_graph(ctx))) return r;
  SchedState *s = sched(ctx);
  const float frac = opts.wake_fraction > 0.f ? std::min(opts.wake_fraction, 1.f) : 1.f / 16.f;
  // pir_fixpoint bumped the store version once since the embeddings
  pir_stats pre;
  std::memset(&pre, 0, sizeof(pre));
  if (opts.local_frontier >= 0 && s->since_ok && s->base_version + 1 == ctx->store_version &&
      s->base_bc == ctx->bytecode_version) {
    bool handed_over = false;
    if ((r = fixpoint_learned_local(ctx, opts, frac, &pre, &handed_over))) return r;
    if (!handed_over) {
      s->dirty.clear();
      if (pre.status == PIR_FAILED) ctx->failed = true;
      ctx->at_fixpoint = pre.status == PIR_OK;
      if (stats) *stats = pre;
      return pre.status;
    }
  }
  if ((r = reset_stamps(ctx))) return r;
  if ((r = reset_control(ctx))) return r;
  PIR_CK(cudaMemsetAsync(s->d_counts, 0, 4 * sizeof(unsigned long long), ctx->stream));
  LearnedArgs a;
  a.op = ctx->d_op;
  a.x = ctx->d_x;
  a.y = ctx->d_y;
  a.z = ctx->d_z;
  a.n = ctx->n;
  a.store = ctx->d_store;
  a.var_last = s->d_var_last;
  a.pdeg = s->d_pdeg;
  a.wbf = s->d_wbf;
  a.score = s->d_score;
  a.counts = s->d_counts;
  a.ctl = ctx->d_ctl;
  a.max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  a.timeout_ns = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  a.frac = frac;
  int occ = 0;
  PIR_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fixpoint_learned, 256, 0));
  if (occ < 1) return set_err(ctx, PIR_ECUDA, "learned kernel does not fit on an SM");
  const int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ;
  const int grid = std::max(1, (int)std::min<long long>((long long)ctx->num_sms * per_sm, (ctx->n + 255) / 256));
  void *args[] = {&a};
  PIR_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  PIR_CK(cudaLaunchCooperativeKernel((const void *)k_fixpoint_learned, dim3(grid), dim3(256), args, 0, ctx->stream));
  PIR_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  unsigned long long cnt[4];
  PIR_CK(cudaMemcpyAsync(cnt, s->d_counts, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
  if ((r = read_control(ctx, &h))) return r;
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  PIR_CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  // executions: woken propagators of the learned rounds + full certifying sweeps
  st.rounds = h.rounds + pre.rounds;
  st.narrowed = (int64_t)h.narrowed + pre.narrowed;
  st.executions = (int64_t)cnt[0] + (int64_t)cnt[1] * ctx->n + pre.executions;
  st.certify_executions = (int64_t)cnt[1] * ctx->n + pre.certify_executions;
  st.device_ms += pre.device_ms;
  int status = h.status ? h.status : (h.failed ? PIR_FAILED : (h.changed[0] ? PIR_TIMEOUT : PIR_OK));
  st.status = status;
  if (status == PIR_FAILED) ctx->failed = true;
  ctx->at_fixpoint = status == PIR_OK;
  if (stats) *stats = st;
  return status;
}

}  // namespace pirgpu

using namespace pirgpu;

extern "C" int pir_sched_collect(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                                 const int32_t *lb, const int32_t *ub, int64_t max_samples, float keep_negative,
                                 int64_t *out_samples, int64_t *out_positives) {
  if (!ctx || nnodes < 0 || max_samples <= 0 || (nnodes > 0 && (!off || !var || !lb || !ub)))
    return PIR_EINVAL;
  ++ctx->store_version;  // the store is used as scratch and put back
  for (int j = 0; j < nnodes; ++j)
    if (off[j + 1] < off[j]) return set_err(ctx, PIR_EINVAL, "node offsets decrease");
  for (int k = 0; k < (nnodes ? off[nnodes] : 0); ++k)
    if (var[k] < 0 || var[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "tightening var out of range");
  if (ctx->n == 0 || ctx->failed) return set_err(ctx, PIR_EINVAL, "nothing to trace");
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure_params(ctx)) || (r = ensure_graph(ctx))) return r;
  SchedState *s = sched(ctx);
  if (s->tcap < max_samples) {
    if (s->d_tx) cudaFree(s->d_tx);
    if (s->d_ty) cudaFree(s->d_ty);
    s->d_tx = s->d_ty = nullptr;
    if (cudaMalloc(&s->d_tx, (size_t)max_samples * NF * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->d_ty, (size_t)max_samples * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      s->tcap = 0;
      return set_err(ctx, PIR_ENOMEM, "trace buffer");
    }
    s->tcap = max_samples;
  }
  // base store saved, restored before every node
  int2 *base = nullptr;
  const size_t sb = (size_t)ctx->nvars * sizeof(int2);
  if (cudaMalloc(&base, sb) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "trace base store");
  }
  PIR_CK(cudaMemcpyAsync(base, ctx->d_store, sb, cudaMemcpyDeviceToDevice, ctx->stream));
  const bool fix0 = ctx->at_fixpoint;
  PIR_CK(cudaMemsetAsync(s->d_counts, 0, 4 * sizeof(unsigned long long), ctx->stream));
  const int grid = std::max(1, (int)std::min<long long>(ctx->num_sms * 8, (ctx->n + 255) / 256));
  unsigned long long tcount = 0;
  long long positives = 0;
  for (int j = 0; j < nnodes && (long long)tcount < max_samples; ++j) {
    PIR_CK(cudaMemcpyAsync(ctx->d_store, base, sb, cudaMemcpyDeviceToDevice, ctx->stream));
    const int cnt = off[j + 1] - off[j];
    std::vector<int> v(var + off[j], var + off[j + 1]), l(lb + off[j], lb + off[j + 1]), u(ub + off[j], ub + off[j + 1]);
    ctx->failed = false;
    if (cnt && (r = pir_embed_many(ctx, cnt, v.data(), l.data(), u.data(), nullptr))) break;
    if ((r = reset_stamps(ctx))) break;
    if (ctx->failed) continue;
    for (int round = 1; round < 100000; ++round) {
      if ((r = reset_control(ctx))) break;
      k_trace_round<<<grid, 256, 0, ctx->stream>>>(ctx->d_op, ctx->d_x, ctx->d_y, ctx->d_z, ctx->n, ctx->d_store,
                                                   s->d_var_last, s->d_pdeg, round, keep_negative,
                                                   0x5EED0000u + (unsigned)j, s->d_tx, s->d_ty, s->tcap, s->d_counts,
                                                   ctx->d_ctl);
      PIR_CK(cudaGetLastError());
      Control h;
      if ((r = read_control(ctx, &h))) break;
      if (h.failed || !h.changed[0]) break;
    }
    if (r) break;
  }
  PIR_CK(cudaMemcpyAsync(ctx->d_store, base, sb, cudaMemcpyDeviceToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(&tcount, s->d_counts, sizeof(tcount), cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(base);
  ctx->failed = false;
  ctx->at_fixpoint = fix0;
  if (r) return r;
  s->tcount = std::min<long long>((long long)tcount, s->tcap);
  if (s->tcount > 0) {
    std::vector<float> ys((size_t)s->tcount);
    PIR_CK(cudaMemcpy(ys.data(), s->d_ty, ys.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (float y : ys) positives += y > 0.5f;
  }
  if (out_samples) *out_samples = s->tcount;
  if (out_positives) *out_positives = positives;
  return PIR_OK;
}

extern "C" int pir_sched_train(pirgpu_ctx *ctx, int32_t epochs, int32_t batch, float lr, float pos_weight,
                               float *out_loss) {
  if (!ctx || epochs < 0 || batch <= 0) return PIR_EINVAL;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure_params(ctx))) return r;
  SchedState *s = sched(ctx);
  if (s->tcount <= 0) return set_err(ctx, PIR_EINVAL, "no trace samples: call pir_sched_collect first");
  const long long N = s->tcount;
  batch = (int)std::min<long long>(((long long)batch + TRAIN_CTA - 1) / TRAIN_CTA * TRAIN_CTA, ((N + TRAIN_CTA - 1) / TRAIN_CTA) * TRAIN_CTA);
  std::vector<int> perm((size_t)N);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937 g(777);
  int *d_idx = nullptr;
  if (cudaMalloc(&d_idx, (size_t)N * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "training index");
  }
  const size_t smem = (((NPARAM + 31) / 32) * 32 + 4 * TRAIN_CTA * (NH + 1) + TRAIN_CTA * NF + TRAIN_CTA) * sizeof(float);
  r = PIR_OK;
  if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    r = cuda_err(ctx, cudaGetLastError(), "k_mlp_grad smem");
  for (int e = 0; e < epochs && !r; ++e) {
    std::shuffle(perm.begin(), perm.end(), g);
    if (cudaMemcpyAsync(d_idx, perm.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(s->d_loss, 0, sizeof(float), ctx->stream) != cudaSuccess) {
      r = cuda_err(ctx, cudaGetLastError(), "training epoch setup");
      break;
    }
    for (long long b0 = 0; b0 < N; b0 += batch) {
      const long long cnt = std::min<long long>(batch, N - b0);
      const int blocks = (int)((cnt + TRAIN_CTA - 1) / TRAIN_CTA);
      k_mlp_grad<<<blocks, TRAIN_CTA, smem, ctx->stream>>>(s->d_tx, s->d_ty, d_idx + b0, cnt, s->d_wbf, pos_weight,
                                                           1.f / (float)cnt, s->d_grad, s->d_loss);
      ++s->adam_t;
      const float b1 = 0.9f, b2 = 0.999f;
      k_adam<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(s->d_param, s->d_grad, s->d_m, s->d_v, s->d_wbf, lr, b1, b2,
                                                            1e-8f, 1.f - std::pow(b1, (float)s->adam_t),
                                                            1.f - std::pow(b2, (float)s->adam_t));
    }
    if (cudaGetLastError() != cudaSuccess) {
      r = set_err(ctx, PIR_ECUDA, "training kernels");
      break;
    }
    float loss = 0.f;
    if (cudaMemcpyAsync(&loss, s->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      r = cuda_err(ctx, cudaGetLastError(), "training loss");
      break;
    }
    if (out_loss) out_loss[e] = loss / (float)N;
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(d_idx);
  if (!r) s->trained = true;
  return r;
}

extern "C" int pir_sched_grad(pirgpu_ctx *ctx, int32_t count, const float *X, const float *Y, float pos_weight,
                              float *grad_out, float *loss_out) {
  if (!ctx || count <= 0 || !X || !Y || !grad_out) return PIR_EINVAL;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure_params(ctx))) return r;
  SchedState *s = sched(ctx);
  const size_t bytes = (size_t)count * (NF + 1) * sizeof(float);
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, bytes))) return r;
  float *dx = (float *)ctx->d_scratch, *dy = dx + (size_t)count * NF;
  PIR_CK(cudaMemcpyAsync(dx, X, (size_t)count * NF * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(dy, Y, (size_t)count * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_grad, 0, NPARAM * sizeof(float), ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_loss, 0, sizeof(float), ctx->stream));
  const size_t smem = (((NPARAM + 31) / 32) * 32 + 4 * TRAIN_CTA * (NH + 1) + TRAIN_CTA * NF + TRAIN_CTA) * sizeof(float);
  PIR_CK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_mlp_grad<<<(count + TRAIN_CTA - 1) / TRAIN_CTA, TRAIN_CTA, smem, ctx->stream>>>(
      dx, dy, nullptr, count, s->d_wbf, pos_weight, 1.f / (float)count, s->d_grad, s->d_loss);
  PIR_CK(cudaGetLastError());
  PIR_CK(cudaMemcpyAsync(grad_out, s->d_grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  float loss = 0.f;
  PIR_CK(cudaMemcpyAsync(&loss, s->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemsetAsync(s->d_grad, 0, NPARAM * sizeof(float), ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  if (loss_out) *loss_out = loss / (float)count;
  return PIR_OK;
}

// Scores of given feature rows with the inference path of the learned
// fixpoint (tensor-core MLP), 32 rows per warp.
__global__ void __launch_bounds__(256) k_score_batch(const __nv_bfloat16 *wbf, const float *X, long long count,
                                                     float *out) {
  __shared__ float sw[NPARAM];
  __shared__ __align__(16) __nv_bfloat16 s_tile[256 / 32][32 * NF];
  stage_weights(wbf, sw);
  __syncthreads();
  MmaWeights W;
  W.load(wbf);
  const int lane = threadIdx.x & 31;
  const long long gwarp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long w = gwarp; w * 32 < count; w += nwarps) {
    const long long p = w * 32 + lane;
    float f[NF];
#pragma unroll
    for (int i = 0; i < NF; ++i) f[i] = p < count ? X[p * NF + i] : 0.f;
    const float s = mlp_forward_mma(f, W, sw, s_tile[threadIdx.x >> 5]);
    if (p < count) out[p] = s;
  }
}

extern "C" int pir_sched_score(pirgpu_ctx *ctx, int32_t count, const float *X, float *out_scores) {
  if (!ctx || count < 0 || (count > 0 && (!X || !out_scores))) return ctx ? set_err(ctx, PIR_EINVAL, "bad arguments") : PIR_EINVAL;
  if (count == 0) return PIR_OK;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure_params(ctx))) return r;
  SchedState *s = sched(ctx);
  float *d = nullptr;
  if (cudaMalloc(&d, (size_t)count * (NF + 1) * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "score buffers");
  }
  cudaError_t e = cudaMemcpyAsync(d, X, (size_t)count * NF * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    const int grid = std::max(1, std::min(ctx->num_sms * 8, (count + 255) / 256));
    k_score_batch<<<grid, 256, 0, ctx->stream>>>(s->d_wbf, d, count, d + (size_t)count * NF);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_scores, d + (size_t)count * NF, (size_t)count * sizeof(float), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_err(ctx, e, "pir_sched_score");
  return PIR_OK;
}

extern "C" int pir_sched_params(pirgpu_ctx *ctx, float *params, int32_t count, int32_t set) {
  if (!ctx || !params || count != NPARAM) return ctx ? set_err(ctx, PIR_EINVAL, "the scorer has %d parameters", NPARAM) : PIR_EINVAL;
  PIR_CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure_params(ctx))) return r;
  SchedState *s = sched(ctx);
  if (set) {
    PIR_CK(cudaMemcpyAsync(s->d_param, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(s->d_param, s->d_wbf);
    PIR_CK(cudaGetLastError());
  } else {
    PIR_CK(cudaMemcpyAsync(params, s->d_param, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  }
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}
