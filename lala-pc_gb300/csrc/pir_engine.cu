// pirgpu engine: context, single-instance fixpoint kernels and the C ABI of
// include/pirgpu.h for the PIR surface of lala-pc (include/lala/pir.hpp).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "pir_engine.h"
#include "pir_sort.h"

using namespace pirgpu;

// ============================================================== kernels =====

// Persistent AC-1 fixpoint: one cooperative launch, rounds separated by the
// bounded grid barrier.  PPI propagators per thread and step; MINB CTAs of 256
// threads per SM bound the register budget; PIPE selects the software-pipelined
// sweep (next step's gathers in flight while this step computes).  Thread 0 of
// CTA 0 writes the round count.
// LEAD (the event schedule's lead; the ten AC-1 variants are built without
// it): stop, as if the round cap were reached, after a round whose narrowed
// bounds have not shrunk by an eighth against the round `handover` rounds
// before -- a steady trickle, such as a long chain whose links each narrow a
// little round after round, where a dense phase keeps shrinking -- and the
// event schedule goes on from that store.  Each CTA adds its narrowings to
// the round's counter before it arrives at the grid barrier and reads the
// total after it, so every CTA takes the same decision in the same round.
constexpr unsigned BIT_HANDOVER = 1u << 28;
constexpr int HANDOVER_WINDOW = 64;  // the longest window

// Thread 0 of each CTA, around the grid barrier of `round`: adds the CTA's
// narrowings to the round's counter, passes the barrier, reads the total and
// returns the barrier word, with BIT_HANDOVER when the trickle rule holds.
// Out of line: the sweep loop keeps its registers.
static __device__ __noinline__ unsigned barrier_handover(Control *ctl, long long round, int changed, int failed,
                                                         long long timeout_ns, unsigned long long mine,
                                                         unsigned window, unsigned long long *hist) {
  const int slot3 = (int)(round % 3);
  // before the arrival (a release): the total is complete once all CTAs arrived
  if (mine) atomicAdd(&ctl->joins[slot3], mine);
  unsigned w = grid_sync_rot(ctl, gridDim.x, round, changed, failed, timeout_ns);
  if ((w & BIT_CHANGED) && !(w & (BIT_FAILED | BIT_ERROR))) {
    const unsigned long long joins = *(volatile unsigned long long *)&ctl->joins[slot3];
    // round + 2's counter was last read after barrier round - 1, which every CTA has left
    if (blockIdx.x == 0) ctl->joins[(round + 2) % 3] = 0ull;
    const int slot = (int)(round % window);
    const bool flat = round >= window && 8ull * joins > 7ull * hist[slot];
    hist[slot] = joins;
    if (flat) w |= BIT_HANDOVER;
  }
  return w;
}

template <int PPI, int MINB, bool PIPE = false, bool LEAD = false>
__global__ void __launch_bounds__(256, MINB) k_fixpoint_persistent(Bytecode bc, int2 *store, Control *ctl,
                                                                   long long max_rounds, long long timeout_ns,
                                                                   unsigned handover) {
  // per round parity: the CTA's OR of changed (bit 0) / failed (bit 1), and the
  // barrier's decision word; two block barriers per round
  __shared__ unsigned s_bits[2], s_word[2];
  // LEAD: this CTA's narrowings of the round, the grid's of the last rounds
  __shared__ unsigned s_joins[LEAD ? 2 : 1];
  __shared__ unsigned long long s_hist[LEAD ? HANDOVER_WINDOW : 1];
  RedStore st{store};
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = gridDim.x * blockDim.x;
  const int nsteps = steps_of<PPI>(bc);
  unsigned long long narrowed = 0;
  long long round = 0;
  if (threadIdx.x == 0) {
    s_bits[0] = s_bits[1] = 0u;
    if constexpr (LEAD) s_joins[0] = s_joins[1] = 0u;
  }
  __syncthreads();
  for (;;) {
    const int p = (int)(round & 1);
    int changed = 0, failed = 0;
    if (PIPE)
      changed = sweep_pipelined<PPI>(bc, gtid, gstride, nsteps, st, failed);
    else
      for (int c = gtid; c < nsteps; c += gstride) changed += sweep_step<PPI>(bc, c, st, failed);
    narrowed += changed;
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((threadIdx.x & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
    if constexpr (LEAD) {
      const unsigned wsum = __reduce_add_sync(0xFFFFFFFFu, (unsigned)changed);
      if ((threadIdx.x & 31) == 0 && wsum) atomicAdd(&s_joins[p], wsum);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned b = s_bits[p];
      s_bits[p ^ 1] = 0u;
      if constexpr (LEAD) {
        const unsigned long long mine = s_joins[p];
        s_joins[p ^ 1] = 0u;
        s_word[p] = barrier_handover(ctl, round, b & 1u, b & 2u, timeout_ns, mine, handover, s_hist);
      } else {
        s_word[p] = grid_sync_rot(ctl, gridDim.x, round, b & 1u, b & 2u, timeout_ns);
      }
    }
    __syncthreads();
    const unsigned w = s_word[p];
    ++round;
    if ((w & BIT_ERROR) || (w & BIT_FAILED) || !(w & BIT_CHANGED) || (max_rounds > 0 && round >= max_rounds) ||
        (LEAD && (w & BIT_HANDOVER))) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->rounds = round;
        if (w & BIT_FAILED) ctl->failed = 1;
        if ((w & BIT_CHANGED) && !(w & (BIT_FAILED | BIT_ERROR))) ctl->changed[0] = 1;
      }
      break;
    }
  }
  narrowed = warp_sum64(narrowed);
  if ((threadIdx.x & 31) == 0 && narrowed) atomicAdd(&ctl->narrowed, narrowed);
}

// The persistent variants the autotuner chooses from: (propagators per thread
// and step, minimum resident CTAs per SM).
struct PersistentVariant {
  int ppi, minb;
  const void *fn;
};
static const PersistentVariant kPersistent[] = {
    {4, 2, (const void *)k_fixpoint_persistent<4, 2>}, {4, 3, (const void *)k_fixpoint_persistent<4, 3>},
    {2, 3, (const void *)k_fixpoint_persistent<2, 3>}, {2, 4, (const void *)k_fixpoint_persistent<2, 4>},
    {1, 4, (const void *)k_fixpoint_persistent<1, 4>}, {1, 6, (const void *)k_fixpoint_persistent<1, 6>},
    {4, 1, (const void *)k_fixpoint_persistent<4, 1>}, {2, 2, (const void *)k_fixpoint_persistent<2, 2>},
    {1, 3, (const void *)k_fixpoint_persistent<1, 3, true>}, {2, 2, (const void *)k_fixpoint_persistent<2, 2, true>},
};
static const int kNumPersistent = sizeof(kPersistent) / sizeof(kPersistent[0]);
// The event schedule's AC-1 lead: the pipelined one-propagator variant with the handover rule.
static const PersistentVariant kLead = {1, 3, (const void *)k_fixpoint_persistent<1, 3, true, true>};
static_assert(sizeof(kPersistent) / sizeof(kPersistent[0]) == PIR_PERSISTENT_VARIANTS, "variant count");

// One AC-1 round per launch (host-driven loop).  Change flag per round parity.
__global__ void __launch_bounds__(256) k_sweep_round(Bytecode bc, int2 *store, Control *ctl, int parity) {
  RedStore st{store};
  int changed = 0, failed = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < bc.nchunks; c += gridDim.x * blockDim.x)
    changed += sweep_chunk(bc, c, st, failed);
  const unsigned any_ch = __any_sync(0xFFFFFFFFu, changed), any_f = __any_sync(0xFFFFFFFFu, failed);
  const unsigned nar = __reduce_add_sync(0xFFFFFFFFu, (unsigned)changed);
  if ((threadIdx.x & 31) == 0) {
    if (any_ch) atomicOr(&ctl->changed[parity], 1);
    if (any_f) atomicOr(&ctl->failed, 1);
    if (nar) atomicAdd(&ctl->narrowed, (unsigned long long)nar);
  }
}

__global__ void k_clear_flag(Control *ctl, int parity) { ctl->changed[parity] = 0; }

// Single-CTA fixpoint with the store (and the bytecode when it fits) staged in
// shared memory; rounds are separated by __syncthreads.
template <bool BC_SMEM>
__global__ void __launch_bounds__(1024) k_fixpoint_smem(Bytecode bc, int2 *store, int nvars, Control *ctl,
                                                        long long max_rounds) {
  extern __shared__ int4 smem4[];
  int2 *s_store = reinterpret_cast<int2 *>(smem4);
  const int nchunks = bc.nchunks;
  // bytecode region starts 16-byte aligned after the store
  int4 *s_bc = smem4 + ((nvars * 2 + 3) / 4);
  for (int v = threadIdx.x; v < nvars; v += blockDim.x) s_store[v] = store[v];
  Bytecode sb = bc;
  if (BC_SMEM) {
    int4 *sop = s_bc, *sx = s_bc + nchunks, *sy = s_bc + 2 * nchunks, *sz = s_bc + 3 * nchunks;
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
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
  SmemStore st{s_store};
  unsigned long long narrowed = 0;
  long long round = 0;
  int any_failed = 0, any_changed = 0;
  for (;;) {
    int changed = 0, failed = 0;
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
      const int4 o = sb.op[c], X = sb.x[c], Y = sb.y[c], Z = sb.z[c];
      changed += deduce(o.x, X.x, Y.x, Z.x, st, failed);
      changed += deduce(o.y, X.y, Y.y, Z.y, st, failed);
      changed += deduce(o.z, X.z, Y.z, Z.z, st, failed);
      changed += deduce(o.w, X.w, Y.w, Z.w, st, failed);
    }
    narrowed += changed;
    any_changed = __syncthreads_or(changed);
    any_failed = __syncthreads_or(failed);
    ++round;
    if (any_failed || !any_changed || (max_rounds > 0 && round >= max_rounds)) break;
  }
  for (int v = threadIdx.x; v < nvars; v += blockDim.x) store[v] = s_store[v];
  narrowed = warp_sum64(narrowed);
  if ((threadIdx.x & 31) == 0 && narrowed) atomicAdd(&ctl->narrowed, narrowed);
  if (threadIdx.x == 0) {
    ctl->rounds = round;
    if (any_failed) ctl->failed = 1;
    if (any_changed && !any_failed) ctl->changed[0] = 1;
  }
}

// deduce(i): one propagator of the engine order.
__global__ void k_deduce_one(Bytecode bc, long long i, int2 *store, Control *ctl) {
  GlobalStore st{store};
  const int4 o = bc.op[i >> 2], X = bc.x[i >> 2], Y = bc.y[i >> 2], Z = bc.z[i >> 2];
  const int k = (int)(i & 3);
  const int op = k == 0 ? o.x : k == 1 ? o.y : k == 2 ? o.z : o.w;
  const int x = k == 0 ? X.x : k == 1 ? X.y : k == 2 ? X.z : X.w;
  const int y = k == 0 ? Y.x : k == 1 ? Y.y : k == 2 ? Y.z : Y.w;
  const int z = k == 0 ? Z.x : k == 1 ? Z.y : k == 2 ? Z.z : Z.w;
  int failed = 0;
  const int ch = deduce(op, x, y, z, st, failed);
  ctl->changed[0] = ch > 0;
  if (failed) ctl->failed = 1;
  ctl->narrowed += ch;
}

// ask(i) for all i.
__global__ void k_ask_all(const int *op, const int *x, const int *y, const int *z, long long n,
                          const int2 *store, unsigned char *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int2 a = store[x[i]], b = store[y[i]], c = store[z[i]];
    out[i] = ask(op[i], mk(a.x, a.y), mk(b.x, b.y), mk(c.x, c.y)) ? 1 : 0;
  }
}

// Interleave lb[] / ub[] into the int2 store and flag an empty variable.
__global__ void k_pack_store(const int *lb, const int *ub, int nvars, int2 *store, Control *ctl) {
  int bad = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvars; v += gridDim.x * blockDim.x) {
    const int2 t = make_int2(lb[v], ub[v]);
    store[v] = t;
    bad |= is_bot(mk(t.x, t.y));
  }
  if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctl->failed, 1);
}

__global__ void k_unpack_store(const int2 *store, int nvars, int *lb, int *ub) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvars; v += gridDim.x * blockDim.x) {
    const int2 t = store[v];
    lb[v] = t.x;
    ub[v] = t.y;
  }
}

// Meets into the store (embed / install of reified EQ/LEQ targets).
__global__ void k_meet_list(int2 *store, const int *var, const int *lb, const int *ub, int count, Control *ctl) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int v = var[k];
    const int ol = atomicMax(&store[v].x, lb[k]);
    const int ou = atomicMin(&store[v].y, ub[k]);
    const int nl = max(ol, lb[k]), nu = min(ou, ub[k]);
    if (ol < lb[k] || ou > ub[k]) atomicOr(&ctl->changed[0], 1);
    if (is_bot(mk(nl, nu))) atomicOr(&ctl->failed, 1);
  }
}

// Second pass of a meet list: flag a variable left empty by the joins of
// several entries.
__global__ void k_check_list(const int2 *store, const int *var, int count, Control *ctl) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int2 t = store[var[k]];
    if (is_bot(mk(t.x, t.y))) atomicOr(&ctl->failed, 1);
  }
}

// deduce(bytecode) on thread-private stores.
__global__ void k_deduce_batch(long long count, const int *op, const int *in_lb, const int *in_ub, int *out_lb,
                               int *out_ub, unsigned char *out_changed, unsigned char *out_failed) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x) {
    LocalStore st;
    for (int j = 0; j < 3; ++j) st.v[j] = mk(in_lb[3 * k + j], in_ub[3 * k + j]);
    int failed = 0;
    const int ch = deduce(op[k], 0, 1, 2, st, failed);
    for (int j = 0; j < 3; ++j) {
      out_lb[3 * k + j] = st.v[j].l;
      out_ub[3 * k + j] = st.v[j].u;
    }
    out_changed[k] = ch > 0;
    out_failed[k] = failed;
  }
}

// ============================================================ host side =====

namespace pirgpu {

int set_err(pirgpu_ctx *ctx, int code, const char *fmt, ...) {
  if (ctx) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

int cuda_err(pirgpu_ctx *ctx, cudaError_t e, const char *what) {
  return set_err(ctx, PIR_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call) PIR_CK(call)

int ensure(pirgpu_ctx *ctx, void **ptr, size_t *cap, size_t bytes) {
  if (*cap >= bytes && *ptr) return PIR_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  size_t want = std::max<size_t>(bytes, 256);
  if (cudaMalloc(ptr, want) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return set_err(ctx, PIR_ENOMEM, "cudaMalloc(%zu) failed", want);
  }
  *cap = want;
  return PIR_OK;
}

int read_control(pirgpu_ctx *ctx, Control *h) {
  CK(cudaMemcpyAsync(h, ctx->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int reset_control(pirgpu_ctx *ctx) {
  CK(cudaMemsetAsync(ctx->d_ctl, 0, sizeof(Control), ctx->stream));
  return PIR_OK;
}

Bytecode bytecode_view(const pirgpu_ctx *ctx) {
  Bytecode b;
  b.op = reinterpret_cast<const int4 *>(ctx->d_op);
  b.x = reinterpret_cast<const int4 *>(ctx->d_x);
  b.y = reinterpret_cast<const int4 *>(ctx->d_y);
  b.z = reinterpret_cast<const int4 *>(ctx->d_z);
  b.nchunks = (int)((ctx->n + 3) / 4);
  return b;
}

// Uploads the host bytecode (engine order), padded with NOP to a multiple of 4.
int upload_bytecode(pirgpu_ctx *ctx) {
  const size_t npad = (size_t)((ctx->n + 3) / 4) * 4;
  const size_t bytes = std::max<size_t>(npad, 4) * sizeof(int);
  int r;
  if ((r = ensure(ctx, (void **)&ctx->d_op, &ctx->cap_op, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_x, &ctx->cap_x, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_y, &ctx->cap_y, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_z, &ctx->cap_z, bytes))) return r;
  std::vector<int> *arrs[4] = {&ctx->h_op, &ctx->h_x, &ctx->h_y, &ctx->h_z};
  int *dst[4] = {ctx->d_op, ctx->d_x, ctx->d_y, ctx->d_z};
  for (int a = 0; a < 4; ++a) {
    std::vector<int> &v = *arrs[a];
    const size_t n = (size_t)ctx->n;
    v.resize(npad);
    for (size_t i = n; i < npad; ++i) v[i] = (a == 0) ? OP_NOP : 0;
    if (npad) CK(cudaMemcpyAsync(dst[a], v.data(), npad * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    v.resize(n);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int apply_meets(pirgpu_ctx *ctx, const std::vector<int> &var, const std::vector<int> &lb,
                const std::vector<int> &ub, int *changed) {
  const int count = (int)var.size();
  ++ctx->store_version;
  if (changed) *changed = 0;
  if (count == 0) return PIR_OK;
  int r;
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, (size_t)count * 3 * sizeof(int)))) return r;
  int *dv = (int *)ctx->d_scratch, *dl = dv + count, *du = dl + count;
  CK(cudaMemcpyAsync(dv, var.data(), count * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(dl, lb.data(), count * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(du, ub.data(), count * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if ((r = reset_control(ctx))) return r;
  const int grid = std::min(1024, (count + 255) / 256);
  k_meet_list<<<grid, 256, 0, ctx->stream>>>(ctx->d_store, dv, dl, du, count, ctx->d_ctl);
  k_check_list<<<grid, 256, 0, ctx->stream>>>(ctx->d_store, dv, count, ctx->d_ctl);
  CK(cudaGetLastError());
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  if (h.failed) ctx->failed = true;
  if (h.changed[0]) ctx->at_fixpoint = false;
  if (changed) *changed = h.changed[0];
  return PIR_OK;
}

// The persistent AC-1 kernel on the context's store (the autotuned variant
// unless opts.variant names one); window > 0: the lead variant, which stops
// after a round whose narrowings have not shrunk by an eighth against the
// round `window` rounds before.
static int launch_persistent(pirgpu_ctx *ctx, const pir_opts &opts, long long max_rounds, long long timeout,
                             int window) {
  const int block = 256;
  Bytecode bc = bytecode_view(ctx);
  int vi = opts.variant > 0 ? opts.variant - 1 : (ctx->tuned_variant >= 0 ? ctx->tuned_variant : 0);
  if (vi < 0 || vi >= kNumPersistent) return set_err(ctx, PIR_EINVAL, "unknown kernel variant %d", opts.variant);
  const PersistentVariant &pv = window > 0 ? kLead : kPersistent[vi];
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pv.fn, block, 0));
  if (occ < 1) return set_err(ctx, PIR_ECUDA, "persistent kernel does not fit on an SM");
  int per_sm = opts.ctas_per_sm > 0 ? std::min(opts.ctas_per_sm, occ) : occ;
  int grid = ctx->num_sms * per_sm;
  const int nsteps = bc.nchunks * (4 / pv.ppi);
  grid = std::max(1, std::min(grid, (nsteps + block - 1) / block));
  unsigned handover = window > 0 ? (unsigned)std::min(window, HANDOVER_WINDOW) : 0u;
  void *args[] = {&bc, &ctx->d_store, &ctx->d_ctl, (void *)&max_rounds, (void *)&timeout, (void *)&handover};
  CK(cudaLaunchCooperativeKernel(pv.fn, dim3(grid), dim3(block), args, 0, ctx->stream));
  ctx->last_grid = grid;
  if (window <= 0) ctx->last_variant = vi;
  return PIR_OK;
}

int ac1_lead(pirgpu_ctx *ctx, const pir_opts &opts, int window, pir_stats *st, bool *done) {
  int r;
  const long long timeout = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  if ((r = reset_control(ctx))) return r;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if ((r = launch_persistent(ctx, opts, 0, timeout, window))) return r;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  std::memset(st, 0, sizeof(*st));
  CK(cudaEventElapsedTime(&st->device_ms, ctx->ev0, ctx->ev1));
  st->rounds = h.rounds;
  st->executions = h.rounds * ctx->n;
  st->narrowed = (int64_t)h.narrowed;
  st->status = h.status ? h.status : (h.failed ? PIR_FAILED : (h.changed[0] ? PIR_TIMEOUT : PIR_OK));
  // the lead's last round narrowed nothing: every propagator ran on the final store
  if (st->status == PIR_OK) st->certify_executions = ctx->n;
  *done = st->status != PIR_TIMEOUT;
  return PIR_OK;
}

}  // namespace pirgpu

// =============================================================== C ABI ======

extern "C" {

int pir_ctx_create(pirgpu_ctx **out, int device) {
  if (!out) return PIR_EINVAL;
  *out = nullptr;
  pirgpu_ctx *ctx = new pirgpu_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete ctx;
    return PIR_ECUDA;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&ctx->d_ctl, sizeof(Control)) != cudaSuccess || cudaEventCreate(&ctx->ev0) != cudaSuccess ||
      cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    cudaGetLastError();
    pir_ctx_destroy(ctx);
    return PIR_ECUDA;
  }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
  snprintf(ctx->dev_name, sizeof(ctx->dev_name), "%.*s", (int)sizeof(ctx->dev_name) - 1, prop.name);
  *out = ctx;
  return PIR_OK;
}

void pir_ctx_destroy(pirgpu_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  void *ptrs[] = {ctx->d_store, ctx->d_op, ctx->d_x, ctx->d_y, ctx->d_z, ctx->d_ctl, ctx->d_scratch, ctx->d_io,
                  ctx->d_install};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  destroy_batch_state(ctx);
  destroy_sched_state(ctx);
  destroy_pc_state(ctx);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *pir_last_error(const pirgpu_ctx *ctx) { return ctx ? ctx->err : "no context"; }

int pir_load_store(pirgpu_ctx *ctx, int32_t nvars, const int32_t *lb, const int32_t *ub) {
  if (ctx) ++ctx->store_version;
  if (!ctx) return PIR_EINVAL;
  if (nvars < 0 || (nvars > 0 && (!lb || !ub))) return set_err(ctx, PIR_EINVAL, "bad store arguments");
  if (nvars < std::max(ctx->max_var_used, pc_max_var_used(ctx)) + 1)
    return set_err(ctx, PIR_EINVAL, "store smaller than the variables used by the propagators");
  CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure(ctx, (void **)&ctx->d_store, &ctx->cap_store, (size_t)nvars * sizeof(int2)))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_io, &ctx->cap_io, (size_t)nvars * 2 * sizeof(int)))) return r;
  ctx->nvars = nvars;
  ctx->failed = false;
  ctx->at_fixpoint = false;
  if (nvars == 0) return PIR_OK;
  if ((r = reset_control(ctx))) return r;
  CK(cudaMemcpyAsync(ctx->d_io, lb, (size_t)nvars * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_io + nvars, ub, (size_t)nvars * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  const int blocks = std::min(ctx->num_sms * 8, (nvars + 255) / 256);
  k_pack_store<<<blocks, 256, 0, ctx->stream>>>(ctx->d_io, ctx->d_io + nvars, nvars, ctx->d_store, ctx->d_ctl);
  CK(cudaGetLastError());
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  ctx->failed = h.failed != 0;
  return PIR_OK;
}

int pir_read_store(pirgpu_ctx *ctx, int32_t *lb, int32_t *ub) {
  if (!ctx || (ctx->nvars > 0 && (!lb || !ub))) return PIR_EINVAL;
  if (ctx->nvars == 0) return PIR_OK;
  CK(cudaSetDevice(ctx->device));
  const int nvars = ctx->nvars;
  const int blocks = std::min(ctx->num_sms * 8, (nvars + 255) / 256);
  k_unpack_store<<<blocks, 256, 0, ctx->stream>>>(ctx->d_store, nvars, ctx->d_io, ctx->d_io + nvars);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(lb, ctx->d_io, (size_t)nvars * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ub, ctx->d_io + nvars, (size_t)nvars * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int pir_project(pirgpu_ctx *ctx, int32_t var, int32_t *lb, int32_t *ub) {
  if (!ctx || !lb || !ub) return PIR_EINVAL;
  if (var < 0 || var >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "var %d out of range", var);
  CK(cudaSetDevice(ctx->device));
  int2 t;
  CK(cudaMemcpyAsync(&t, ctx->d_store + var, sizeof(int2), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *lb = t.x;
  *ub = t.y;
  return PIR_OK;
}

int pir_embed(pirgpu_ctx *ctx, int32_t var, int32_t lb, int32_t ub, int *changed) {
  if (!ctx) return PIR_EINVAL;
  if (var < 0 || var >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "var %d out of range", var);
  CK(cudaSetDevice(ctx->device));
  std::vector<int> v{var}, l{lb}, u{ub};
  note_embedded(ctx, &var, 1);
  return apply_meets(ctx, v, l, u, changed);
}

int pir_embed_many(pirgpu_ctx *ctx, int32_t count, const int32_t *var, const int32_t *lb, const int32_t *ub,
                   int *changed) {
  if (!ctx) return PIR_EINVAL;
  if (changed) *changed = 0;
  if (count < 0 || (count > 0 && (!var || !lb || !ub))) return set_err(ctx, PIR_EINVAL, "bad arguments");
  for (int32_t k = 0; k < count; ++k)
    if (var[k] < 0 || var[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "var %d out of range", var[k]);
  CK(cudaSetDevice(ctx->device));
  std::vector<int> v(var, var + count), l(lb, lb + count), u(ub, ub + count);
  note_embedded(ctx, var, count);
  return apply_meets(ctx, v, l, u, changed);
}

int pir_tell(pirgpu_ctx *ctx, int32_t n, const int32_t *op, const int32_t *x, const int32_t *y, const int32_t *z,
             int *changed) {
  if (!ctx) return PIR_EINVAL;
  if (changed) *changed = 0;
  if (n < 0 || (n > 0 && (!op || !x || !y || !z))) return set_err(ctx, PIR_EINVAL, "bad bytecode arguments");
  if (n == 0) return PIR_OK;
  if ((long long)ctx->n + n > (long long)INT32_MAX - 8) return set_err(ctx, PIR_EINVAL, "too many propagators");
  int maxv = ctx->max_var_used;
  for (int32_t i = 0; i < n; ++i) {
    if (op[i] < 0 || op[i] >= OP_COUNT) return set_err(ctx, PIR_EINVAL, "bytecode %d: bad opcode %d", i, op[i]);
    if (x[i] < 0 || x[i] >= ctx->nvars || y[i] < 0 || y[i] >= ctx->nvars || z[i] < 0 || z[i] >= ctx->nvars)
      return set_err(ctx, PIR_EINVAL, "bytecode %d: var index out of range [0, %d)", i, ctx->nvars);
    maxv = std::max(maxv, std::max(x[i], std::max(y[i], z[i])));
  }
  CK(cudaSetDevice(ctx->device));
  // pir.hpp:333-335: reified targets are forced to [0, 1].
  std::vector<int> mv, ml, mu;
  for (int32_t i = 0; i < n; ++i)
    if (op[i] == OP_EQ || op[i] == OP_LEQ) {
      mv.push_back(x[i]);
      ml.push_back(0);
      mu.push_back(1);
    }
  int r;
  if ((r = apply_meets(ctx, mv, ml, mu, nullptr))) return r;
  // Append, then stable-sort the whole bytecode by (op, y, x, z) (pir.hpp:343-347).
  const size_t old = (size_t)ctx->n, tot = old + (size_t)n;
  std::vector<int> o2(tot), x2(tot), y2(tot), z2(tot);
  std::copy(ctx->h_op.begin(), ctx->h_op.begin() + old, o2.begin());
  std::copy(ctx->h_x.begin(), ctx->h_x.begin() + old, x2.begin());
  std::copy(ctx->h_y.begin(), ctx->h_y.begin() + old, y2.begin());
  std::copy(ctx->h_z.begin(), ctx->h_z.begin() + old, z2.begin());
  std::copy(op, op + n, o2.begin() + old);
  std::copy(x, x + n, x2.begin() + old);
  std::copy(y, y + n, y2.begin() + old);
  std::copy(z, z + n, z2.begin() + old);
  if ((long long)tot >= DEVICE_INSTALL_MIN) {
    // the stable (op, y, x, z) sort on the device (pir_install.cu)
    if ((r = device_install(ctx, (long long)tot, o2.data(), x2.data(), y2.data(), z2.data()))) return r;
    ctx->n = (long long)tot;
    ctx->max_var_used = maxv;
    ctx->bytecode_version++;
    ctx->at_fixpoint = false;
    if (changed) *changed = 1;
    return PIR_OK;
  }
  // on the host's threads, the permutation std::stable_sort gives (4M propagators: 0.91 s on one core)
  std::vector<int> perm(tot);
  std::iota(perm.begin(), perm.end(), 0);
  const int T = adjacency_threads((long long)tot);
  parallel_stable_sort(perm, [&](int a, int b) {
    if (o2[a] != o2[b]) return o2[a] < o2[b];
    if (y2[a] != y2[b]) return y2[a] < y2[b];
    if (x2[a] != x2[b]) return x2[a] < x2[b];
    return z2[a] < z2[b];
  }, T);
  ctx->h_op.resize(tot);
  ctx->h_x.resize(tot);
  ctx->h_y.resize(tot);
  ctx->h_z.resize(tot);
  run_threads(T, [&](int t) {
    for (size_t i = tot * (size_t)t / (size_t)T; i < tot * (size_t)(t + 1) / (size_t)T; ++i) {
      ctx->h_op[i] = o2[(size_t)perm[i]];
      ctx->h_x[i] = x2[(size_t)perm[i]];
      ctx->h_y[i] = y2[(size_t)perm[i]];
      ctx->h_z[i] = z2[(size_t)perm[i]];
    }
  });
  ctx->n = (long long)tot;
  ctx->max_var_used = maxv;
  ctx->bytecode_version++;
  ctx->at_fixpoint = false;
  if ((r = upload_bytecode(ctx))) return r;
  if (changed) *changed = 1;
  return PIR_OK;
}

int64_t pir_num_deductions(const pirgpu_ctx *ctx) { return ctx ? ctx->n : 0; }
int32_t pir_vars(const pirgpu_ctx *ctx) { return ctx ? ctx->nvars : 0; }

int pir_get_bytecode(pirgpu_ctx *ctx, int32_t *op, int32_t *x, int32_t *y, int32_t *z) {
  if (!ctx) return PIR_EINVAL;
  const size_t n = (size_t)ctx->n;
  if (n && (!op || !x || !y || !z)) return set_err(ctx, PIR_EINVAL, "null output");
  std::copy(ctx->h_op.begin(), ctx->h_op.begin() + n, op);
  std::copy(ctx->h_x.begin(), ctx->h_x.begin() + n, x);
  std::copy(ctx->h_y.begin(), ctx->h_y.begin() + n, y);
  std::copy(ctx->h_z.begin(), ctx->h_z.begin() + n, z);
  return PIR_OK;
}

static int fixpoint_any(pirgpu_ctx *ctx, const pir_opts *opts_in, pir_stats *stats);

int pir_fixpoint(pirgpu_ctx *ctx, const pir_opts *opts_in, pir_stats *stats) {
  const int rc = fixpoint_any(ctx, opts_in, stats);
  if (rc == PIR_OK && ctx && !ctx->failed) note_fixpoint(ctx);
  return rc;
}

static int fixpoint_any(pirgpu_ctx *ctx, const pir_opts *opts_in, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  int r = PIR_OK;
  CK(cudaSetDevice(ctx->device));
  if (ctx->failed) {
    st.status = PIR_FAILED;
    if (stats) *stats = st;
    return PIR_FAILED;
  }
  if (ctx->n == 0) {
    st.status = PIR_OK;
    if (stats) *stats = st;
    return PIR_OK;
  }
  ++ctx->store_version;
  if (opts.sched == PIR_SCHED_LEARNED) return fixpoint_learned(ctx, opts, stats);
  if (opts.sched == PIR_SCHED_EVENTS) return fixpoint_events(ctx, opts, stats);
  const long long max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  const long long timeout = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  Bytecode bc = bytecode_view(ctx);
  int mode = opts.mode;
  const size_t store_bytes = (size_t)ctx->nvars * sizeof(int2);
  const size_t store_pad = (((size_t)ctx->nvars * 2 + 3) / 4) * 16;
  const size_t bc_bytes = (size_t)bc.nchunks * 64;
  const size_t smem_cap = (size_t)ctx->smem_optin;
  if (mode == PIR_MODE_AUTO) {
    // A single CTA wins while one round's work is small next to a grid barrier.
    mode = (store_pad + bc_bytes <= smem_cap && ctx->n <= 65536) ? PIR_MODE_SMEM : PIR_MODE_PERSISTENT;
  }
  if (mode == PIR_MODE_SMEM && store_bytes > smem_cap)
    return set_err(ctx, PIR_EINVAL, "store of %d vars does not fit in shared memory", ctx->nvars);
  if ((r = reset_control(ctx))) return r;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  long long rounds = 0;
  if (mode == PIR_MODE_SMEM) {
    const bool bc_in = store_pad + bc_bytes <= smem_cap;
    const size_t smem = bc_in ? store_pad + bc_bytes : store_pad;
    const int block = opts.block > 0 ? std::min(opts.block, 1024) : 1024;
    if (bc_in) {
      CK(cudaFuncSetAttribute(k_fixpoint_smem<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_fixpoint_smem<true><<<1, block, smem, ctx->stream>>>(bc, ctx->d_store, ctx->nvars, ctx->d_ctl, max_rounds);
    } else {
      CK(cudaFuncSetAttribute(k_fixpoint_smem<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k_fixpoint_smem<false><<<1, block, smem, ctx->stream>>>(bc, ctx->d_store, ctx->nvars, ctx->d_ctl, max_rounds);
    }
    CK(cudaGetLastError());
  } else if (mode == PIR_MODE_PERSISTENT) {
    if ((r = launch_persistent(ctx, opts, max_rounds, timeout, 0))) return r;
  } else if (mode == PIR_MODE_HOSTLOOP) {
    const int block = opts.block > 0 ? opts.block : 256;
    const int grid = std::max(1, std::min(ctx->num_sms * 8, (bc.nchunks + block - 1) / block));
    Control h;
    for (;;) {
      const int parity = (int)(rounds & 1);
      k_clear_flag<<<1, 1, 0, ctx->stream>>>(ctx->d_ctl, parity);
      k_sweep_round<<<grid, block, 0, ctx->stream>>>(bc, ctx->d_store, ctx->d_ctl, parity);
      CK(cudaGetLastError());
      ++rounds;
      CK(cudaMemcpyAsync(&h, ctx->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      if (h.failed || !h.changed[parity] || (max_rounds > 0 && rounds >= max_rounds)) break;
    }
  } else {
    return set_err(ctx, PIR_EINVAL, "unknown mode %d", mode);
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  CK(cudaEventElapsedTime(&st.device_ms, ctx->ev0, ctx->ev1));
  if (mode != PIR_MODE_HOSTLOOP) rounds = h.rounds;
  st.rounds = rounds;
  st.executions = rounds * ctx->n;
  st.narrowed = (int64_t)h.narrowed;
  int status;
  if (h.status) status = h.status;
  else if (h.failed) status = PIR_FAILED;
  else if (mode == PIR_MODE_HOSTLOOP ? (h.changed[(rounds - 1) & 1] != 0) : (h.changed[0] != 0)) status = PIR_TIMEOUT;
  else status = PIR_OK;
  if (status == PIR_FAILED) ctx->failed = true;
  ctx->at_fixpoint = status == PIR_OK;
  st.status = status;
  ctx->last_mode = mode;
  if (stats) *stats = st;
  if (status == PIR_BARRIER_TIMEOUT) set_err(ctx, status, "grid barrier wait exceeded %lld ns", timeout);
  return status;
}

int pir_autotune(pirgpu_ctx *ctx, int32_t rounds, int32_t *out_variant, float *out_us_per_round) {
  if (ctx) ++ctx->store_version;
  if (!ctx) return PIR_EINVAL;
  if (out_variant) *out_variant = 0;
  if (out_us_per_round) *out_us_per_round = 0.f;
  if (ctx->n == 0 || ctx->failed || ctx->nvars == 0) return PIR_OK;
  if (rounds <= 0) rounds = 64;
  CK(cudaSetDevice(ctx->device));
  int2 *saved = nullptr;
  if (cudaMalloc(&saved, (size_t)ctx->nvars * sizeof(int2)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, PIR_ENOMEM, "autotune: no room to save the store");
  }
  const size_t bytes = (size_t)ctx->nvars * sizeof(int2);
  CK(cudaMemcpyAsync(saved, ctx->d_store, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  const bool failed0 = ctx->failed, fix0 = ctx->at_fixpoint;
  int best = -1;
  float best_us = 0.f;
  int rc = PIR_OK;
  for (int v = 0; v < kNumPersistent && rc == PIR_OK; ++v) {
    float us = -1.f;
    for (int rep = 0; rep < 2; ++rep) {
      if (cudaMemcpyAsync(ctx->d_store, saved, bytes, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess) {
        rc = cuda_err(ctx, cudaGetLastError(), "autotune restore");
        break;
      }
      ctx->failed = failed0;
      pir_opts o;
      std::memset(&o, 0, sizeof(o));
      o.mode = PIR_MODE_PERSISTENT;
      o.max_rounds = rounds;
      o.variant = v + 1;
      pir_stats st;
      const int r = pir_fixpoint(ctx, &o, &st);
      if (r != PIR_OK && r != PIR_TIMEOUT && r != PIR_FAILED) {
        rc = r;
        break;
      }
      const float t = st.rounds > 0 ? st.device_ms * 1e3f / (float)st.rounds : 0.f;
      if (us < 0.f || t < us) us = t;
    }
    if (rc == PIR_OK && us >= 0.f && (best < 0 || us < best_us)) {
      best = v;
      best_us = us;
    }
  }
  cudaMemcpyAsync(ctx->d_store, saved, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(saved);
  ctx->failed = failed0;
  ctx->at_fixpoint = fix0;
  if (rc != PIR_OK) return rc;
  ctx->tuned_variant = best;
  ctx->tuned_version = ctx->bytecode_version;
  if (out_variant) *out_variant = best + 1;
  if (out_us_per_round) *out_us_per_round = best_us;
  return PIR_OK;
}

int pir_deduce_one(pirgpu_ctx *ctx, int64_t i, int *changed) {
  if (ctx) ++ctx->store_version;
  if (!ctx) return PIR_EINVAL;
  if (i < 0 || i >= ctx->n) return set_err(ctx, PIR_EINVAL, "deduce(%lld) out of range", (long long)i);
  CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = reset_control(ctx))) return r;
  k_deduce_one<<<1, 1, 0, ctx->stream>>>(bytecode_view(ctx), i, ctx->d_store, ctx->d_ctl);
  CK(cudaGetLastError());
  Control h;
  if ((r = read_control(ctx, &h))) return r;
  if (h.failed) ctx->failed = true;
  if (h.changed[0]) ctx->at_fixpoint = false;
  if (changed) *changed = h.changed[0];
  return PIR_OK;
}

int pir_ask_all(pirgpu_ctx *ctx, uint8_t *entailed) {
  if (!ctx) return PIR_EINVAL;
  if (ctx->n == 0) return PIR_OK;
  if (!entailed) return set_err(ctx, PIR_EINVAL, "null output");
  CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, (size_t)ctx->n))) return r;
  unsigned char *d = (unsigned char *)ctx->d_scratch;
  const int grid = (int)std::min<long long>(ctx->num_sms * 8, (ctx->n + 255) / 256);
  k_ask_all<<<grid, 256, 0, ctx->stream>>>(ctx->d_op, ctx->d_x, ctx->d_y, ctx->d_z, ctx->n, ctx->d_store, d);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(entailed, d, (size_t)ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int pir_ask_bytecodes(pirgpu_ctx *ctx, int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
                      const int32_t *z, uint8_t *entailed) {
  if (!ctx) return PIR_EINVAL;
  if (n < 0 || (n > 0 && (!op || !x || !y || !z || !entailed))) return set_err(ctx, PIR_EINVAL, "bad arguments");
  if (n == 0) return PIR_OK;
  for (int32_t i = 0; i < n; ++i) {
    if (op[i] < 0 || op[i] >= OP_COUNT) return set_err(ctx, PIR_EINVAL, "bytecode %d: bad opcode %d", i, op[i]);
    if (x[i] < 0 || x[i] >= ctx->nvars || y[i] < 0 || y[i] >= ctx->nvars || z[i] < 0 || z[i] >= ctx->nvars)
      return set_err(ctx, PIR_EINVAL, "bytecode %d: var index out of range [0, %d)", i, ctx->nvars);
  }
  CK(cudaSetDevice(ctx->device));
  int r;
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, (size_t)n * 17))) return r;
  int *d = (int *)ctx->d_scratch;
  unsigned char *out = (unsigned char *)(d + 4 * (size_t)n);
  CK(cudaMemcpyAsync(d, op, n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d + n, x, n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d + 2 * (size_t)n, y, n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d + 3 * (size_t)n, z, n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  const int grid = std::min(ctx->num_sms * 8, (n + 255) / 256);
  k_ask_all<<<grid, 256, 0, ctx->stream>>>(d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, n, ctx->d_store, out);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(entailed, out, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int pir_ask(pirgpu_ctx *ctx, int64_t i, int *entailed) {
  if (!ctx || !entailed) return PIR_EINVAL;
  if (i < 0 || i >= ctx->n) return set_err(ctx, PIR_EINVAL, "ask(%lld) out of range", (long long)i);
  std::vector<uint8_t> all((size_t)ctx->n);
  int r = pir_ask_all(ctx, all.data());
  if (r) return r;
  *entailed = all[(size_t)i];
  return PIR_OK;
}

int pir_is_bot(pirgpu_ctx *ctx, int *bot) {
  if (!ctx || !bot) return PIR_EINVAL;
  *bot = ctx->failed ? 1 : 0;
  return PIR_OK;
}

int pir_is_top(pirgpu_ctx *ctx, int *top) {
  if (!ctx || !top) return PIR_EINVAL;
  *top = 0;
  if (ctx->n != 0 || ctx->failed) return PIR_OK;
  std::vector<int32_t> lb((size_t)ctx->nvars), ub((size_t)ctx->nvars);
  int r = pir_read_store(ctx, lb.data(), ub.data());
  if (r) return r;
  for (int v = 0; v < ctx->nvars; ++v)
    if (lb[v] != MINF || ub[v] != INF) return PIR_OK;
  *top = 1;
  return PIR_OK;
}

int pir_is_extractable(pirgpu_ctx *ctx, int *extractable) {
  if (!ctx || !extractable) return PIR_EINVAL;
  *extractable = 0;
  if (ctx->failed) return PIR_OK;
  std::vector<uint8_t> all((size_t)ctx->n);
  int r = pir_ask_all(ctx, all.data());
  if (r) return r;
  for (uint8_t a : all)
    if (!a) return PIR_OK;
  *extractable = 1;
  return PIR_OK;
}

struct pirgpu_snapshot {
  int device;
  long long n;
  long long pc_n;  // PC propagators (PC::snapshot_type::num_props, pc.hpp:47-51)
  int nvars;
  bool failed;
  bool at_fixpoint;
  int2 *d_store;
};

int pir_snapshot(pirgpu_ctx *ctx, pirgpu_snapshot **out) {
  if (!ctx || !out) return PIR_EINVAL;
  CK(cudaSetDevice(ctx->device));
  pirgpu_snapshot *s = new pirgpu_snapshot();
  s->device = ctx->device;
  s->n = ctx->n;
  s->pc_n = pc_count(ctx);
  s->nvars = ctx->nvars;
  s->failed = ctx->failed;
  s->at_fixpoint = ctx->at_fixpoint;
  s->d_store = nullptr;
  if (ctx->nvars > 0) {
    if (cudaMalloc(&s->d_store, (size_t)ctx->nvars * sizeof(int2)) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      return set_err(ctx, PIR_ENOMEM, "snapshot allocation failed");
    }
    CK(cudaMemcpyAsync(s->d_store, ctx->d_store, (size_t)ctx->nvars * sizeof(int2), cudaMemcpyDeviceToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  *out = s;
  return PIR_OK;
}

int pir_restore(pirgpu_ctx *ctx, const pirgpu_snapshot *snap) {
  if (ctx) ++ctx->store_version;
  if (!ctx || !snap) return PIR_EINVAL;
  if (snap->nvars != ctx->nvars) return set_err(ctx, PIR_EINVAL, "snapshot has %d vars, store has %d", snap->nvars, ctx->nvars);
  if (snap->n > ctx->n || snap->pc_n > pc_count(ctx))
    return set_err(ctx, PIR_EINVAL, "snapshot has more propagators than the context");
  CK(cudaSetDevice(ctx->device));
  if (ctx->nvars > 0)
    CK(cudaMemcpyAsync(ctx->d_store, snap->d_store, (size_t)ctx->nvars * sizeof(int2), cudaMemcpyDeviceToDevice,
                       ctx->stream));
  if (snap->n != ctx->n) {
    // pir.hpp:865-868 pops from the end of the (sorted) bytecode vector.
    ctx->n = snap->n;
    ctx->h_op.resize((size_t)ctx->n);
    ctx->h_x.resize((size_t)ctx->n);
    ctx->h_y.resize((size_t)ctx->n);
    ctx->h_z.resize((size_t)ctx->n);
    ctx->bytecode_version++;
    int r = upload_bytecode(ctx);
    if (r) return r;
  }
  if (snap->pc_n != pc_count(ctx)) {
    int r = pc_truncate(ctx, snap->pc_n);
    if (r) return r;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->failed = snap->failed;
  ctx->at_fixpoint = snap->at_fixpoint && snap->n == ctx->n;
  if (ctx->at_fixpoint && !ctx->failed) note_fixpoint(ctx);
  return PIR_OK;
}

void pir_snapshot_free(pirgpu_snapshot *snap) {
  if (!snap) return;
  if (snap->d_store) {
    cudaSetDevice(snap->device);
    cudaFree(snap->d_store);
  }
  delete snap;
}

int pir_deduce_batch(pirgpu_ctx *ctx, int64_t count, const int32_t *op, const int32_t *in_lb, const int32_t *in_ub,
                     int32_t *out_lb, int32_t *out_ub, uint8_t *out_changed, uint8_t *out_failed) {
  if (!ctx || count < 0) return PIR_EINVAL;
  if (count == 0) return PIR_OK;
  if (!op || !in_lb || !in_ub || !out_lb || !out_ub || !out_changed || !out_failed)
    return set_err(ctx, PIR_EINVAL, "null argument");
  for (int64_t k = 0; k < count; ++k)
    if (op[k] < 0 || op[k] >= OP_COUNT) return set_err(ctx, PIR_EINVAL, "bad opcode %d at %lld", op[k], (long long)k);
  CK(cudaSetDevice(ctx->device));
  const size_t bytes = (size_t)count * (4 + 6 * 4 + 6 * 4 + 2);
  int r;
  if ((r = ensure(ctx, &ctx->d_scratch, &ctx->cap_scratch, bytes))) return r;
  char *base = (char *)ctx->d_scratch;
  int *d_op = (int *)base;
  int *d_il = d_op + count, *d_iu = d_il + 3 * count, *d_ol = d_iu + 3 * count, *d_ou = d_ol + 3 * count;
  unsigned char *d_ch = (unsigned char *)(d_ou + 3 * count), *d_f = d_ch + count;
  CK(cudaMemcpyAsync(d_op, op, count * 4, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d_il, in_lb, count * 12, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(d_iu, in_ub, count * 12, cudaMemcpyHostToDevice, ctx->stream));
  const int grid = (int)std::min<long long>(ctx->num_sms * 16, (count + 255) / 256);
  k_deduce_batch<<<grid, 256, 0, ctx->stream>>>(count, d_op, d_il, d_iu, d_ol, d_ou, d_ch, d_f);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out_lb, d_ol, count * 12, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_ub, d_ou, count * 12, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_changed, d_ch, count, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_failed, d_f, count, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int pir_device_info(pirgpu_ctx *ctx, int32_t *num_sms, char *name, size_t name_len) {
  if (!ctx) return PIR_EINVAL;
  if (num_sms) *num_sms = ctx->num_sms;
  if (name && name_len) snprintf(name, name_len, "%s", ctx->dev_name);
  return PIR_OK;
}

}  // extern "C"
