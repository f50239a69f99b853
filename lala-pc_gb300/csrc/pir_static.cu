// pir_fixpoint_static: the persistent AC-1 fixpoint for callers that cannot
// allocate device memory.
//
// Some callers of this engine own every byte of device memory themselves: a
// solver that hands the engine slices of its own arena or pool, or a search
// loop running many streams that cannot afford cudaMalloc / cudaFree, which may
// synchronize the whole device and stall the other streams.  This entry point
// takes the bytecode and the store as device pointers the caller owns, and it
// allocates nothing: its only scratch (the grid-barrier control block, two
// timestamps and one counter per CTA) lives in the file-scope array
// g_static_scratch below, which every GPU that loads the library holds until
// the process exits.  The array's device address is looked up once per device
// with cudaGetSymbolAddress on the first call made on that device, so that
// first call should come before any stream capture; after cudaDeviceReset the
// address is stale and the process must not call this entry point again on that
// device.  All calls share the array: it is cleared at the start of each call,
// and calls that overlap on the GPU (from different streams or threads) race on
// it and must not be issued.  Every call waits for its stream to finish (it
// reads the outcome back) before it returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>

#include "pir_engine.h"

namespace pirgpu {
namespace {

// Largest grid the scratch array has slots for.
constexpr int kStaticMaxCtas = 1024;
constexpr int kStaticMaxDevices = 64;

struct StaticScratch {
  Control ctl;                                    // barrier, status, failure / change flags, rounds
  unsigned long long t_start, t_end;              // %globaltimer at kernel start and end
  int bad_input;                                  // set by the validation pass
  int pad[3];
  unsigned long long cta_narrowed[kStaticMaxCtas];  // bounds narrowed, one slot per CTA
};

}  // namespace
}  // namespace pirgpu

// The scratch of pir_fixpoint_static (about 8.5 KB per device).
static __device__ __align__(256) unsigned char g_static_scratch[sizeof(pirgpu::StaticScratch)];

namespace pirgpu {
namespace {

// Device address of g_static_scratch, per device, filled on first use (with
// that device current).  Host threads making their first calls on one device
// at once may both look it up; they store the same address.
std::atomic<StaticScratch *> g_scratch_ptr[kStaticMaxDevices];

int scratch_for_device(int dev, StaticScratch **out) {
  if (dev < 0 || dev >= kStaticMaxDevices) return PIR_EINVAL;
  StaticScratch *p = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    void *q = nullptr;
    if (cudaGetSymbolAddress(&q, g_static_scratch) != cudaSuccess || !q) {
      cudaGetLastError();
      return PIR_ECUDA;
    }
    p = static_cast<StaticScratch *>(q);
    g_scratch_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return PIR_OK;
}

// Rejects opcodes outside the PIR set and var indices outside [0, nvars), and
// flags a store that is already empty.
__global__ void k_static_validate(const int *op, const int *x, const int *y, const int *z, long long n,
                                  const int2 *store, int nvars, StaticScratch *sc) {
  int bad = 0, empty = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int o = op[i], a = x[i], b = y[i], c = z[i];
    bad |= (o < 0) | (o >= OP_COUNT) | (a < 0) | (a >= nvars) | (b < 0) | (b >= nvars) | (c < 0) | (c >= nvars);
  }
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvars; v += stride) {
    const int2 t = store[v];
    empty |= is_bot(mk(t.x, t.y));
  }
  if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(&sc->bad_input, 1);
  if (__any_sync(0xFFFFFFFFu, empty) && (threadIdx.x & 31) == 0) atomicOr(&sc->ctl.failed, 1);
}

// The persistent AC-1 kernel with its control block in the static scratch:
// one propagator per thread and step, scalar loads of the caller's unpadded
// bytecode, rounds separated by the bounded grid barrier.
__global__ void __launch_bounds__(256, 3) k_fixpoint_static(const int *op, const int *x, const int *y,
                                                            const int *z, long long n, int2 *store,
                                                            StaticScratch *sc, long long max_rounds,
                                                            long long timeout_ns) {
  __shared__ unsigned s_bits[2], s_word[2];
  __shared__ unsigned long long s_narrowed;
  if (threadIdx.x == 0) {
    s_narrowed = 0ull;
    s_bits[0] = s_bits[1] = 0u;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->t_start = globaltimer();
  __syncthreads();
  RedStore st{store};
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long gstride = (long long)gridDim.x * blockDim.x;
  unsigned long long narrowed = 0;
  long long round = 0;
  for (;;) {
    int changed = 0, failed = 0;
    for (long long i = gtid; i < n; i += gstride) {
      const int o = __ldg(op + i), a = __ldg(x + i), b = __ldg(y + i), c = __ldg(z + i);
      const Itv ia = st.load(a), ib = st.load(b), ic = st.load(c);
      changed += deduce_loaded(o, a, b, c, ia, ib, ic, st, failed);
    }
    narrowed += changed;
    const int p = (int)(round & 1);
    const unsigned bits = __reduce_or_sync(0xFFFFFFFFu, (changed ? 1u : 0u) | (failed ? 2u : 0u));
    if ((threadIdx.x & 31) == 0 && bits) atomicOr(&s_bits[p], bits);
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned b = s_bits[p];
      s_bits[p ^ 1] = 0u;
      s_word[p] = grid_sync_rot(&sc->ctl, gridDim.x, round, b & 1u, b & 2u, timeout_ns);
    }
    __syncthreads();
    const unsigned w = s_word[p];
    ++round;
    if ((w & BIT_ERROR) || (w & BIT_FAILED) || !(w & BIT_CHANGED) || (max_rounds > 0 && round >= max_rounds)) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->ctl.rounds = round;
        if (w & BIT_FAILED) sc->ctl.failed = 1;
        if ((w & BIT_CHANGED) && !(w & (BIT_FAILED | BIT_ERROR))) sc->ctl.changed[0] = 1;
      }
      break;
    }
  }
  narrowed = warp_sum64(narrowed);
  if ((threadIdx.x & 31) == 0 && narrowed) atomicAdd(&s_narrowed, narrowed);
  __syncthreads();
  if (threadIdx.x == 0) sc->cta_narrowed[blockIdx.x] = s_narrowed;
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->t_end = globaltimer();
}

}  // namespace
}  // namespace pirgpu

using namespace pirgpu;

extern "C" int pir_fixpoint_static(const int32_t *d_op, const int32_t *d_x, const int32_t *d_y, const int32_t *d_z,
                                   int64_t n, int32_t *d_store, int32_t nvars, const pir_opts *opts_in,
                                   pir_stats *stats, void *stream) {
  pir_stats st;
  std::memset(&st, 0, sizeof(st));
  if (stats) *stats = st;
  if (n < 0 || nvars < 0) return PIR_EINVAL;
  if (n > 0 && (!d_op || !d_x || !d_y || !d_z || !d_store || nvars == 0)) return PIR_EINVAL;
  if (nvars > 0 && !d_store) return PIR_EINVAL;
  if (reinterpret_cast<uintptr_t>(d_store) % 8 != 0) return PIR_EINVAL;
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PIR_ECUDA;
  StaticScratch *sc = nullptr;
  int rc = scratch_for_device(dev, &sc);
  if (rc != PIR_OK) return rc;
  int sms = 0, occ = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PIR_ECUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fixpoint_static, 256, 0) != cudaSuccess || occ < 1)
    return PIR_ECUDA;
  // The grid needs one scratch slot per CTA: a request beyond the slots is rejected.
  long long grid = (long long)sms * (opts.ctas_per_sm > 0 ? opts.ctas_per_sm : occ);
  if (opts.ctas_per_sm > 0 && (opts.ctas_per_sm > occ || grid > kStaticMaxCtas)) return PIR_EINVAL;
  if (grid > kStaticMaxCtas) grid = kStaticMaxCtas;
  grid = std::max<long long>(1, std::min<long long>(grid, ((long long)n + 255) / 256));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(sc, 0, sizeof(StaticScratch), s) != cudaSuccess) return PIR_ECUDA;
  int2 *store = reinterpret_cast<int2 *>(d_store);
  const int vgrid =
      (int)std::max<long long>(1, std::min<long long>((long long)sms * 4, (std::max<long long>(n, nvars) + 255) / 256));
  k_static_validate<<<vgrid, 256, 0, s>>>(d_op, d_x, d_y, d_z, n, store, nvars, sc);
  if (cudaGetLastError() != cudaSuccess) return PIR_ECUDA;
  int flags[2] = {0, 0};
  if (cudaMemcpyAsync(&flags[0], &sc->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&flags[1], &sc->ctl.failed, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PIR_ECUDA;
  if (flags[0]) return PIR_EINVAL;
  if (flags[1]) {
    st.status = PIR_FAILED;
    if (stats) *stats = st;
    return PIR_FAILED;
  }
  if (n == 0) {
    if (stats) *stats = st;
    return PIR_OK;
  }
  long long max_rounds = opts.max_rounds > 0 ? opts.max_rounds : 0;
  long long timeout = opts.barrier_timeout_ns > 0 ? opts.barrier_timeout_ns : 2000000000ll;
  long long nn = n;
  void *args[] = {(void *)&d_op, (void *)&d_x, (void *)&d_y, (void *)&d_z, (void *)&nn, (void *)&store,
                  (void *)&sc, (void *)&max_rounds, (void *)&timeout};
  if (cudaLaunchCooperativeKernel((const void *)k_fixpoint_static, dim3((unsigned)grid), dim3(256), args, 0, s) !=
      cudaSuccess) {
    cudaGetLastError();
    return PIR_ECUDA;
  }
  StaticScratch h;
  if (cudaMemcpyAsync(&h, sc, sizeof(StaticScratch), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PIR_ECUDA;
  st.rounds = h.ctl.rounds;
  st.executions = h.ctl.rounds * n;
  for (long long b = 0; b < grid; ++b) st.narrowed += (int64_t)h.cta_narrowed[b];
  st.device_ms = (float)((double)(h.t_end - h.t_start) * 1e-6);
  if (h.ctl.status) st.status = h.ctl.status;
  else if (h.ctl.failed) st.status = PIR_FAILED;
  else if (h.ctl.changed[0]) st.status = PIR_TIMEOUT;
  else st.status = PIR_OK;
  if (stats) *stats = st;
  return st.status;
}
