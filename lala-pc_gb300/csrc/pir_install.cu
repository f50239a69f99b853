// Install on the device: the engine order of the bytecode and the event
// schedules' variable -> propagator adjacency, by a stable LSD radix sort.
//
// lala-pc sorts the bytecode at install (PIR::deduce(tell), pir.hpp:337-348:
// by (op, y, x, z) with std::stable_sort on the CPU; on the GPU the reference
// calls battery::sorti by opcode, :337-341).  The engine keeps the CPU order
// (deduce(i) and ask(i) index it).  A stable sort by (op, y, x, z) is a
// stable sort by (x, z) followed by a stable sort by (op, y): two phases of
// 8-bit LSD passes over 64-bit keys (x << b | z, then op << b | y, with b the
// bits of the largest variable index), the propagator index carried as the
// value.  Each pass: per-tile digit counts, one exclusive scan of the counts
// in digit-major order (tile order within a digit), and a scatter that ranks
// each element among the equal digits before it in its tile (warp matching,
// then the warps in order), so equal keys keep their order: the permutation
// equals std::stable_sort's.
//
// The adjacency (variable -> propagators, in increasing propagator order, x
// before y before z: the arrays of pir_csr.h) is a stable sort of the 3 n
// occurrences (3 p + slot, in that order) by variable.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "pir_engine.h"

namespace pirgpu {
namespace {

constexpr int RS_THREADS = 256, RS_ITEMS = 8, RS_TILE = RS_THREADS * RS_ITEMS, RS_RADIX = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
static_assert(RS_THREADS == RS_RADIX, "one thread per digit");

// Digit counts of each tile, digit-major: hist[d * ntiles + tile].
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long *key, long long n, int shift,
                                                       unsigned *hist, int ntiles) {
  __shared__ unsigned h[RS_RADIX];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const long long base = (long long)blockIdx.x * RS_TILE;
#pragma unroll
  for (int k = 0; k < RS_ITEMS; ++k) {
    const long long i = base + k * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(unsigned)(key[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m counts in place on one CTA of 1024 threads: each thread
// sums a contiguous chunk, the chunk sums are scanned in shared memory, and
// each thread rewrites its chunk.
__global__ void __launch_bounds__(1024) k_rs_scan(unsigned *a, long long m) {
  __shared__ unsigned s[1024];
  const long long per = (m + 1023) / 1024;
  const long long b = (long long)threadIdx.x * per, e = min(m, b + per);
  unsigned sum = 0;
  for (long long i = b; i < e; ++i) sum += a[i];
  s[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const unsigned v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? s[threadIdx.x - 1] : 0u;
  for (long long i = b; i < e; ++i) {
    const unsigned c = a[i];
    a[i] = run;
    run += c;
  }
}

// Scatter of one pass: a tile's elements in order, 256 at a time; an
// element's place is its digit's offset for the tile, plus the equal digits
// earlier in the tile (earlier chunks: the running base; this chunk: earlier
// warps, then earlier lanes of its warp).
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned long long *key_in, const unsigned *val_in,
                                                          unsigned long long *key_out, unsigned *val_out,
                                                          long long n, int shift, const unsigned *offs,
                                                          int ntiles) {
  __shared__ unsigned base[RS_RADIX];
  __shared__ unsigned wcnt[RS_WARPS][RS_RADIX];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  base[tid] = offs[(size_t)tid * ntiles + blockIdx.x];
  const long long tile = (long long)blockIdx.x * RS_TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int k = 0; k < RS_ITEMS; ++k) {
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][tid] = 0u;
    __syncthreads();
    const long long i = tile + (long long)k * RS_THREADS + tid;
    const bool valid = i < n;
    unsigned long long kk = 0ull;
    unsigned vv = 0u, d = RS_RADIX;  // tail lanes form their own group
    if (valid) {
      kk = key_in[i];
      vv = val_in[i];
      d = (unsigned)(kk >> shift) & 255u;
    }
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const unsigned rank = __popc(peers & lt);
    if (valid && rank == 0u) wcnt[warp][d] = (unsigned)__popc(peers);
    __syncthreads();
    if (valid) {
      unsigned pre = 0u;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const unsigned pos = base[d] + pre + rank;
      key_out[pos] = kk;
      val_out[pos] = vv;
    }
    __syncthreads();
    unsigned tot = 0u;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) tot += wcnt[w][tid];
    base[tid] += tot;
    __syncthreads();
  }
}

// Phase 1 keys: x << b | z, values the propagator indices.
__global__ void k_keys_xz(const int *x, const int *z, long long n, int b, unsigned long long *key, unsigned *val) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    key[i] = ((unsigned long long)(unsigned)x[i] << b) | (unsigned)z[i];
    val[i] = (unsigned)i;
  }
}

// Phase 2 keys, in phase-1 order: op << b | y of the propagator each value names.
__global__ void k_keys_opy(const int *op, const int *y, const unsigned *val, long long n, int b,
                           unsigned long long *key) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned p = val[i];
    key[i] = ((unsigned long long)(unsigned)op[p] << b) | (unsigned)y[p];
  }
}

// Occurrences 3 p + slot keyed by their variable, valued by p; counts per variable.
__global__ void k_keys_occ(const int *x, const int *y, const int *z, long long n, unsigned long long *key,
                           unsigned *val, unsigned *cnt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long p = i / 3;
    const int s = (int)(i - 3 * p);
    const int v = s == 0 ? x[p] : (s == 1 ? y[p] : z[p]);
    key[i] = (unsigned long long)(unsigned)v;
    val[i] = (unsigned)p;
    atomicAdd(cnt + v, 1u);
  }
}

// The engine-order SoA (padded with NOP to a multiple of 4) gathered through
// the permutation.
__global__ void k_gather_bytecode(const int *op, const int *x, const int *y, const int *z, const unsigned *perm,
                                  long long n, long long npad, int *dop, int *dx, int *dy, int *dz) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npad;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < n) {
      const unsigned p = perm[i];
      dop[i] = op[p];
      dx[i] = x[p];
      dy[i] = y[p];
      dz[i] = z[p];
    } else {
      dop[i] = OP_NOP;
      dx[i] = dy[i] = dz[i] = 0;
    }
  }
}

__global__ void k_soa_to_aos(const int *op, const int *x, const int *y, const int *z, long long n, int4 *bc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    bc[i] = make_int4(op[i], x[i], y[i], z[i]);
}

__global__ void k_u32_to_i32(const unsigned *a, long long n, int *b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (int)a[i];
}

int bits_for(int nvars) {
  int b = 1;
  while (b < 31 && (1ll << b) < (long long)nvars) ++b;
  return b;
}

int grid_for(const pirgpu_ctx *ctx, long long n) {
  return (int)std::max<long long>(1, std::min<long long>((long long)ctx->num_sms * 8, (n + 255) / 256));
}

// Stable LSD sort of n (key, value) pairs by the low `bits` bits of the key:
// the pairs start in (k[0], v[0]) and end in (k[*which], v[*which]).
int radix_sort(pirgpu_ctx *ctx, unsigned long long *k[2], unsigned *v[2], long long n, int bits, unsigned *hist,
               int *which) {
  const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<ntiles, RS_THREADS, 0, ctx->stream>>>(k[cur], n, shift, hist, ntiles);
    k_rs_scan<<<1, 1024, 0, ctx->stream>>>(hist, (long long)RS_RADIX * ntiles);
    k_rs_scatter<<<ntiles, RS_THREADS, 0, ctx->stream>>>(k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, shift, hist,
                                                         ntiles);
    PIR_CK(cudaGetLastError());
    cur ^= 1;
  }
  *which = cur;
  return PIR_OK;
}

// Scratch of a sort of m pairs: two key and two value buffers, the counts,
// and `extra` bytes for the caller.
struct SortScratch {
  unsigned long long *k[2];
  unsigned *v[2];
  unsigned *hist;
};

int sort_scratch(pirgpu_ctx *ctx, long long m, size_t extra, SortScratch *s, char **extra_ptr) {
  const size_t ntiles = (size_t)((m + RS_TILE - 1) / RS_TILE);
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t kb = al((size_t)m * 8), vb = al((size_t)m * 4), hb = al((size_t)RS_RADIX * ntiles * 4 + 4);
  int r;
  if ((r = ensure(ctx, &ctx->d_install, &ctx->cap_install, 2 * kb + 2 * vb + hb + al(extra)))) return r;
  char *p = (char *)ctx->d_install;
  s->k[0] = (unsigned long long *)p;
  s->k[1] = (unsigned long long *)(p + kb);
  s->v[0] = (unsigned *)(p + 2 * kb);
  s->v[1] = (unsigned *)(p + 2 * kb + vb);
  s->hist = (unsigned *)(p + 2 * kb + 2 * vb);
  *extra_ptr = p + 2 * kb + 2 * vb + hb;
  return PIR_OK;
}

}  // namespace

int device_install(pirgpu_ctx *ctx, long long n, const int *op, const int *x, const int *y, const int *z) {
  const long long npad = std::max<long long>((n + 3) / 4 * 4, 4);
  const size_t bytes = (size_t)npad * sizeof(int);
  int r;
  if ((r = ensure(ctx, (void **)&ctx->d_op, &ctx->cap_op, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_x, &ctx->cap_x, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_y, &ctx->cap_y, bytes))) return r;
  if ((r = ensure(ctx, (void **)&ctx->d_z, &ctx->cap_z, bytes))) return r;
  SortScratch s;
  char *raw = nullptr;
  if ((r = sort_scratch(ctx, n, (size_t)n * 16, &s, &raw))) return r;
  int *rop = (int *)raw, *rx = rop + n, *ry = rx + n, *rz = ry + n;
  PIR_CK(cudaMemcpyAsync(rop, op, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(rx, x, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(ry, y, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  PIR_CK(cudaMemcpyAsync(rz, z, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  const int b = bits_for(ctx->nvars), g = grid_for(ctx, n);
  k_keys_xz<<<g, 256, 0, ctx->stream>>>(rx, rz, n, b, s.k[0], s.v[0]);
  int which = 0;
  if ((r = radix_sort(ctx, s.k, s.v, n, 2 * b, s.hist, &which))) return r;
  if (which) {
    std::swap(s.k[0], s.k[1]);
    std::swap(s.v[0], s.v[1]);
  }
  k_keys_opy<<<g, 256, 0, ctx->stream>>>(rop, ry, s.v[0], n, b, s.k[0]);
  if ((r = radix_sort(ctx, s.k, s.v, n, b + 4, s.hist, &which))) return r;
  k_gather_bytecode<<<grid_for(ctx, npad), 256, 0, ctx->stream>>>(rop, rx, ry, rz, s.v[which], n, npad, ctx->d_op,
                                                                   ctx->d_x, ctx->d_y, ctx->d_z);
  PIR_CK(cudaGetLastError());
  // the host copy of the engine order
  ctx->h_op.resize((size_t)n);
  ctx->h_x.resize((size_t)n);
  ctx->h_y.resize((size_t)n);
  ctx->h_z.resize((size_t)n);
  PIR_CK(cudaMemcpyAsync(ctx->h_op.data(), ctx->d_op, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemcpyAsync(ctx->h_x.data(), ctx->d_x, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemcpyAsync(ctx->h_y.data(), ctx->d_y, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaMemcpyAsync(ctx->h_z.data(), ctx->d_z, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PIR_CK(cudaStreamSynchronize(ctx->stream));
  return PIR_OK;
}

int device_events_graph(pirgpu_ctx *ctx, int4 *bc, int *adj_ptr, int *adj) {
  const long long n = ctx->n;
  const int nv = ctx->nvars;
  const long long m = 3 * n;
  SortScratch s;
  char *cntp = nullptr;
  int r;
  if ((r = sort_scratch(ctx, m, ((size_t)nv + 1) * 4, &s, &cntp))) return r;
  unsigned *cnt = (unsigned *)cntp;
  PIR_CK(cudaMemsetAsync(cnt, 0, ((size_t)nv + 1) * 4, ctx->stream));
  const int g = grid_for(ctx, m);
  k_soa_to_aos<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(ctx->d_op, ctx->d_x, ctx->d_y, ctx->d_z, n, bc);
  k_keys_occ<<<g, 256, 0, ctx->stream>>>(ctx->d_x, ctx->d_y, ctx->d_z, n, s.k[0], s.v[0], cnt);
  int which = 0;
  if ((r = radix_sort(ctx, s.k, s.v, m, bits_for(nv), s.hist, &which))) return r;
  k_u32_to_i32<<<g, 256, 0, ctx->stream>>>(s.v[which], m, adj);
  k_rs_scan<<<1, 1024, 0, ctx->stream>>>(cnt, (long long)nv + 1);
  PIR_CK(cudaMemcpyAsync(adj_ptr, cnt, ((size_t)nv + 1) * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  PIR_CK(cudaGetLastError());
  return PIR_OK;
}

}  // namespace pirgpu
