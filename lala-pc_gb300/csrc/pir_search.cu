// Search driver around the batched node kernel: depth-first branch and prune
// over decision variables, the loop a solver runs on top of lala-pc's PIR
// (branch, propagate with deduce, snapshot / restore: pir.hpp:857-870), with
// the children of up to `batch` open nodes propagated in one launch of the
// event node kernel.  Host code: node bookkeeping and branching; every
// propagation runs on the GPU.  A batch's tightenings (the bisections on each
// node's path) are written straight into pinned staging and the batch runs
// as one CUDA graph (clear the counters, copy in, node kernel, copy out),
// updated in place from batch to batch.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "pir_engine.h"

namespace pirgpu {
struct BatchState;
BatchState *batch(pirgpu_ctx *ctx);
int fixpoint_nodes_events(pirgpu_ctx *ctx, BatchState *b, int32_t nnodes, const int32_t *off, const int32_t *var,
                          const int32_t *lb, const int32_t *ub, const pir_opts &opts, int32_t *out_lb,
                          int32_t *out_ub, int32_t *out_status, int32_t *out_rounds, pir_stats *stats,
                          int32_t nwatch, const int32_t *watch, int32_t *out_wlb, int32_t *out_wub);
// Staged batches (pir_batch.cu): pinned inputs filled in place, one graph
// launch per batch, outputs read from pinned memory.
int nodes_stage(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, int32_t **in);
int nodes_run_staged(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, const pir_opts &opts,
                     int32_t *out_status, int32_t *out_rounds, const int2 **wout, pir_stats *stats);
}  // namespace pirgpu

using namespace pirgpu;

extern "C" int pir_fixpoint_nodes_watch(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                                        const int32_t *lb, const int32_t *ub, const pir_opts *opts_in, int32_t nwatch,
                                        const int32_t *watch, int32_t *out_wlb, int32_t *out_wub,
                                        int32_t *out_status, int32_t *out_rounds, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  if (nnodes < 0 || nwatch < 0 || (nnodes > 0 && (!off || !out_status)))
    return set_err(ctx, PIR_EINVAL, "bad arguments");
  if (nwatch > 0 && (!watch || (nnodes > 0 && (!out_wlb || !out_wub))))
    return set_err(ctx, PIR_EINVAL, "watch list without outputs");
  for (int k = 0; k < nwatch; ++k)
    if (watch[k] < 0 || watch[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "watch %d: var out of range", k);
  if (stats) std::memset(stats, 0, sizeof(*stats));
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
  opts.sched = PIR_SCHED_EVENTS;
  int r;
  if (!ctx->failed && ctx->n > 0 && !ctx->at_fixpoint) {
    pir_opts fo;
    std::memset(&fo, 0, sizeof(fo));
    r = pir_fixpoint(ctx, &fo, nullptr);
    if (r != PIR_OK && r != PIR_FAILED) return r;
  }
  if (ctx->failed || ctx->n == 0) {
    // nothing to propagate: a node is the base met with its tightenings
    std::vector<int32_t> blb((size_t)ctx->nvars), bub((size_t)ctx->nvars);
    if ((r = pir_read_store(ctx, blb.data(), bub.data()))) return r;
    for (int j = 0; j < nnodes; ++j) {
      bool f = ctx->failed;
      std::vector<int32_t> nl(blb), nu(bub);
      for (int k = off[j]; k < off[j + 1]; ++k) {
        nl[var[k]] = std::max(nl[var[k]], lb[k]);
        nu[var[k]] = std::min(nu[var[k]], ub[k]);
        f |= nl[var[k]] > nu[var[k]] || nl[var[k]] == INT_MAX || nu[var[k]] == INT_MIN;
      }
      out_status[j] = f ? PIR_FAILED : PIR_OK;
      if (out_rounds) out_rounds[j] = 0;
      for (int k = 0; k < nwatch; ++k) {
        out_wlb[(size_t)j * nwatch + k] = nl[watch[k]];
        out_wub[(size_t)j * nwatch + k] = nu[watch[k]];
      }
    }
    return PIR_OK;
  }
  PIR_CK(cudaSetDevice(ctx->device));
  return fixpoint_nodes_events(ctx, batch(ctx), nnodes, off, var, lb, ub, opts, nullptr, nullptr, out_status,
                               out_rounds, stats, nwatch, watch, out_wlb, out_wub);
}

extern "C" int pir_nodes_stage(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, int32_t **in) {
  if (!ctx || !in) return PIR_EINVAL;
  *in = nullptr;
  if (nnodes < 0 || ntight < 0 || nwatch < 0) return set_err(ctx, PIR_EINVAL, "negative batch size");
  PIR_CK(cudaSetDevice(ctx->device));
  return nodes_stage(ctx, nnodes, ntight, nwatch, in);
}

extern "C" int pir_fixpoint_nodes_staged(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch,
                                         const pir_opts *opts_in, int32_t *out_status, int32_t *out_rounds,
                                         int32_t *out_wlb, int32_t *out_wub, pir_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (nnodes < 0 || ntight < 0 || nwatch < 0) return set_err(ctx, PIR_EINVAL, "negative batch size");
  if (nnodes == 0) return PIR_OK;
  if (!out_status || (nwatch > 0 && (!out_wlb || !out_wub))) return set_err(ctx, PIR_EINVAL, "null output");
  int32_t *in = nullptr;
  int r;
  // the staging the caller wrote (pir_nodes_stage with these sizes returns the same buffer)
  if ((r = pir_nodes_stage(ctx, nnodes, ntight, nwatch, &in))) return r;
  const int32_t *watch = in, *off = in + nwatch, *var = off + nnodes + 1, *lb = var + ntight, *ub = lb + ntight;
  if (off[0] != 0 || off[nnodes] != ntight) return set_err(ctx, PIR_EINVAL, "offsets must run from 0 to ntight");
  for (int j = 0; j < nnodes; ++j)
    if (off[j + 1] < off[j]) return set_err(ctx, PIR_EINVAL, "node %d: offsets decrease", j);
  for (int k = 0; k < ntight; ++k)
    if (var[k] < 0 || var[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "tightening %d: var out of range", k);
  for (int k = 0; k < nwatch; ++k)
    if (watch[k] < 0 || watch[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "watch %d: var out of range", k);
  pir_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  opts.sched = PIR_SCHED_EVENTS;
  if (!ctx->failed && ctx->n > 0 && !ctx->at_fixpoint) {
    pir_opts fo;
    std::memset(&fo, 0, sizeof(fo));
    r = pir_fixpoint(ctx, &fo, nullptr);
    if (r != PIR_OK && r != PIR_FAILED) return r;
  }
  if (ctx->failed || ctx->n == 0)  // nothing to propagate: the plain path
    return pir_fixpoint_nodes_watch(ctx, nnodes, off, var, lb, ub, &opts, nwatch, watch, out_wlb, out_wub,
                                    out_status, out_rounds, stats);
  const int2 *wout = nullptr;
  if ((r = nodes_run_staged(ctx, nnodes, ntight, nwatch, opts, out_status, out_rounds, &wout, stats))) return r;
  for (size_t k = 0; k < (size_t)nnodes * (size_t)nwatch; ++k) {
    out_wlb[k] = wout[k].x;
    out_wub[k] = wout[k].y;
  }
  return PIR_OK;
}

namespace {

// An open node: the parent and the bisection that made it (root: var -1).
struct SearchNode {
  int parent;
  int var;
  int lb, ub;
  int depth;
};

}  // namespace

extern "C" int pir_search(pirgpu_ctx *ctx, int32_t ndec, const int32_t *dec, const pir_search_opts *opts_in,
                          int32_t *out_solutions, pir_search_stats *stats) {
  if (!ctx) return PIR_EINVAL;
  pir_search_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  if (opts_in) opts = *opts_in;
  if (ndec <= 0 || !dec) return set_err(ctx, PIR_EINVAL, "no decision variables");
  for (int k = 0; k < ndec; ++k)
    if (dec[k] < 0 || dec[k] >= ctx->nvars) return set_err(ctx, PIR_EINVAL, "decision %d: var out of range", k);
  if (opts.max_solutions < 0 || opts.max_nodes < 0) return set_err(ctx, PIR_EINVAL, "negative limit");
  if (opts.max_solutions > 0 && !out_solutions) return set_err(ctx, PIR_EINVAL, "no solution buffer");
  if (opts.order != PIR_ORDER_INPUT && opts.order != PIR_ORDER_MIN_DOMAIN)
    return set_err(ctx, PIR_EINVAL, "unknown order %d", opts.order);
  const int bmax = opts.batch > 0 ? opts.batch : 4096;
  pir_search_stats st;
  std::memset(&st, 0, sizeof(st));
  std::vector<SearchNode> pool;
  pool.push_back(SearchNode{-1, -1, 0, 0, 0});
  std::vector<int> open{0};  // depth-first: the next node is open.back()
  std::vector<int32_t> off, tv, tl, tu, status, wlb, wub;
  pir_opts no;
  std::memset(&no, 0, sizeof(no));
  int rc = PIR_OK;
  bool done = false;
  // the base at its fixpoint first; a failed or empty base takes the plain
  // path (every node is the base met with its tightenings)
  if (!ctx->failed && ctx->n > 0 && !ctx->at_fixpoint) {
    rc = pir_fixpoint(ctx, &no, nullptr);
    if (rc != PIR_OK && rc != PIR_FAILED) return rc;
    rc = PIR_OK;
  }
  const bool staged = !ctx->failed && ctx->n > 0;
  pir_opts eo = no;
  eo.sched = PIR_SCHED_EVENTS;
  const int2 *wout = nullptr;
  while (!open.empty() && !done) {
    int64_t take = std::min<int64_t>(bmax, (int64_t)open.size());
    if (opts.max_nodes > 0) take = std::min<int64_t>(take, opts.max_nodes - st.nodes);
    if (take <= 0) {
      st.status = PIR_TIMEOUT;
      break;
    }
    // the batch, leftmost (top of the stack) first, with its tightenings: the bisections on its path
    std::vector<int> ids((size_t)take);
    for (int64_t i = 0; i < take; ++i) ids[(size_t)i] = open[open.size() - 1 - (size_t)i];
    open.resize(open.size() - (size_t)take);
    status.assign((size_t)take, 0);
    pir_stats ns;
    if (staged) {
      // a node's path holds one bisection per level
      int64_t ntight = 0;
      for (int id : ids) ntight += pool[(size_t)id].depth;
      int32_t *in = nullptr;
      if ((rc = nodes_stage(ctx, (int32_t)take, (int32_t)ntight, ndec, &in))) break;
      int32_t *w = in, *o = w + ndec, *v = o + take + 1, *l = v + ntight, *u = l + ntight;
      std::copy(dec, dec + ndec, w);
      int64_t t = 0;
      o[0] = 0;
      for (int64_t i = 0; i < take; ++i) {
        for (int p = ids[(size_t)i]; p >= 0 && pool[(size_t)p].var >= 0; p = pool[(size_t)p].parent, ++t) {
          v[t] = pool[(size_t)p].var;
          l[t] = pool[(size_t)p].lb;
          u[t] = pool[(size_t)p].ub;
        }
        o[i + 1] = (int32_t)t;
      }
      rc = nodes_run_staged(ctx, (int32_t)take, (int32_t)ntight, ndec, eo, status.data(), nullptr, &wout, &ns);
    } else {
      off.assign(1, 0);
      tv.clear();
      tl.clear();
      tu.clear();
      for (int id : ids) {
        for (int p = id; p >= 0 && pool[(size_t)p].var >= 0; p = pool[(size_t)p].parent) {
          tv.push_back(pool[(size_t)p].var);
          tl.push_back(pool[(size_t)p].lb);
          tu.push_back(pool[(size_t)p].ub);
        }
        off.push_back((int32_t)tv.size());
      }
      wlb.assign((size_t)take * ndec, 0);
      wub.assign((size_t)take * ndec, 0);
      rc = pir_fixpoint_nodes_watch(ctx, (int32_t)take, off.data(), tv.data(), tl.data(), tu.data(), &no, ndec, dec,
                                    wlb.data(), wub.data(), status.data(), nullptr, &ns);
    }
    if (rc != PIR_OK) break;
    {
      // the batch's copies: watch list, offsets and tightenings in; counters, per-node status and
      // watched bounds out
      int64_t ntight = 0;
      for (int id : ids) ntight += pool[(size_t)id].depth;
      st.h2d_bytes += 4 * ((int64_t)ndec + take + 1 + 3 * ntight);
      st.d2h_bytes += 64 + 8 * take + 8 * take * (int64_t)ndec;
    }
    // watched bounds of node i, decision k
    auto lo = [&](int64_t i, int k) -> int32_t {
      return staged ? wout[(size_t)i * ndec + k].x : wlb[(size_t)i * ndec + k];
    };
    auto hi = [&](int64_t i, int k) -> int32_t {
      return staged ? wout[(size_t)i * ndec + k].y : wub[(size_t)i * ndec + k];
    };
    st.nodes += take;
    st.launches += 1;
    st.device_ms += ns.device_ms;
    // solutions in left-to-right order; branching variables
    std::vector<int> branch((size_t)take, -1);
    for (int64_t i = 0; i < take && !done; ++i) {
      const SearchNode &nd = pool[(size_t)ids[(size_t)i]];
      st.max_depth = std::max<int64_t>(st.max_depth, nd.depth);
      if (status[(size_t)i] == PIR_FAILED) {
        ++st.failures;
        continue;
      }
      int best = -1;
      long long best_w = LLONG_MAX;
      for (int k = 0; k < ndec; ++k) {
        const int32_t lk = lo(i, k), uk = hi(i, k);
        if (lk >= uk) continue;
        const long long w = (long long)uk - (long long)lk;
        if (opts.order == PIR_ORDER_INPUT) {
          best = k;
          break;
        }
        if (w < best_w) {
          best_w = w;
          best = k;
        }
      }
      if (best < 0) {
        if (opts.max_solutions > 0)
          for (int k = 0; k < ndec; ++k) out_solutions[(size_t)st.solutions * ndec + k] = lo(i, k);
        ++st.solutions;
        if (opts.max_solutions > 0 && st.solutions >= opts.max_solutions) done = true;
        continue;
      }
      branch[(size_t)i] = best;
    }
    if (done) break;
    // children, pushed so that the leftmost node's left child is explored next
    for (int64_t i = take - 1; i >= 0; --i) {
      const int k = branch[(size_t)i];
      if (k < 0) continue;
      const int32_t lk = lo(i, k), hk = hi(i, k);
      const int32_t mid = (int32_t)((long long)lk + ((long long)hk - (long long)lk) / 2);
      const int parent = ids[(size_t)i], depth = pool[(size_t)parent].depth + 1;
      pool.push_back(SearchNode{parent, dec[k], mid + 1, hk, depth});
      open.push_back((int)pool.size() - 1);
      pool.push_back(SearchNode{parent, dec[k], lk, mid, depth});
      open.push_back((int)pool.size() - 1);
    }
  }
  if (rc == PIR_OK && st.status == 0) st.status = PIR_OK;
  if (rc != PIR_OK) st.status = rc;
  if (stats) *stats = st;
  return rc;
}
