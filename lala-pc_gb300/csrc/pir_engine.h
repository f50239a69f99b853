// Internal declarations shared by the pirgpu translation units.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pirgpu.h"
#include "pir_kernels.cuh"

namespace pirgpu {
struct BatchState;
struct SchedState;
struct PcState;
}  // namespace pirgpu

// One PIR (bytecode + store) on one device.
struct pirgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int num_sms = 0;
  int smem_optin = 0;
  char dev_name[128] = {0};
  char err[512] = {0};

  // Store: nvars int2 {lb, ub} in HBM.
  int nvars = 0;
  int2 *d_store = nullptr;
  size_t cap_store = 0;
  int *d_io = nullptr;  // 2 * nvars int32 staging for pack / unpack
  size_t cap_io = 0;
  bool failed = false;  // is_bot()
  bool at_fixpoint = false;  // the store is a fixpoint of the bytecode (last pir_fixpoint returned OK)

  // Bytecode in engine order (sorted by op, y, x, z), host copy and device SoA.
  long long n = 0;
  int max_var_used = -1;
  long long bytecode_version = 0;
  long long store_version = 0;  // bumped by every call that may change d_store (caches key on it)
  std::vector<int> h_op, h_x, h_y, h_z;
  int *d_op = nullptr, *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
  size_t cap_op = 0, cap_x = 0, cap_y = 0, cap_z = 0;

  pirgpu::Control *d_ctl = nullptr;
  void *d_scratch = nullptr;
  size_t cap_scratch = 0;
  void *d_install = nullptr;  // scratch of the device install (radix sorts)
  size_t cap_install = 0;
  int last_grid = 0;
  int last_mode = 0;
  int last_variant = 0;
  int tuned_variant = -1;      // autotuned persistent variant (index), -1: none
  long long tuned_version = -1;  // bytecode_version the tuning was made for

  pirgpu::BatchState *batch = nullptr;
  pirgpu::SchedState *sched = nullptr;
  pirgpu::PcState *pc = nullptr;  // PC tree propagators (pir_pc.cu)
};

namespace pirgpu {

int set_err(pirgpu_ctx *ctx, int code, const char *fmt, ...);
int cuda_err(pirgpu_ctx *ctx, cudaError_t e, const char *what);
int ensure(pirgpu_ctx *ctx, void **ptr, size_t *cap, size_t bytes);
int read_control(pirgpu_ctx *ctx, Control *h);
int reset_control(pirgpu_ctx *ctx);
Bytecode bytecode_view(const pirgpu_ctx *ctx);

void destroy_batch_state(pirgpu_ctx *ctx);
void destroy_sched_state(pirgpu_ctx *ctx);
void destroy_pc_state(pirgpu_ctx *ctx);
// PC propagators: largest variable they use, how many there are, and
// restore()'s pop from the end of their engine order
int pc_max_var_used(const pirgpu_ctx *ctx);
long long pc_count(const pirgpu_ctx *ctx);
int pc_truncate(pirgpu_ctx *ctx, long long n);
// The event schedules' view of the context's bytecode (engine order), built
// on the host's threads once per bytecode version (pir_batch.cu): the AoS
// bytecode, the variable -> propagator adjacency (CSR) and, for the
// single-instance event kernel, the path segments with the variable -> unit
// adjacency (pir_segments.h; equal to the propagator adjacency when there are
// no segments).
struct EventsGraph {
  const int4 *bc = nullptr;
  const int *adj_ptr = nullptr, *adj = nullptr;
  int nseg = 0;
  long long seg_nvar = 0;  // local variable slots of all segments
  const int *uptr = nullptr, *uadj = nullptr;
  const int *seg_pptr = nullptr, *seg_code = nullptr, *seg_vptr = nullptr;
  const unsigned *seg_var = nullptr, *in_seg = nullptr;
  const unsigned long long *seg_umask = nullptr;
};
int events_graph(pirgpu_ctx *ctx, EventsGraph *g, bool segments);

// Install on the device (pir_install.cu), for bytecodes of at least
// DEVICE_INSTALL_MIN propagators: device_install sorts the n given
// propagators (host arrays, any order) into the engine order (op, y, x, z),
// stably, and writes the padded device SoA and the host copies h_op .. h_z;
// device_events_graph builds the AoS bytecode and the variable -> propagator
// adjacency of the context's bytecode into the given device arrays.
constexpr long long DEVICE_INSTALL_MIN = 1 << 16;
int device_install(pirgpu_ctx *ctx, long long n, const int *op, const int *x, const int *y, const int *z);
int device_events_graph(pirgpu_ctx *ctx, int4 *bc, int *adj_ptr, int *adj);

int fixpoint_learned(pirgpu_ctx *ctx, const pir_opts &opts, pir_stats *stats);
int fixpoint_events(pirgpu_ctx *ctx, const pir_opts &opts, pir_stats *stats);
// AC-1 rounds of the persistent kernel on the context's store until a round
// whose narrowings have not shrunk by an eighth against the round `window`
// rounds before (at most 64); *done: the run ended (fixpoint, failure or
// error: st->status), else the store is handed on.
int ac1_lead(pirgpu_ctx *ctx, const pir_opts &opts, int window, pir_stats *st, bool *done);
// Records variables embedded since the last learned fixpoint (its "just
// changed" feature).
void note_embedded(pirgpu_ctx *ctx, const int32_t *var, int count);
// Records that the store is a fixpoint of the current bytecode (a fixpoint
// returned PIR_OK, or a snapshot taken at one was restored): the learned
// schedule then starts from the variables embedded after it.
void note_fixpoint(pirgpu_ctx *ctx);

}  // namespace pirgpu

#define PIR_CK(call)                                                     \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return pirgpu::cuda_err(ctx, _e, #call);      \
  } while (0)
