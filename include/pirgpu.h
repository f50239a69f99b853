/* pirgpu — C ABI of the GB300 (sm_103a) PIR propagation engine.
 *
 * Drop-in for lala-pc's PIR abstract domain (include/lala/pir.hpp:53-942) over
 * a VStore<Interval<ZLB<int>>>: ternary propagators x = y <op> z plus reified
 * x = (y == z) and x = (y <= z), propagated to a fixpoint over int32 interval
 * bounds.  Plain pointers and sizes only; host buffers are caller-owned, device
 * buffers engine-owned.  One CUDA stream per context; a context is not
 * thread-safe.  Every call returns a pir_status; pir_last_error() gives the
 * message of the last failing call.
 *
 * Variable stores are given as two int32 arrays lb[nvars], ub[nvars].
 * INT32_MIN as lb and INT32_MAX as ub mean "no bound" (pir.hpp:403-404).
 * Propagators are given as four int32 arrays (structure of arrays) op[], x[],
 * y[], z[]: the bytecode_type {Sig op; AVar x, y, z} of pir.hpp:37-47.
 */
#ifndef PIRGPU_H
#define PIRGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opcodes: the Sig values PIR accepts (pir.hpp:270-273). */
enum pir_op {
  PIR_ADD = 0,  /* x = y + z          pir.hpp:758-766 */
  PIR_MUL = 1,  /* x = y * z          pir.hpp:767-779 */
  PIR_TDIV = 2, /* x = y tdiv z       pir.hpp:780-792 */
  PIR_FDIV = 3, /* x = y fdiv z */
  PIR_CDIV = 4, /* x = y cdiv z */
  PIR_EDIV = 5, /* x = y ediv z */
  PIR_MIN = 6,  /* x = min(y, z)      pir.hpp:793-801 */
  PIR_MAX = 7,  /* x = max(y, z)      pir.hpp:802-810 */
  PIR_EQ = 8,   /* x = (y == z)       pir.hpp:730-744 */
  PIR_LEQ = 9   /* x = (y <= z)       pir.hpp:745-757 */
};

typedef enum pir_status {
  PIR_OK = 0,              /* fixpoint reached, store not empty */
  PIR_FAILED = 1,          /* the store is empty (is_bot(), pir.hpp:831-833): a result, not an error */
  PIR_TIMEOUT = 2,         /* opts.max_rounds reached before the fixpoint */
  PIR_BARRIER_TIMEOUT = 3, /* a grid-barrier wait exceeded opts.barrier_timeout_ns */
  PIR_EINVAL = 4,          /* bad argument (var index, opcode, size); nothing was changed */
  PIR_ECUDA = 5,           /* CUDA error */
  PIR_ENOMEM = 6           /* device allocation failed */
} pir_status;

/* Fixpoint drivers. */
enum pir_mode {
  PIR_MODE_AUTO = 0,       /* shared-memory kernel when the instance fits one SM, else persistent */
  PIR_MODE_PERSISTENT = 1, /* one cooperative launch; AC-1 rounds separated by a bounded grid barrier */
  PIR_MODE_HOSTLOOP = 2,   /* one launch per round, the host reads the change flag */
  PIR_MODE_SMEM = 3        /* one CTA, store staged in shared memory (small instances) */
};

/* Propagator schedules. */
enum pir_sched {
  PIR_SCHED_AC1 = 0,      /* every propagator every round (plain AC-1 sweeps) */
  PIR_SCHED_LEARNED = 1,  /* wake set chosen by the trained scorer, certified by a full sweep */
  PIR_SCHED_EVENTS = 2    /* each round runs the propagators of the variables narrowed in the previous
                             round (the first round runs all).  pir_fixpoint: one instance, rounds
                             with at most opts.local_frontier propagators on one CTA, the
                             propagators of narrowed variables with at most 4 propagators run at
                             once by the narrowing thread (opts.chase);
                             pir_fixpoint_nodes: one CTA per node, when the base store is at its
                             fixpoint (else AC-1 rounds); pir_fixpoint_instances: per instance, a
                             round runs the propagators with a variable narrowed in the previous
                             round (per-round bitmaps of the narrowed variables beside the store) */
};

/* Number of persistent-kernel variants (propagators per thread and step x CTAs
 * per SM x pipelined sweep) that pir_autotune chooses from. */
#define PIR_PERSISTENT_VARIANTS 10

typedef struct pir_opts {
  int64_t max_rounds;         /* 0: no cap */
  int64_t barrier_timeout_ns; /* 0: 2 s; bound on every grid-barrier wait */
  int32_t mode;               /* enum pir_mode */
  int32_t block;              /* threads per CTA, 0: tuned default */
  int32_t ctas_per_sm;        /* persistent grid = SMs * ctas_per_sm, 0: occupancy limit */
  int32_t sched;              /* enum pir_sched */
  float wake_fraction;        /* learned schedule: fraction of propagators woken per round (0: 1/16) */
  int32_t variant;            /* persistent kernel variant 1..PIR_PERSISTENT_VARIANTS (0: autotuned, else the default) */
  int32_t local_frontier;     /* event schedule: rounds of at most this many propagators run on one CTA (0: 256) */
  int32_t chase;              /* event schedule: propagators of narrowed small variables a thread runs at once,
                                 per frontier entry (0: 64; at most 256; < 0: none, everything waits for the next
                                 round) */
  int32_t certify;            /* event schedules (pir_fixpoint, pir_fixpoint_nodes, pir_search): 0 or > 0 end the
                                 run with a certifying sweep (pir_fixpoint: every propagator once; a node: every
                                 propagator of a variable the node narrowed that is not entailed at the base
                                 store, whose other propagators see the base store, a fixpoint); a sweep that
                                 narrows something resumes the rounds, so the result is always a fixpoint;
                                 < 0: none */
  int32_t segments;           /* pir_fixpoint's event schedule: 0 or > 0 run the propagators of paths joined by
                                 variables with two occurrences as segments (a warp sweeps up to 64 of them in
                                 shared memory); < 0: every propagator on its own */
  int32_t dense;              /* pir_fixpoint's event schedule: a dense round (every propagator once, AC-1
                                 style, noting only which variables narrowed: one atomic per variable instead
                                 of listing each narrowed variable's propagators) is followed by another while
                                 the propagators of the variables it narrowed number at least 1/dense of all
                                 (0: 1/32) and those variables keep getting fewer; < 0: dense only for the first
                                 round and the certifying sweep */
  int32_t lead;               /* pir_fixpoint's event schedule: AC-1 rounds of the persistent kernel run first, until
                                 a round whose narrowed bounds have not shrunk by an eighth against the round lead
                                 rounds before (0: 8; at most 64): a steady trickle, such as a long chain, goes to
                                 the event kernel, which continues from that store (a lead that reaches the
                                 fixpoint ends the run: its last round narrowed nothing); < 0, or
                                 opts.max_rounds > 0: the event kernel from the start */
} pir_opts;

typedef struct pir_stats {
  int64_t rounds;      /* propagation rounds (AC-1 sweeps), including the final no-change one */
  int64_t executions;  /* propagator executions */
  int64_t narrowed;    /* bounds narrowed (atomic joins that changed the store) */
  float device_ms;     /* device time of the fixpoint (CUDA events on the context stream) */
  int32_t status;      /* pir_status of the run */
  int64_t certify_executions; /* executions of the certifying sweeps (part of executions) */
  int64_t certify_narrowed;   /* bounds the certifying sweeps narrowed: 0 unless the schedule stopped short of
                                 the fixpoint (then the rounds resumed from those narrowings) */
} pir_stats;

typedef struct pirgpu_ctx pirgpu_ctx;
typedef struct pirgpu_snapshot pirgpu_snapshot;

/* Context = one PIR over one VStore on one device (PIR::PIR, pir.hpp:158-163). */
int pir_ctx_create(pirgpu_ctx **out, int device);
void pir_ctx_destroy(pirgpu_ctx *ctx);
const char *pir_last_error(const pirgpu_ctx *ctx);

/* Replaces the variable store (VStore construction / sub-domain tell). */
int pir_load_store(pirgpu_ctx *ctx, int32_t nvars, const int32_t *lb, const int32_t *ub);
/* Copies the store out (operator[] over all variables, pir.hpp:840-842). */
int pir_read_store(pirgpu_ctx *ctx, int32_t *lb, int32_t *ub);
/* operator[](x) / project(x), pir.hpp:840-851. */
int pir_project(pirgpu_ctx *ctx, int32_t var, int32_t *lb, int32_t *ub);
/* embed(x, dom), pir.hpp:354-356: meet [lb, ub] into x; *changed = narrowed. */
int pir_embed(pirgpu_ctx *ctx, int32_t var, int32_t lb, int32_t ub, int *changed);

/* embed() applied to count (var, [lb, ub]) pairs in one call (pir.hpp:354-356
 * repeated); *changed = some bound narrowed. */
int pir_embed_many(pirgpu_ctx *ctx, int32_t count, const int32_t *var, const int32_t *lb,
                   const int32_t *ub, int *changed);

/* deduce(tell) for the bytecode part of a tell, pir.hpp:326-352: appends n
 * propagators, meets x of every EQ/LEQ with [0,1] and re-sorts the whole
 * bytecode by (op, y, x, z) (the CPU order of pir.hpp:343-347).  Var indices
 * must be < nvars and opcodes valid (PIR_EINVAL otherwise, nothing appended).
 * *changed is set to 1 when propagators were added (has_changed). */
int pir_tell(pirgpu_ctx *ctx, int32_t n, const int32_t *op, const int32_t *x, const int32_t *y,
             const int32_t *z, int *changed);
/* num_deductions(), pir.hpp:382-384. */
int64_t pir_num_deductions(const pirgpu_ctx *ctx);
/* vars(), pir.hpp:853-855. */
int32_t pir_vars(const pirgpu_ctx *ctx);
/* The bytecode in engine order (the order deduce(i) and ask(i) index). */
int pir_get_bytecode(pirgpu_ctx *ctx, int32_t *op, int32_t *x, int32_t *y, int32_t *z);

/* Runs propagators to the fixpoint (the driver loop around deduce(i) of
 * tests/pir_test.cpp:60-62).  Returns PIR_OK, PIR_FAILED, PIR_TIMEOUT or an
 * error.  opts may be NULL (defaults); stats may be NULL. */
int pir_fixpoint(pirgpu_ctx *ctx, const pir_opts *opts, pir_stats *stats);
/* Autotuner: times every persistent-kernel variant (propagators per thread
 * and step, CTAs per SM, pipelining) for `rounds` rounds (0: 64; the first
 * rounds of a fixpoint narrow far more than the later ones, so short windows
 * favour the wrong variant) from the current store,
 * keeps the fastest for this context's later pir_fixpoint calls
 * (opts.variant = 0) and puts the store back.  out_variant (1-based) and
 * out_us_per_round may be NULL. */
int pir_autotune(pirgpu_ctx *ctx, int32_t rounds, int32_t *out_variant, float *out_us_per_round);

/* deduce(i), pir.hpp:387-390: one propagator; *changed = has_changed. */
int pir_deduce_one(pirgpu_ctx *ctx, int64_t i, int *changed);

/* ask(i), pir.hpp:368-370 and ask(bytecode), :417-438. */
int pir_ask(pirgpu_ctx *ctx, int64_t i, int *entailed);
/* ask(i) for every i (engine order); out has num_deductions() bytes. */
int pir_ask_all(pirgpu_ctx *ctx, uint8_t *entailed);
/* ask(ask_type) for its bytecode part, pir.hpp:372-380 with :417-438: the
 * entailment of n given propagators (not installed) against the store. */
int pir_ask_bytecodes(pirgpu_ctx *ctx, int32_t n, const int32_t *op, const int32_t *x,
                      const int32_t *y, const int32_t *z, uint8_t *entailed);
/* is_bot(), pir.hpp:831-833. */
int pir_is_bot(pirgpu_ctx *ctx, int *bot);
/* is_top(), pir.hpp:836-838. */
int pir_is_top(pirgpu_ctx *ctx, int *top);
/* is_extractable(), pir.hpp:874-884: not bot and every propagator entailed. */
int pir_is_extractable(pirgpu_ctx *ctx, int *extractable);

/* snapshot() / restore(), pir.hpp:857-870.  restore pops bytecodes from the
 * end of the engine order back to the snapshot's count, as the reference pops
 * from the end of its sorted vector, and restores the store. */
int pir_snapshot(pirgpu_ctx *ctx, pirgpu_snapshot **out);
int pir_restore(pirgpu_ctx *ctx, const pirgpu_snapshot *snap);
void pir_snapshot_free(pirgpu_snapshot *snap);

/* deduce(bytecode) applied to `count` independent private stores: bytecode
 * k is (op[k], 0, 1, 2) over the three intervals in_lb/in_ub[3k..3k+2];
 * results go to out_lb/out_ub, out_changed[k] (0/1) and out_failed[k] (0/1).
 * The batched form of pir.hpp:721-817 for many candidate stores. */
int pir_deduce_batch(pirgpu_ctx *ctx, int64_t count, const int32_t *op, const int32_t *in_lb,
                     const int32_t *in_ub, int32_t *out_lb, int32_t *out_ub, uint8_t *out_changed,
                     uint8_t *out_failed);

/* Batched search nodes: the snapshot / embed / fixpoint / restore loop of
 * tests/bound_consistency_test.hpp:175-196 over many nodes at once.  Node j
 * starts from the context's store, meets its tightenings (var[k], lb[k], ub[k]
 * for k in off[j] .. off[j+1]-1) and runs to its own fixpoint with the
 * context's bytecode (shared by all nodes, as the shared copies of
 * pir.hpp:182-195).  out_lb/out_ub (nnodes * nvars each, may be NULL) receive
 * the node stores; out_status[j] a pir_status; out_rounds[j] (may be NULL) the
 * rounds of node j.  The context's own store is not modified. */
int pir_fixpoint_nodes(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                       const int32_t *lb, const int32_t *ub, const pir_opts *opts,
                       int32_t *out_lb, int32_t *out_ub, int32_t *out_status,
                       int32_t *out_rounds, pir_stats *stats);

/* Number of event node kernel variants (one node per CTA or one per warp x
 * threads per CTA x resident CTAs per SM) that pir_autotune_nodes chooses
 * from; opts.variant of the node calls. */
#define PIR_NODE_VARIANTS 10

/* Autotuner of the batched search nodes (event schedule): runs the batch with
 * every node kernel variant (twice, keeping the faster run) and keeps the
 * fastest for this context's later node calls with opts.variant = 0.  The
 * node results are not returned.  out_variant / out_ms may be NULL. */
int pir_autotune_nodes(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                       const int32_t *lb, const int32_t *ub, int32_t *out_variant, float *out_ms);

/* pir_fixpoint_nodes for a search driver: instead of whole stores, every node
 * reports the final bounds of the `nwatch` variables `watch` (out_wlb/out_wub,
 * nnodes x nwatch, node-major).  Runs the event schedule; the context's store
 * is first brought to its fixpoint when it is not known to be one (node
 * results do not depend on it: a node's fixpoint is that of base + its
 * tightenings).  Replaces reading the decision variables of each child node
 * (pir.hpp:840-851) after its propagation. */
int pir_fixpoint_nodes_watch(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                             const int32_t *lb, const int32_t *ub, const pir_opts *opts, int32_t nwatch,
                             const int32_t *watch, int32_t *out_wlb, int32_t *out_wub, int32_t *out_status,
                             int32_t *out_rounds, pir_stats *stats);

/* Repeated batches of search nodes as CUDA graphs.  A solver that runs its
 * own search loop around the batched nodes (the per-node shared copies of
 * pir.hpp:182-195, the snapshot / embed / fixpoint / restore loop of
 * tests/bound_consistency_test.hpp:175-196) writes each batch into pinned
 * host memory the context owns, and the batch then runs as one CUDA graph
 * (clear the counters, copy in, node kernel, copy out) whose copy sizes and
 * kernel arguments are updated in place from batch to batch; the graph is
 * rebuilt only when a staging buffer has to grow or the kernel variant
 * changes.
 *
 * pir_nodes_stage returns in *in the staging of a batch of nnodes nodes with
 * ntight tightenings in all and nwatch watched variables, as int32:
 * watch[nwatch] | off[nnodes + 1] | var[ntight] | lb[ntight] | ub[ntight]
 * (the arguments of pir_fixpoint_nodes_watch, back to back).  It stays valid
 * until the next pir_nodes_stage call on the context. */
int pir_nodes_stage(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch, int32_t **in);
/* Runs the staged batch (sizes as given to pir_nodes_stage): the event node
 * kernel with its certifying sweeps, as pir_fixpoint_nodes_watch does (the
 * context's store is first brought to its fixpoint when it is not known to be
 * one).  out_status[j], out_rounds[j] (may be NULL) and the watched bounds
 * out_wlb / out_wub (nnodes x nwatch, node-major) as pir_fixpoint_nodes_watch
 * returns them.  The staged input is checked first (offsets, variable
 * indices): PIR_EINVAL runs nothing. */
int pir_fixpoint_nodes_staged(pirgpu_ctx *ctx, int32_t nnodes, int32_t ntight, int32_t nwatch,
                              const pir_opts *opts, int32_t *out_status, int32_t *out_rounds,
                              int32_t *out_wlb, int32_t *out_wub, pir_stats *stats);

/* Branching order of pir_search. */
enum pir_order {
  PIR_ORDER_INPUT = 0,     /* the first decision variable that is not fixed */
  PIR_ORDER_MIN_DOMAIN = 1 /* the unfixed decision variable with the smallest domain (first on ties) */
};

typedef struct pir_search_opts {
  int64_t max_nodes;     /* nodes to propagate, 0: no limit */
  int64_t max_solutions; /* stop after this many solutions (rows of out_solutions); 0: count them all */
  int32_t batch;         /* nodes per launch, 0: 4096 */
  int32_t order;         /* enum pir_order */
  int32_t reserved[6];
} pir_search_opts;

typedef struct pir_search_stats {
  int64_t nodes;      /* nodes propagated, the root included */
  int64_t failures;   /* nodes whose store became empty */
  int64_t solutions;  /* nodes with every decision variable fixed */
  int64_t launches;   /* batched node launches */
  int64_t max_depth;  /* deepest node */
  float device_ms;    /* summed device time of the node launches */
  int32_t status;     /* PIR_OK: space exhausted or max_solutions reached; PIR_TIMEOUT: max_nodes reached */
  int64_t h2d_bytes;  /* bytes copied to the device for the node batches (tightenings, watch list) */
  int64_t d2h_bytes;  /* bytes copied back (per-node status and counters, watched bounds) */
} pir_search_stats;

/* Depth-first search over the decision variables `dec` (ndec of them) from the
 * context's store: a node whose decision variables are all fixed is a solution
 * (its values go to row k of out_solutions, max_solutions x ndec); otherwise
 * the branching variable's interval [l, u] is bisected into [l, m] (explored
 * first) and [m + 1, u], m = l + (u - l) / 2.  Up to opts->batch open nodes
 * are propagated per launch (as pir_fixpoint_nodes_watch does; each batch is
 * written into pinned staging the context owns and runs as one CUDA graph),
 * so with batch > 1 the solutions come in the order of the batches.  The decision variables must
 * determine the others (typically: all variables).  The loop a solver runs
 * around lala-pc's PIR with snapshot / restore (pir.hpp:857-870); the context
 * keeps its store (brought to its fixpoint). */
int pir_search(pirgpu_ctx *ctx, int32_t ndec, const int32_t *dec, const pir_search_opts *opts,
               int32_t *out_solutions, pir_search_stats *stats);

/* Batched independent instances of uneven size, one launch: instance j owns
 * propagators prop_off[j] .. prop_off[j+1]-1 (var indices local to the
 * instance) and variables var_off[j] .. var_off[j+1]-1 of lb/ub, which are
 * updated in place.  Each instance is installed: its propagators are grouped by
 * opcode (stable, the GPU order of pir.hpp:339-341) and its reified targets
 * met with [0, 1] on the device (pir.hpp:333-335).  opts->sched is
 * PIR_SCHED_AC1 (every propagator every round) or PIR_SCHED_EVENTS (after the
 * first round, only the propagators of variables the previous round
 * narrowed; the same fixpoint, fewer executions); PIR_SCHED_LEARNED is
 * rejected with PIR_EINVAL.
 * out_status[j] a pir_status, out_rounds[j] (may be NULL) its rounds,
 * out_device_ms[j] (may be NULL) the device time of that instance's own
 * fixpoint (from the moment a CTA takes it up). */
int pir_fixpoint_instances(pirgpu_ctx *ctx, int32_t ninst, const int64_t *prop_off,
                           const int64_t *var_off, const int32_t *op, const int32_t *x,
                           const int32_t *y, const int32_t *z, int32_t *lb, int32_t *ub,
                           const pir_opts *opts, int32_t *out_status, int32_t *out_rounds,
                           float *out_device_ms, pir_stats *stats);

/* The plain fixpoint for callers that cannot allocate device memory.  No
 * counterpart in the reference: lala-pc's PIR leaves the fixpoint loop and its
 * memory to the caller.  Some callers own all device memory themselves (a
 * solver that gives the engine slices of its own pool, or a search loop on many
 * streams that cannot afford cudaMalloc / cudaFree, which may synchronize the
 * device).  This call takes caller-owned device pointers: the bytecode d_op,
 * d_x, d_y, d_z (n int32 each, already installed, any order) and the store
 * d_store (nvars {lb, ub} int32 pairs, 8-byte aligned), which is updated in
 * place, and allocates nothing: its scratch is a fixed array of about 8.5 KB
 * per device inside the library, which holds it until exit.  The grid is at
 * most 1024 CTAs; opts->ctas_per_sm asking for more (or for more than fit on an
 * SM) is rejected with PIR_EINVAL, as are invalid opcodes or var indices
 * (checked on the device; the store is left untouched).  The first call on a
 * device looks up the scratch address (cudaGetSymbolAddress) and should come
 * before any stream capture.  Calls share the scratch: calls that overlap on
 * the GPU race and must not be issued.  stream may be NULL (default stream);
 * the call waits for the stream (it reads the outcome back) and returns once
 * the fixpoint is done, with the status and stats. */
int pir_fixpoint_static(const int32_t *d_op, const int32_t *d_x, const int32_t *d_y,
                        const int32_t *d_z, int64_t n, int32_t *d_store, int32_t nvars,
                        const pir_opts *opts, pir_stats *stats, void *stream);

/* Learned propagator scheduler (used by pir_fixpoint with opts.sched =
 * PIR_SCHED_LEARNED; no counterpart in the reference, whose fixpoint loop is
 * the caller's).  An 8 -> 32 -> 32 -> 1 MLP with BF16 weights scores
 * propagators on the tensor cores.  When the store was a fixpoint before the
 * last embeddings (a fixpoint returned PIR_OK, or a snapshot taken at one was
 * restored, and only pir_embed / pir_embed_many changed it since), one CTA
 * runs rounds on the frontier of the embedded variables: each round scores
 * its frontier, runs the entries with a logit >= 0 and at least the top
 * opts.wake_fraction of them, and defers the rest; an empty frontier is
 * followed by a certifying round over every propagator of every variable the
 * run embedded or narrowed.  Otherwise (or with opts.local_frontier < 0, or
 * when the frontier outgrows 65,536 entries) every propagator is scored each
 * round on the whole grid, each CTA runs the top opts.wake_fraction of the
 * propagators it scored, and a round of woken propagators without change is
 * followed by a full certifying sweep.  Either way the fixpoint is the plain
 * one bit for bit.
 *
 * pir_sched_collect: change traces of the plain AC-1 fixpoint, node by node
 * (each node = the context's store + its tightenings, as pir_fixpoint_nodes);
 * every positive (a propagator that narrowed a bound in that round) and a
 * keep_negative fraction of the negatives are kept, up to max_samples.  The
 * context's store is left as it was. */
int pir_sched_collect(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *off, const int32_t *var,
                      const int32_t *lb, const int32_t *ub, int64_t max_samples,
                      float keep_negative, int64_t *out_samples, int64_t *out_positives);
/* Trains the scorer on the collected samples with the device kernels
 * (weighted binary cross-entropy, Adam); out_loss[e] = mean loss of epoch e. */
int pir_sched_train(pirgpu_ctx *ctx, int32_t epochs, int32_t batch, float lr, float pos_weight,
                    float *out_loss);
/* Loss and parameter gradient of the current BF16 weights on count samples
 * (X: count x 8 features, Y: labels), for checking the training kernels. */
int pir_sched_grad(pirgpu_ctx *ctx, int32_t count, const float *X, const float *Y, float pos_weight,
                   float *grad_out, float *loss_out);
/* Reads (set = 0) or writes (set = 1) the FP32 master parameters (count must
 * be the parameter count, 1377: W1[32][8], b1[32], W2[32][32], b2[32], W3[32], b3). */
int pir_sched_params(pirgpu_ctx *ctx, float *params, int32_t count, int32_t set);
/* Scores of count feature rows X (count x 8) with the learned fixpoint's
 * inference path: the MLP on the tensor cores (mma, BF16 operands -- the
 * features, the weights and the first hidden layer are rounded to BF16 --
 * FP32 accumulation). */
int pir_sched_score(pirgpu_ctx *ctx, int32_t count, const float *X, float *out_scores);

/* Number of SMs and the library's build string (for reports). */
int pir_device_info(pirgpu_ctx *ctx, int32_t *num_sms, char *name, size_t name_len);

/* ------------------------------------------------------------------ PC ----
 * Tree propagators: lala-pc's PC abstract domain (include/lala/pc.hpp:39-789)
 * with its terms (terms.hpp) and formulas (formula.hpp), over the same store
 * as the PIR propagators of this context.  A propagator is a formula tree;
 * trees are given as a tape of nodes {kind, a, b, c} (four int32 arrays),
 * children before parents: every index a node refers to is smaller than the
 * node's own index.  A propagator is the index of its root formula node.  The
 * pc_* calls run the PC propagators only; pir_fixpoint runs the PIR ones. */
enum pc_kind {
  /* terms: Term's alternatives in order (terms.hpp:572-589) */
  PC_VAR = 0,      /* a = variable                           Variable :48-85 */
  PC_CONST = 1,    /* the interval [a, b]                     Constant :19-45 */
  PC_FORMULA = 2,  /* a = formula node, its truth value 0/1   Formula::project, formula.hpp:1097 */
  PC_NEG = 3,      /* -t, a = t                               Unary<NegOp> :88-102, :122-175 */
  PC_ABS = 4,      /* |t|, a = t                              Unary<AbsOp> :105-119 */
  PC_ADD = 5,      /* a + b (a, b = terms)                    Binary<GroupAdd> :178-207, :334-435 */
  PC_SUB = 6,      /* a - b                                   GroupSub :210-229 */
  PC_MUL = 7,      /* a * b                                   GroupMul<EDIV> :232-262 */
  PC_TDIV = 8,     /* a tdiv b                                GroupDiv :265-299 */
  PC_FDIV = 9, PC_CDIV = 10, PC_EDIV = 11,
  PC_MIN = 12,     /* min(a, b)                               GroupMinMax :302-331 */
  PC_MAX = 13,
  PC_NADD = 14,    /* sum of b operands: the PC_ARG nodes a .. a+b-1   Nary :438-526 */
  PC_NMUL = 15,    /* product of b operands */
  /* formulas: Formula's alternatives in order (formula.hpp:905-920) */
  PC_PVAR = 16,    /* variable a is true (not 0)              VariableLiteral :81-167 */
  PC_NVAR = 17,    /* variable a is false (0) */
  PC_TRUE = 18, PC_FALSE = 19,  /* False :170-204, True :207-239 */
  PC_LEQ = 20,     /* term a <= term b                        Inequality :728-845 */
  PC_GT = 21,      /* term a > term b */
  PC_EQ = 22,      /* term a == term b                        Equality :590-721 */
  PC_NEQ = 23,     /* term a != term b */
  PC_AND = 24,     /* formula a and formula b                 Conjunction :242-308 */
  PC_OR = 25,      /*                                         Disjunction :311-378 */
  PC_EQUIV = 26,   /*                                         Biconditional :381-451 */
  PC_IMPLY = 27,   /*                                         Implication :454-516 */
  PC_XOR = 28,     /*                                         ExclusiveDisjunction :519-587 */
  PC_ARG = 29,     /* operand slot of PC_NADD / PC_NMUL: a = term */
  PC_AE = 30,      /* a formula of the store itself (AbstractElement :14-78): its items are nodes
                      a .. a+b-1; ask = every PC_ASK / PC_ASK_OUT item entailed, nask = every
                      PC_NASK / PC_NASK_OUT item, deduce = meet every PC_TELL item,
                      contradeduce = every PC_NTELL item */
  PC_TELL = 31, PC_NTELL = 32,   /* items {kind, var, lb, ub} (c is ub): meet [lb, ub] into var */
  PC_ASK = 33, PC_NASK = 34,     /* entailed when var's interval is inside [lb, ub] */
  PC_ASK_OUT = 35, PC_NASK_OUT = 36, /* entailed when var's interval misses [lb, ub] (an ask of var != c) */
  PC_NUM_KINDS = 37
};
/* Deepest formula tree accepted (nodes on a root-to-leaf path): bounds the
 * device call stack of the recursive evaluator. */
#define PC_MAX_DEPTH 64

/* PC::deduce(tell) (pc.hpp:625-648): appends nnodes tape nodes (indices in
 * this call's arrays are local to it) and nprops propagators, then stably
 * sorts all propagators by (formula kind, tree length) as the reference does.
 * c[] is the upper bound of an item node and must be 0 elsewhere.  Checks every node (kinds, child order and
 * kinds, variable range, depth <= PC_MAX_DEPTH) first: PIR_EINVAL changes
 * nothing. */
int pc_tell(pirgpu_ctx *ctx, int32_t nnodes, const int32_t *kind, const int32_t *a, const int32_t *b,
            const int32_t *c, int32_t nprops, const int32_t *roots);
/* num_deductions() (pc.hpp:665-667; the sub-store adds none). */
int64_t pc_num_deductions(const pirgpu_ctx *ctx);
/* The propagators' root nodes in engine order (pc_num_deductions entries,
 * indices into the context's whole tape) and the tape itself (pc_tape_size
 * nodes). */
int pc_get_roots(pirgpu_ctx *ctx, int32_t *roots);
int64_t pc_tape_size(const pirgpu_ctx *ctx);
int pc_get_tape(pirgpu_ctx *ctx, int32_t *kind, int32_t *a, int32_t *b, int32_t *c);
/* Fixpoint of all PC propagators in Jacobi rounds, one cooperative launch:
 * every deduction of a round reads the store the round started from, the
 * round's joins are met in at its end, a round with no join or with an empty
 * variable ends the loop.  The result is a deterministic function of the input
 * (PC propagators need not be monotone, formula.hpp:497-503, and then even the
 * reference's Gauss-Seidel result depends on the propagator order; for
 * monotone ones every order reaches this fixpoint).  opts: max_rounds,
 * barrier_timeout_ns, ctas_per_sm, and sched = PIR_SCHED_EVENTS to run in a
 * round only the formulas whose variables the previous round narrowed (the
 * same rounds and result, fewer executions); the other fields are ignored.
 * stats->executions counts propagator executions. */
int pc_fixpoint(pirgpu_ctx *ctx, const pir_opts *opts, pir_stats *stats);
/* deduce(int i) (pc.hpp:671-681): one propagator, engine order.  *changed is
 * the formula's has_changed as the reference computes it. */
int pc_deduce_one(pirgpu_ctx *ctx, int64_t i, int *changed);
/* ask(int i) (pc.hpp:661-663) of one / of every propagator (entailed[i] 0/1). */
int pc_ask(pirgpu_ctx *ctx, int64_t i, int *entailed);
int pc_ask_all(pirgpu_ctx *ctx, uint8_t *entailed);
/* is_extractable() (pc.hpp:727-737): not bot and every PC propagator entailed. */
int pc_is_extractable(pirgpu_ctx *ctx, int *extractable);

#ifdef __cplusplus
}
#endif
#endif
