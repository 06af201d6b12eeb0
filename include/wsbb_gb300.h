/*
 * wsbb_gb300 — C-ABI of the GB300 (sm_103a) flowshop branch-and-bound hot
 * path: batched begin-end child generation, LB2 Johnson two-machine bounds
 * over all machine pairs, prune and compaction, and the exact DFS search
 * built on them.
 *
 * Plain pointers and sizes only. Return codes: 0 = ok, negative = error
 * (wsbb_last_error() describes the last failure on a context). The caller
 * owns every buffer it passes; a context owns its device tables and its
 * search pools. One context per host thread; calls on a context are
 * stream-ordered on the stream they are given, unless documented as
 * synchronous. NULL means the legacy default stream (PyTorch's default
 * stream): calls that run on the library's own stream instead (the
 * searches, training) first wait for the work already queued there.
 *
 * Reference interfaces each entry point replaces (vttuan/WSBB paths):
 *   wsbb_ctx_create     bound_abstract::set_instance -> bound_flowshop::init
 *                       (src/bound_flowshop.cpp:911-927, 953-956) and
 *                       gpu::init / init_bound (src/gpu.cu:126-162,
 *                       src/bound_flowshop_gpu.cu:398-433)
 *   wsbb_lb2_eval       Evaluate_ON_GPU (src/bound_flowshop_gpu.cu:619-674)
 *                       and bound_abstract::bornes_calculer
 *                       (headers/bound_abstract.h:9-19,
 *                       src/bound_flowshop.cpp:929-951)
 *   wsbb_lb2_eval_host  gpu::decompose_on_cpu's H2D -> kernel -> D2H round
 *                       trip (src/gpu.cu:211-234) for a caller-built pool
 *   wsbb_explore        explorer::_explore_cpu / _explore_cpu_gpu
 *                       (src/explorer.cu:92-148, 154-305) with
 *                       decompose_beginend (src/decompose_beginend.cpp:26-107),
 *                       gpu::prune (src/gpu.cu:257-408) and tree::take/insert
 *                       (src/tree.cpp:257-304)
 */
#ifndef WSBB_GB300_H
#define WSBB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WSBB_OK 0
#define WSBB_ERR_ARG (-1)      /* bad argument or unsupported size */
#define WSBB_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define WSBB_ERR_NOMEM (-3)    /* device or host allocation failed */
#define WSBB_ERR_RANGE (-4)    /* processing times outside the table limits */
#define WSBB_ERR_WATCHDOG (-5) /* a bounded device-side wait gave up */
#define WSBB_ERR_CAPACITY (-6) /* search pool capacity exceeded */

#define WSBB_MAX_JOBS 128     /* n <= 128 */
#define WSBB_MAX_MACHINES 32  /* 2 <= m <= 32 */

typedef struct wsbb_ctx wsbb_ctx;

/*
 * Node record (the pool format on the boundary; replaces the ~196-byte
 * raw_bb_problem of the reference's missing bb_problem_calculator.h):
 *
 *   int16 job[n]    the permutation; job[0..limite1] is the front
 *                   sequence, job[limite2..n-1] the back sequence
 *   int16 limite1   last front position (-1: none)
 *   int16 limite2   first back position (n: none); limite2 - limite1 == 1
 *                   marks a leaf (complete permutation)
 *   int16 depth     jobs fixed (informative; the bound does not read it)
 *   int16 reserved
 *   padding to wsbb_node_stride(n) bytes (a multiple of 16)
 */
size_t wsbb_node_stride(int n);

/* Precompute the bound tables for an instance and upload them to `device`.
 * p_mxn[k*n + j] = processing time of job j on machine k (the reference's
 * machine-major stream order, src/instance_flowshop.cpp:88). Requires
 * 2 <= n <= 128, 2 <= m <= 32, 0 <= p <= 65535 and, for every job and
 * machine pair (m1, m2), p[m1] + lag + p[m2] <= 65535 (lag: the sum of p
 * strictly between the two machines). */
int wsbb_ctx_create(const int32_t *p_mxn, int n, int m, int device,
                    wsbb_ctx **out);
void wsbb_ctx_destroy(wsbb_ctx *ctx);
const char *wsbb_last_error(const wsbb_ctx *ctx);
/* Bytes of bound tables wsbb_ctx_create copied host -> device. */
size_t wsbb_ctx_device_bytes(const wsbb_ctx *ctx);

/* Copies of the host-side precompute (for inspection and tests): pair
 * machines (P each), lags and Johnson orders (P x n), static heads and
 * tails (m). Any pointer may be NULL. */
int wsbb_ctx_tables(const wsbb_ctx *ctx, int32_t *mach0, int32_t *mach1,
                    int32_t *lag_pxn, int32_t *johnson_pxn, int32_t *heads,
                    int32_t *tails);

/* Host-only form of the same precompute (no device, no context): fills
 * the same arrays wsbb_ctx_tables returns. */
int wsbb_precompute(const int32_t *p_mxn, int n, int m, int32_t *mach0,
                    int32_t *mach1, int32_t *lag_pxn, int32_t *johnson_pxn,
                    int32_t *heads, int32_t *tails);

/* Pool bounds on device memory, asynchronous on `stream`:
 *   lb_out[i] = LB2 of record i (bornes_calculer with best = 999999), or
 *   the makespan of its permutation when limite2 - limite1 == 1.
 * `recs` holds `count` records of wsbb_node_stride(n) bytes, 16-byte
 * aligned. */
int wsbb_lb2_eval(wsbb_ctx *ctx, const void *recs, int64_t count,
                  int32_t *lb_out, void *stream);
/* One-machine bound LB1 = max_k(head_k + remaining work on k + tail_k),
 * with LB2's head / tail conventions (leaf: makespan). */
int wsbb_lb1_eval(wsbb_ctx *ctx, const void *recs, int64_t count,
                  int32_t *lb_out, void *stream);
/* Makespan of each record's full permutation (cursors ignored). */
int wsbb_makespan_eval(wsbb_ctx *ctx, const void *recs, int64_t count,
                       int32_t *out, void *stream);

/* Branch and bound a batch of fathers, asynchronous on `stream`: both sides
 * of every father (decompose_beginend::operator(),
 * src/decompose_beginend.cpp:91-107, bounding each child with
 * bornes_calculer, src/bound_flowshop.cpp:929-951). Father f's children
 * are child_off[f] .. child_off[f+1]-1 (device int64, count + 1 entries):
 * its u BEGIN children (the job at free position l1+1+k moved to l1+1),
 * then its u END children (moved to l2-1); a father with two free jobs has
 * two leaf children (both orders; their makespans). child_lb gets each
 * child's LB2 (bit-exact to bounding the child record with wsbb_lb2_eval),
 * child_job the job it moved. The children share one pass over each
 * pair's Johnson order of the father's free jobs (max-plus prefix and
 * suffix products), so no child record is materialised. */
int wsbb_decompose_lb2(wsbb_ctx *ctx, const void *fathers, int64_t count,
                       const int64_t *child_off, int32_t *child_lb,
                       int16_t *child_job, void *stream);

/* Synchronous host-buffer form of wsbb_lb2_eval: copies the records to the
 * device, bounds them and copies the bounds back before returning. */
int wsbb_lb2_eval_host(wsbb_ctx *ctx, const void *host_recs, int64_t count,
                       int32_t *host_lb_out);

/*
 * Exact begin-end DFS search on the GPU.
 *
 * Same semantics as the reference CPU search (src/explorer.cu:92-148):
 * the smallest rank path is taken first; leaves update the incumbent when
 * strictly better; a node whose bound is not below the incumbent is pruned;
 * otherwise its 2u children are bounded, the side is chosen with
 * threshold `best` (decompose_beginend::choise) and the chosen side is
 * ranked by (bound, job). Counters, optimum and optimal permutation equal
 * the sequential search's exactly. The search state stays on the device;
 * iterations are replayed from a CUDA graph.
 */
#define WSBB_EXPLORE_NO_GRAPH 1  /* launch iterations one by one */
#define WSBB_EXPLORE_CHILD_LB2 2 /* bound each child record on its own (the
                                    per-node LB2 kernel) instead of each
                                    father's children together; same bounds */
#define WSBB_EXPLORE_RESUME 4    /* continue the context's stopped (or seeded)
                                    search — its stack, incumbent and
                                    counters — instead of starting at the
                                    root; cfg->ub0 may lower the incumbent
                                    (a cost found elsewhere), and window and
                                    capacity must be those of the stopped
                                    search */

typedef struct {
	int32_t ub0;         /* initial incumbent cost (INT32_MAX: none) */
	int32_t best;        /* choise threshold (the reference default is 99999) */
	int32_t window;      /* largest number of nodes branched per iteration
	                        (0: 16384); the search widens up to it */
	int32_t graph_iters; /* iterations per graph launch (0: 16) */
	int64_t capacity;    /* stack capacity in nodes (0: max(2^22, 2 window n^2),
	                        within half the free device memory); at least
	                        16 window + 8192 */
	int64_t max_iters;   /* stop after this many iterations (0: none) */
	int32_t flags;       /* WSBB_EXPLORE_* */
	int32_t family_smem_kb; /* form of the family bounds (a tile shape the
	                           autotuner picks): 0 stages the instance's whole
	                           packed Johnson table in shared memory when it
	                           fits (times <= 127, m <= 20; else 56 applies);
	                           > 0 bounds pairs in chunks whose rows take
	                           this many KB of shared memory per CTA, which
	                           also sets how many CTAs share an SM */
	int64_t max_bounded; /* stop once this many tree nodes are bounded,
	                        checked between graph launches (0: no limit);
	                        the search commits in DFS order, so a budget is
	                        the same tree prefix whatever the window */
} wsbb_explore_cfg;

typedef struct {
	int64_t branched;   /* decomposed nodes (the reference's cpu_explored_nodes) */
	int64_t pruned;     /* taken and pruned (boundedNodesDontExplore) */
	int64_t leaves;     /* leaves taken */
	int64_t improved;   /* incumbent improvements */
	int64_t bounded;    /* child bounds of the search tree */
	int64_t evaluated;  /* child bounds computed, including speculation */
	int64_t discarded;  /* speculative entries dropped after improvements */
	int64_t iterations;
	int32_t best_cost;  /* final incumbent (INT32_MAX if none) */
	int32_t status;     /* 0 complete, 1 iteration cap, <0 error */
	uint64_t depth_hist[WSBB_MAX_JOBS + 1]; /* pruned + leaves per depth */
	int32_t best_perm[WSBB_MAX_JOBS];       /* incumbent permutation */
	double seconds;     /* device time of the search */
	int64_t scanned;    /* stack entries scanned to select fathers */
	int64_t committed;  /* stack entries committed */
	int64_t early;      /* children settled by the learned K-pair test */
	int64_t settled_fathers; /* fathers whose children the K-pair test settled
	                            all (family bounds) */
	int64_t d2h_bytes;  /* bytes the search copied device -> host (its state
	                       between graph launches, the incumbent) */
	/* Exact prefix of a stopped search. Children whose bound the incumbent
	 * already reaches when they are generated are counted (pruned,
	 * depth_hist) when their father is, but the sequential search takes
	 * them after the subtrees of their open siblings. `pending` of them are
	 * still ahead of the sequential search where this one stopped
	 * (pending_hist: by their depth), so the sequential search's counters
	 * after exactly `takes` takes (nodes popped: branched + pruned + leaves
	 * - pending) are these counters with pruned - pending and depth_hist -
	 * pending_hist. Both are 0 once the search completes. The accounting
	 * runs for searches that may stop early — started with max_iters or
	 * max_bounded, or seeded; a search started without either runs to its
	 * end and reports pending = 0. */
	int64_t takes;
	int64_t pending;
	uint32_t pending_hist[WSBB_MAX_JOBS + 1];
} wsbb_stats;

int wsbb_explore(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, wsbb_stats *stats,
                 void *stream);

/*
 * The search of one or many instances in one launch of resident CTAs
 * (replaces the reference's host-driven pipeline, explorer::_explore_cpu_gpu
 * with gpu::decompose_on_cpu / gpu::prune, src/explorer.cu:154-305,
 * src/gpu.cu:180-408, and its peers' work stealing between processes,
 * src/work_stealing/node.cpp:154-162, by stealing between CTAs).
 *
 * One cooperative launch: each instance gets a group of CTAs that runs its
 * iterations (the same phases as wsbb_explore, met at group barriers); in
 * the bound phase each CTA of a group owns a share of the fathers and
 * steals from its group's other shares when its own is empty, and CTAs
 * whose instance has finished steal fathers from the instances still
 * running. Same counters and trees as wsbb_explore with the same cfg
 * (window, capacity, best, ub0, max_iters, max_bounded apply per instance;
 * no WSBB_EXPLORE_RESUME, no WSBB_EXPLORE_CHILD_LB2). Instances must be on
 * one device, fit the staged family bounds (times <= 127, m <= 20) and
 * number at most the resident CTAs (the SM count). Each instance's
 * iterations run on a group of CTAs, an equal share of the grid (at most
 * opts->group_ctas when it is above 0); the CTAs left over, and those of
 * instances that have ended, take fathers from the bound phases of the
 * instances still running. Every wait between CTAs gives up after opts->wait_ms (0:
 * 2000 ms): the launch then ends with WSBB_ERR_WATCHDOG and the contexts
 * stay usable. opts->self_test = 1 makes the first wait also wait for a
 * flag that nothing sets, so that the watchdog must run out (a test of that
 * path). opts may be NULL. stats[k]: instance k; `seconds` is the launch's
 * time.
 */
typedef struct {
	int32_t wait_ms;
	int32_t self_test;
	int32_t group_ctas;
} wsbb_resident_opts;
#define WSBB_EXPLORE_RESIDENT 8 /* wsbb_explore: run as the resident search */
int wsbb_explore_resident(wsbb_ctx *const *ctxs, int count, const wsbb_explore_cfg *cfgs,
                          const wsbb_resident_opts *opts, wsbb_stats *stats, void *stream);

/*
 * Work hand-off between searches (the reference's peers hand each other
 * node lists, BB_PROBLEM_PACKET, src/work_stealing/node.cpp:524-560 and
 * 1240-1283).
 *
 * wsbb_explore_export takes up to max_count open nodes from the bottom of
 * the context's stopped search — the shallowest ones, whose subtrees the
 * search would take last — out of that search and copies their records and
 * bounds to host memory in stack order (bottom first); *count_out receives
 * how many. Open nodes the incumbent already prunes are not taken.
 *
 * wsbb_explore_seed replaces the context's search state by one whose stack
 * holds `count` given open nodes (host records of wsbb_node_stride(n) bytes,
 * recs[0] at the bottom and the last one taken first, with their bounds),
 * incumbent cfg->ub0 and zero counters; wsbb_explore with
 * WSBB_EXPLORE_RESUME (and the same window and capacity) runs it. Records
 * that are not open nodes of this instance are rejected.
 *
 * A peer's counters cover the subtrees it explored; they add up across
 * peers to the whole tree's as long as no node was exported from under a
 * branched node that the incumbent later prunes (such a node's subtree is
 * counted as pruned where it was branched).
 */
int wsbb_explore_export(wsbb_ctx *ctx, int64_t max_count, void *recs_out, int32_t *lbs_out,
                        int64_t *count_out, void *stream);
int wsbb_explore_seed(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, const void *recs,
                      const int32_t *lbs, int64_t count, void *stream);

/*
 * The same search for callers that cannot allocate GPU memory — code that
 * runs under a memory budget fixed at start-up, inside a host callback or
 * allocator hook where cudaMalloc may not be called, or on a path where an
 * allocation failure mid-run is not acceptable. No counterpart in the
 * reference.
 *
 * It makes no allocation of its own (no cudaMalloc / cudaFree, no events,
 * no graph): the whole search state lives in one fixed device array of
 * WSBB_NOALLOC_SCRATCH_BYTES that the library defines at file scope, and
 * which every GPU that loads the library holds until the process exits.
 * The context must exist already (wsbb_ctx_create allocates the instance
 * tables). Limits: the stack capacity and window are derived from the
 * fixed size — cfg->window 0 means the widest of 1024, 512, ..., 64 that
 * leaves the stack room for 8 iterations of that many fathers (n = 20:
 * window 1024, about 397k stack nodes; n = 50: 256, about 178k; n = 100:
 * 64, about 99k), cfg->capacity 0 means as many nodes as fit; a
 * configuration that does not fit is rejected with WSBB_ERR_CAPACITY
 * before anything runs, and a search that outgrows the capacity stops with
 * WSBB_ERR_CAPACITY (the context and the entry point stay usable).
 * Iterations are launched one by one (cfg->flags and cfg->graph_iters only
 * set how often the host polls; WSBB_EXPLORE_RESUME is rejected: the array
 * keeps no search between calls). With a NULL stream it follows the rule
 * above: it runs on the context's stream after the work already queued on
 * the legacy default stream (through an event made with the context).
 *
 * Every call looks up the array's device address (cudaGetSymbolAddress)
 * with the context's device current; the first such lookup on a device may
 * load the library's device code, so make the first call before any stream
 * capture. All calls share the one array and the search re-initialises
 * what it reads, so consecutive calls are independent, but calls that
 * overlap on the GPU (from two threads or two streams) race on the array
 * and must be serialised by the caller.
 */
#define WSBB_NOALLOC_SCRATCH_BYTES (24u << 20)
int wsbb_explore_noalloc(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg,
                         wsbb_stats *stats, void *stream);

/*
 * Learned machine-pair selector (no counterpart in the reference: the
 * reference only counts binding pairs, nbFois at src/bound_flowshop.cpp:157,
 * and its pair re-ordering is commented out, :129-130).
 *
 * A 3-layer MLP (D -> 128 -> 128 -> P, ReLU, bf16 operands, fp32
 * accumulation) maps a node's features — effective heads and tails and the
 * remaining work per machine, divided by the largest machine load, and the
 * free-job mask; D = round_up(3m + n, 16) — to scores of the P machine
 * pairs. Trained on
 * the GPU (Adam, softmax cross-entropy against the node's binding pair).
 * In a search it ranks, per father, the K pairs tried first on all of its
 * children; a child whose bound over those K pairs already reaches
 * max(best, incumbent) is settled without the other pairs. That leaves
 * the tree unchanged: such a child is pruned at birth either way and only
 * counts (never sums) in the side choice. With the reference default
 * best = 99999 nothing can be settled (the side choice sums every child's
 * exact bound), so the learned search is run with best = the initial
 * incumbent, and compared with the plain search at the same `best`.
 */
typedef struct wsbb_model wsbb_model;

int wsbb_model_create(int n, int m, uint64_t seed, wsbb_model **out); /* m <= 20 */
void wsbb_model_destroy(wsbb_model *model);
const char *wsbb_model_last_error(const wsbb_model *model);
int wsbb_model_dims(const wsbb_model *model, int *D, int *O, int64_t *nparams);
/* fp32 weights W1[D][128], b1, W2[128][128], b2, W3[128][O], b3 (O =
 * round_up(P, 8); columns >= P are padding) */
int wsbb_model_get_weights(const wsbb_model *model, float *host, int64_t count);
int wsbb_model_set_weights(wsbb_model *model, const float *host, int64_t count);
/* re-derive the bf16 inference weights after the fp32 ones changed */
int wsbb_model_pack(wsbb_model *model);

/* Features (rows of D floats, device) and, when `labels` is not NULL, the
 * binding pair of each record (-1 for leaves), for device records. */
float wsbb_feature_scale(const wsbb_ctx *ctx);
int wsbb_features(wsbb_ctx *ctx, const void *recs, int64_t count, float inv_scale, int D,
                  float *X, int32_t *labels, void *stream);
/* One forward/backward pass over B device rows: fp32 gradients (host,
 * nparams floats) and the summed loss (host). Synchronous. */
int wsbb_model_grads(wsbb_model *model, const float *X, const int32_t *y, int B,
                     float *grad_host, float *loss_host);
/* Adam training over `count` device rows; mean loss per epoch to host. */
int wsbb_model_train(wsbb_model *model, const float *X, const int32_t *y, int64_t count,
                     int epochs, int batch, float lr, uint64_t seed, float *epoch_loss_host);
/* Inference: top-K pair indices per row (device, best first) and,
 * optionally, the O logits per row (device). */
int wsbb_model_topk(wsbb_model *model, const float *X, int64_t rows, int K, int16_t *topk,
                    float *logits, void *stream);

/* The search of wsbb_explore with the learned K-pair test ahead of LB2
 * (1 <= K <= 32). Same counters as wsbb_explore with the same cfg;
 * stats->early counts children settled by the K pairs. */
int wsbb_explore_learned(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, wsbb_model *model, int K,
                         wsbb_stats *stats, void *stream);
/* The plain search, also copying a sample of the bounded children (every
 * `stride`-th, hashed per iteration) into `recs_out` (device, `cap`
 * records); *logged receives how many were written. Training data. */
int wsbb_explore_log(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, void *recs_out, int64_t cap,
                     int stride, int64_t *logged, wsbb_stats *stats, void *stream);

/* Measured integer max-plus issue rate of `device` (add + max operations
 * per second over every SM): the denominator of the LB2 kernel's
 * roofline. Synchronous; allocates a few bytes of device memory. No
 * counterpart in the reference. */
int wsbb_probe_maxplus_peak(int device, double *ops_per_s);

/* Host helpers (no device work). */
void wsbb_gen_instance(uint64_t seed, int n, int m, int32_t *p_mxn);
/* Times uniform in [1, 99] from Taillard's generator and time seed `seed`
 * (replaces instance_flowshop::unif / generate_instance,
 * src/instance_flowshop.cpp:74-89, for a given seed), machine-major. */
int wsbb_taillard_instance(int64_t seed, int n, int m, int32_t *p_mxn);
int32_t wsbb_neh(const int32_t *p_mxn, int n, int m, int32_t *perm_out);
/* Seeded random pool in the record format (f in [0, n-3], b in
 * [0, n-3-f]; a share of leaves). */
int wsbb_gen_pool(uint64_t seed, int n, int64_t count, double leaf_share,
                  void *recs_out);

#ifdef __cplusplus
}
#endif

#endif
