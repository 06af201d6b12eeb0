/*
 * TEST INFRASTRUCTURE — CPU oracle for the flowshop begin-end
 * branch-and-bound hot path. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only as the checker (or as
 * the timed CPU port). The product path never calls into it.
 *
 * It restates, in plain C, the reference's CPU algorithm:
 *   - bound precompute        src/bound_flowshop.cpp:486-659
 *   - LB2 / leaf makespan     src/bound_flowshop.cpp:64-168, 841-951
 *   - begin-end children      src/bb_problem_calculator.cpp:25-79
 *                             src/decompose_beginend.cpp:26-107
 *   - side choice / ranks     src/decompose_beginend.cpp:39-50,
 *                             src/problems.cpp:13-62, src/select_worst.cpp:7-12
 *   - DFS explorer            src/explorer.cu:92-148, src/tree.cpp:37-46,257-314
 *   - incumbent               src/solutions.cpp:37-65, src/eliminate_pareto.cpp:17-22
 * and adds what the reference lacks but the workloads need: a seeded
 * instance generator, the NEH heuristic (initial upper bound) and an LB1
 * one-machine bound. Parity of the restatement is pinned against the
 * reference's own compiled code (oracle/_ref, built by oracle/build_ref.sh)
 * through the golden fixtures in tests/golden/.
 */
#ifndef WSBB_FLOWSHOP_ORACLE_H
#define WSBB_FLOWSHOP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS_MAX_JOBS 128
#define FS_MAX_MACHINES 64

/* Seeded instance: p[k*n + j] = processing time of job j on machine k. */
void fs_gen_instance(uint64_t seed, int n, int m, int32_t *p_mxn);

typedef struct fs_bound fs_bound;

/* Precompute (pairs, lags, Johnson orders, heads, tails). NULL on error. */
fs_bound *fs_bound_create(const int32_t *p_mxn, int n, int m);
void fs_bound_destroy(fs_bound *b);
int fs_bound_pairs(const fs_bound *b);
/* Copies of the precomputed tables, for white-box tests. */
void fs_bound_tables(const fs_bound *b, int32_t *mach0, int32_t *mach1,
                     int32_t *lag_pxn, int32_t *johnson_pxn,
                     int32_t *min_arr, int32_t *min_dep);

/* bornes_calculer(perm, l1, l2, couts, best): LB2 of a partial node, or
 * the makespan when l2 - l1 == 1. best == -1 disables the early exit.
 * *argmax (may be NULL) receives the binding pair (first on ties), or -1. */
int32_t fs_bound_eval(const fs_bound *b, const int32_t *perm, int l1, int l2,
                      int32_t best, int32_t *argmax);
/* LB2 restricted to the given pair subset (max over listed pairs). */
int32_t fs_bound_eval_pairs(const fs_bound *b, const int32_t *perm, int l1,
                            int l2, const int32_t *pairs, int npairs);
/* One-machine bound LB1 (leaf: makespan). */
int32_t fs_lb1_eval(const fs_bound *b, const int32_t *perm, int l1, int l2);
int32_t fs_makespan(const fs_bound *b, const int32_t *perm);

/* Batches; perms is count x n, row-major. nthreads <= 1 runs inline. */
void fs_bound_eval_batch(const fs_bound *b, const int32_t *perms,
                         const int32_t *l1, const int32_t *l2, int64_t count,
                         int32_t *lb_out, int32_t *argmax_out, int nthreads);
void fs_lb1_eval_batch(const fs_bound *b, const int32_t *perms,
                       const int32_t *l1, const int32_t *l2, int64_t count,
                       int32_t *lb_out);

/* Seeded random partial-permutation pool (f in [0,n-3], b in [0,n-3-f]),
 * plus an optional share of leaves (l2 - l1 == 1). */
void fs_random_pool(uint64_t seed, int n, int64_t count, double leaf_share,
                    int32_t *perms, int32_t *l1, int32_t *l2);

/* NEH heuristic: returns the makespan, writes the sequence. */
int32_t fs_neh(const int32_t *p_mxn, int n, int m, int32_t *perm_out);

typedef struct {
	int64_t branched;       /* decomposed nodes (tree.cpp cpu_explored_nodes) */
	int64_t pruned;         /* pruned on take (boundedNodesDontExplore) */
	int64_t leaves;         /* leaves taken */
	int64_t improved;       /* incumbent improvements */
	int64_t bounded;        /* child bound evaluations */
	int64_t early_exits;    /* children settled by the pair-subset test */
	int32_t best_cost;      /* final incumbent (INT32_MAX if none) */
	int32_t pad;
	/* pruned nodes and leaves taken, per depth: the coverage (the sum of
	 * (n - depth)! over them, weights.cpp) is formed from it exactly by the
	 * caller, since it exceeds 128 bits from n = 35 on */
	uint64_t depth_hist[FS_MAX_JOBS + 1];
} fs_stats;

/* Exhaustive begin-end DFS with the reference's semantics.
 *   ub0      initial incumbent cost (INT32_MAX: none)
 *   best     decompose_beginend's choise threshold (99999 by default)
 *   node_cap stop after this many takes (0: no cap); returns 1 if capped
 *   pair_sel optional per-child pair subset used ahead of full LB2: a child
 *            whose max over the subset is >= best is settled as pruned with
 *            that partial value (the tree is unchanged when best <= the
 *            running incumbent); NULL disables it.
 *   log_cb   optional callback per bounded non-leaf child: (perm,l1,l2,
 *            argmax pair, lb, user) — used to log training data.
 * Returns 0 on success, 1 if the node cap was hit, <0 on error. */
typedef void (*fs_log_cb)(const int32_t *perm, int l1, int l2, int32_t argmax,
                          int32_t lb, void *user);
typedef int (*fs_pair_sel_cb)(const int32_t *perm, int l1, int l2,
                              int32_t *pairs_out, void *user);
int fs_explore(const fs_bound *b, int32_t ub0, int32_t best, int64_t node_cap,
               fs_stats *stats, int32_t *best_perm, fs_log_cb log_cb,
               fs_pair_sel_cb pair_sel, void *user);
/* The same search over the subtrees of `count` given open nodes (perms
 * count x n, cursors and bounds; node 0 at the bottom of the stack, the
 * last one taken first) instead of the root: the sequential counterpart of
 * seeding a GPU search with open nodes. */
int fs_explore_seeded(const fs_bound *b, const int32_t *perms, const int32_t *l1,
                      const int32_t *l2, const int32_t *lbs, int64_t count, int32_t ub0,
                      int32_t best, int64_t node_cap, fs_stats *stats, int32_t *best_perm);

#ifdef __cplusplus
}
#endif

#endif
