// The exact search's device side, shared by the graph-launched search
// (explore.cu) and the resident search (resident.cu): the stack's records
// and meta, the device state, and one body per phase of an iteration. Each
// translation unit that includes it gets its own copy of the device code
// (so each can be compiled with its own load-caching flags); the state
// types are plain data, defined alike in both.
#pragma once

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>

#include "node_features.cuh"
#include "wsbb_internal.h"

// The bodies below synchronise the threads that run them: the whole CTA,
// unless the including unit runs them on part of its CTAs' threads and
// defines both macros first (a barrier of those threads, and its
// predicate-or form).
#ifndef WSBB_BODY_SYNC
#define WSBB_BODY_SYNC() __syncthreads()
#define WSBB_BODY_SYNC_OR(p) __syncthreads_or(p)
#endif

namespace wsbb {

// CONDEMNED: a marker the incumbent already prunes whose whole subtree is
// marked DEAD, so commit can count it as pruned without walking the subtree.
// EXPORTED: an open node handed to another search (wsbb_explore_export);
// commit passes over it without counting it.
enum : uint8_t {
	ST_UNPROC = 0,
	ST_LEAF = 1,
	ST_PRUNED = 2,
	ST_BRANCHED = 3,
	ST_DEAD = 4,
	ST_CONDEMNED = 5,
	ST_EXPORTED = 6
};

struct Meta {
	int32_t lb;
	uint8_t depth;
	uint8_t state;
	uint16_t npruned; // BRANCHED: chosen children already pruned when emitted
};
static_assert(sizeof(Meta) == 8, "Meta is 8 bytes");

// Device-resident search state.
struct ExDev {
	long long top;          // index of the top entry (-1: empty)
	long long region_len;   // entries of the current rewrite region
	long long region_slots; // slots it occupies after the rewrite
	long long n_fathers;
	long long n_children;   // child records to bound this iteration
	long long iterations;
	int ub, best, done, error;
	int win, win_min, win_max, doom;
	// growth ceiling of the window: window / 16 after an incumbent
	// improvement, doubling every 128 iterations without one (speculation
	// against a stale incumbent is what an improvement discards)
	int win_cap, calm;
	unsigned long long branched, pruned, leaves, improved, bounded;
	unsigned long long evaluated, discarded, scanned, committed;
	unsigned long long fam_next;   // fathers claimed by the family-bounds CTAs
	unsigned long long early;      // children settled by the learned K-pair test
	unsigned long long settled_fathers; // fathers whose children it settled all
	long long n_unsettled;         // children left for full LB2 this iteration
	long long exported;            // nodes the last export took
	unsigned long long log_count;  // training records written
	unsigned long long hist[WSBB_MAX_JOBS + 1];
	// pend[d]: children of the open ancestor at depth d (of the next node
	// the sequential search takes) that were pruned at birth. They are
	// counted when their father commits, but the sequential search takes
	// them only after the father's open children's subtrees, when the
	// father's block closes; a stopped search subtracts them to report the
	// exact sequential prefix.
	unsigned pend[WSBB_MAX_JOBS + 1];
	// 1: keep pend (a search that may stop before it completes: an
	// iteration or node budget, or a seeded search); 0: a search that runs
	// to its end, where nothing is pending at the end and commit skips the
	// accounting
	int track_pend;
};

struct ExParams {
	ExDev *dev;
	uint8_t *rec;             // stack records [cap][stride]
	Meta *meta;               // stack meta [cap]
	uint8_t *tmp_rec;         // region copy [region_cap][stride]
	Meta *tmp_meta;           // [region_cap]
	int *fathers_before;      // [region_cap] fathers above each region entry
	int *father_of;           // [region_cap] father ordinal or -1
	long long *chunk_cnt;     // [n_chunks] candidates << kKidBits | their children, per
	                          // select chunk (then the chunk's base of both)
	long long *father_ridx;   // [window] region index of each father
	long long *child_off;     // [window + 1] first child record of each father
	int *father_side;         // [window] offset of the chosen side in its children
	int *father_kept;         // [window] chosen children still open
	int *father_npr;          // [window] chosen children pruned at birth
	long long *kept_before;   // [window + 1] slots of the father blocks above
	uint8_t *child_rec;       // [child_cap][stride]
	int32_t *child_lb;        // [child_cap]
	int16_t *child_job;       // [child_cap] job moved by the branching
	int32_t *child_rank;      // [child_cap] rank within the chosen side
	uint8_t *best_rec;        // [stride] incumbent permutation record
	long long cap, region_cap, child_cap;
	int window;               // maximum fathers per iteration
	int n_chunks;             // select chunks covering region_cap
	// learned mode
	float *feat;              // [window][D] father features
	int16_t *fpairs;          // [window][K] pairs ranked by the selector
	int32_t *unsettled;       // [child_cap] children left for full LB2
	int K, D;
	float inv_scale;
	// training-record logging
	uint8_t *log_rec;         // [log_cap][stride]
	long long log_cap;
	int log_stride;
	int n, stride;
};

namespace {

constexpr int kSelThreads = 1024;
// Entries per thread in the single-CTA scans: one block-scan round covers
// kItems * kSelThreads stack entries.
constexpr int kItems = 8;
constexpr int kChunk = kItems * kSelThreads;
// Select chunks: one 256-thread CTA scans kSelChunk entries.
constexpr int kSelCtaThreads = 256;
constexpr int kSelChunk = kItems * kSelCtaThreads;
// Select counts candidates and their children in one 64-bit sum: children
// in the low kKidBits bits (at most 2^24 region entries x 256 children),
// candidates above.
constexpr int kKidBits = 36;
constexpr long long kKidMask = (1ll << kKidBits) - 1;

__device__ __forceinline__ int children_of_depth(int depth, int n)
{
	// a non-leaf at depth d has n - d free jobs (a simple node: 2 leaves)
	return depth == n - 2 ? 2 : 2 * (n - depth);
}

// Block-wide exclusive scan for NT threads; `scratch` holds 32 values;
// `total` (optional) receives the block total.
template <int NT, typename T, typename Op>
__device__ T block_excl_scan(T v, Op op, T identity, T *scratch, T *total)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	T x = v;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		T y = __shfl_up_sync(0xffffffffu, x, d);
		if (lane >= d)
			x = op(x, y);
	}
	if (lane == 31)
		scratch[warp] = x;
	WSBB_BODY_SYNC();
	if (warp == 0) {
		T w = lane < (NT / 32) ? scratch[lane] : identity;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			T y = __shfl_up_sync(0xffffffffu, w, d);
			if (lane >= d)
				w = op(w, y);
		}
		scratch[lane] = w; // inclusive over warps
	}
	WSBB_BODY_SYNC();
	const T warp_prefix = warp == 0 ? identity : scratch[warp - 1];
	const T excl_in_warp = __shfl_up_sync(0xffffffffu, x, 1);
	const T excl = lane == 0 ? warp_prefix : op(warp_prefix, excl_in_warp);
	if (total)
		*total = scratch[NT / 32 - 1];
	WSBB_BODY_SYNC();
	return excl;
}

template <int NT, typename T, typename Op>
__device__ T block_reduce(T v, Op op, T identity, T *scratch)
{
	T total;
	block_excl_scan<NT>(v, op, identity, scratch, &total);
	return total;
}

// Block-wide exclusive suffix scan for NT threads: thread t receives
// op over the values of threads t + 1 .. NT - 1 (identity for the last).
template <int NT, typename T, typename Op>
__device__ T block_excl_suffix_scan(T v, Op op, T identity, T *scratch)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	constexpr int NW = NT / 32;
	T x = v;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		T y = __shfl_down_sync(0xffffffffu, x, d);
		if (lane + d < 32)
			x = op(x, y);
	}
	if (lane == 0)
		scratch[warp] = x; // inclusive suffix of the warp
	WSBB_BODY_SYNC();
	if (warp == 0) {
		T w = lane < NW ? scratch[lane] : identity;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			T y = __shfl_down_sync(0xffffffffu, w, d);
			if (lane + d < 32)
				w = op(w, y);
		}
		scratch[lane] = w; // inclusive suffix over warps
	}
	WSBB_BODY_SYNC();
	const T warp_suffix = warp == NW - 1 ? identity : scratch[warp + 1];
	const T excl_in_warp = __shfl_down_sync(0xffffffffu, x, 1);
	const T excl = lane == 31 ? warp_suffix : op(warp_suffix, excl_in_warp);
	WSBB_BODY_SYNC();
	return excl;
}

struct MinOp {
	__device__ int operator()(int a, int b) const { return a < b ? a : b; }
};
struct SumOp {
	__device__ long long operator()(long long a, long long b) const { return a + b; }
};

__device__ __forceinline__ bool halted(const ExDev *D) { return D->done || D->error; }

// Exclusive prefix sums over `count` items (one CTA of kSelThreads): item i
// has value get(i) (a non-negative int); put(i, sum of the items before
// i). A round stages kScanItems * kSelThreads items in shared memory with
// coalesced loads, each thread scans kScanItems consecutive ones (row
// padding of one word per 32 keeps those reads conflict-free), and the
// results leave with coalesced stores. Returns the total.
constexpr int kScanItems = 8;
__device__ __forceinline__ int scan_pad(int i) { return i + (i >> 5); }
// tile: kScanItems * NT + kScanItems * NT / 32 ints of shared memory
template <int NT, typename Get, typename Put>
__device__ long long cta_scan(long long count, Get get, Put put, long long *s_ll, int *tile)
{
	constexpr int kScanTile = kScanItems * NT;
	const int t = threadIdx.x;
	long long carry = 0;
	for (long long base = 0; base < count; base += kScanTile) {
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) {
			const int j = k * NT + t;
			tile[scan_pad(j)] = base + j < count ? get(base + j) : 0;
		}
		WSBB_BODY_SYNC();
		int v[kScanItems];
		int sum = 0;
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) {
			v[k] = tile[scan_pad(t * kScanItems + k)];
			sum += v[k];
		}
		long long tot;
		// the prefix inside a round fits int: at most kScanTile items of a
		// stack block or child count each
		int run = int(block_excl_scan<NT>((long long)sum, SumOp(), 0ll, s_ll, &tot));
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) {
			tile[scan_pad(t * kScanItems + k)] = run;
			run += v[k];
		}
		WSBB_BODY_SYNC();
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) {
			const int j = k * NT + t;
			if (base + j < count)
				put(base + j, carry + tile[scan_pad(j)]);
		}
		carry += tot;
		WSBB_BODY_SYNC(); // the tile is reused
	}
	return carry;
}

// ---- commit: walk down from the top in DFS order -------------------------
struct CommitShared {
	int s_int[32];
	unsigned long long s_cnt[6];
	// per-iteration depth counts (at most window * n each: 32 bits)
	unsigned s_hist[WSBB_MAX_JOBS + 1];
	// pending pruned-at-birth children per depth of their father (ExDev::pend)
	// and, within a round, the npruned of the round's suffix-minimum markers
	unsigned s_pend[WSBB_MAX_JOBS + 1], s_sfx[WSBB_MAX_JOBS + 1];
	int s_dmin;
};

// One CTA of NT threads, ITEMS stack entries per thread and round.
// `reset_claims`: zero the family bounds' father counter for the next
// iteration (the resident search manages its own).
template <int NT, int ITEMS>
__device__ void commit_body(const ExParams &P, CommitShared &sh, bool reset_claims)
{
	constexpr int kChunkT = ITEMS * NT;
	int *s_int = sh.s_int;
	unsigned long long *s_cnt = sh.s_cnt;
	unsigned *s_hist = sh.s_hist, *s_pend = sh.s_pend, *s_sfx = sh.s_sfx;
	int &s_dmin = sh.s_dmin;
	ExDev *D = P.dev;
	if (halted(D))
		return;
	const int t = threadIdx.x;
	const int n = P.n;
	if (t < 6)
		s_cnt[t] = 0;
	for (int i = t; i <= n; i += NT) {
		s_hist[i] = 0;
		s_pend[i] = D->pend[i];
		s_sfx[i] = 0;
	}
	WSBB_BODY_SYNC();

	long long top = D->top;
	const int ub0 = D->ub;
	const bool track = D->track_pend != 0;
	int ub = ub0;
	unsigned long long c_br = 0, c_pr = 0, c_lf = 0, c_im = 0, c_bd = 0, c_dead = 0;

	while (top >= 0) {
		// thread t holds entries top - (ITEMS*t + i), i = 0 nearest the top
		Meta e[ITEMS];
		int leaf_min = INT_MAX;
#pragma unroll
		for (int i = 0; i < ITEMS; ++i) {
			const long long idx = top - (long long)(ITEMS * t + i);
			e[i] = idx >= 0 ? P.meta[idx] : Meta{INT_MAX, 0, ST_UNPROC, 0};
			if (idx >= 0 && e[i].state == ST_LEAF)
				leaf_min = min(leaf_min, e[i].lb);
		}
		// leaves are rare: without one in the chunk the incumbent cannot
		// change in it, and both leaf scans below are skipped
		const int any_leaf = WSBB_BODY_SYNC_OR(leaf_min != INT_MAX);
		const int ub_in =
		    any_leaf ? min(ub, block_excl_scan<NT>(leaf_min, MinOp(), INT_MAX, s_int,
		                                                    (int *)nullptr))
		             : ub;
		// first entry that cannot be committed: an unprocessed node, the
		// stack bottom, or a marker failing against the running incumbent
		int first_stop = kChunkT;
		{
			int u = ub_in;
#pragma unroll
			for (int i = 0; i < ITEMS; ++i) {
				const long long idx = top - (long long)(ITEMS * t + i);
				const bool stop = idx < 0 || e[i].state == ST_UNPROC ||
				                  (e[i].state == ST_BRANCHED && e[i].lb >= u);
				if (stop && first_stop == kChunkT)
					first_stop = ITEMS * t + i;
				if (e[i].state == ST_LEAF)
					u = min(u, e[i].lb);
			}
		}
		const int s = block_reduce<NT>(first_stop, MinOp(), kChunkT, s_int);
		int chunk_min = INT_MAX, first_min = kChunkT;
		{
			int u = ub_in;
#pragma unroll
			for (int i = 0; i < ITEMS; ++i) {
				const int g = ITEMS * t + i;
				// coverage histogram: (depth, count) of what this entry adds
				int hkey = 255;
				unsigned hval = 0;
				if (g < s) {
					if (e[i].state == ST_BRANCHED) {
						c_br++;
						c_bd += (unsigned long long)children_of_depth(e[i].depth, n);
						if (e[i].npruned) {
							c_pr += e[i].npruned;
							hkey = e[i].depth + 1;
							hval = e[i].npruned;
						}
					} else if (e[i].state == ST_PRUNED || e[i].state == ST_CONDEMNED) {
						c_pr++;
						hkey = e[i].depth;
						hval = 1;
					} else if (e[i].state == ST_DEAD) {
						c_dead++; // inside a subtree the sequential search prunes
					} else if (e[i].state == ST_EXPORTED) {
						// another search took it over
					} else { // leaf
						c_lf++;
						hkey = n;
						hval = 1;
						if (e[i].lb < u)
							c_im++;
						u = min(u, e[i].lb);
						if (e[i].lb < chunk_min) {
							chunk_min = e[i].lb;
							first_min = g;
						}
					}
				}
				// 32-bit shared atomics (64-bit ones under contention cost
				// far more than the lanes that collide here)
				if (hkey != 255)
					atomicAdd(&s_hist[hkey], hval);
			}
		}
		const int cmin =
		    any_leaf ? block_reduce<NT>(chunk_min, MinOp(), INT_MAX, s_int) : INT_MAX;
		if (cmin < ub) {
			// the first leaf reaching the new minimum is the one that set it
			const int first = block_reduce<NT>(chunk_min == cmin ? first_min : kChunkT,
			                                            MinOp(), kChunkT, s_int);
			const long long src = top - first;
			for (int b = t; b < P.stride; b += NT)
				P.best_rec[b] = P.rec[src * P.stride + b];
			ub = cmin;
		}
		// Open blocks (only for a search that may stop early). A committed
		// entry of depth e closes the block of every
		// father of depth >= e (the sequential search has taken that
		// father's pruned-at-birth children just before it); a committed
		// marker opens its own. After the round, pend[d] for d >= the
		// round's smallest depth belongs to the last entry of depth <= d:
		// its npruned if it has depth d and is a marker, else 0. Those last
		// entries are the round's suffix minima of depth (distinct depths).
		if (track) {
			int loc_min = INT_MAX;
			bool has_np = false;
#pragma unroll
			for (int i = 0; i < ITEMS; ++i) {
				const int g = ITEMS * t + i;
				const bool pop = g < s && e[i].state != ST_DEAD && e[i].state != ST_EXPORTED;
				if (pop) {
					loc_min = min(loc_min, int(e[i].depth));
					has_np |= e[i].state == ST_BRANCHED && e[i].npruned;
				}
			}
			if (WSBB_BODY_SYNC_OR(has_np)) {
				int later = block_excl_suffix_scan<NT>(loc_min, MinOp(), INT_MAX, s_int);
				if (t == 0)
					s_dmin = min(later, loc_min);
#pragma unroll
				for (int i = ITEMS - 1; i >= 0; --i) {
					const int g = ITEMS * t + i;
					const bool pop = g < s && e[i].state != ST_DEAD && e[i].state != ST_EXPORTED;
					if (pop && int(e[i].depth) < later) {
						if (e[i].state == ST_BRANCHED)
							s_sfx[e[i].depth] = e[i].npruned;
						later = e[i].depth;
					}
				}
				WSBB_BODY_SYNC();
			} else {
				const int dm = block_reduce<NT>(loc_min, MinOp(), INT_MAX, s_int);
				if (t == 0)
					s_dmin = dm;
				WSBB_BODY_SYNC();
			}
			const int dmin = s_dmin;
			for (int d = t; d <= n; d += NT) {
				if (d >= dmin)
					s_pend[d] = s_sfx[d];
				s_sfx[d] = 0;
			}
		}
		top -= s;
		if (t == 0)
			D->committed += (unsigned long long)s;
		if (s == kChunkT)
			continue;
		if (top < 0)
			break;
		const Meta stopper = P.meta[top];
		if (stopper.state == ST_UNPROC)
			break;
		// A marker whose bound is not below the incumbent the sequential
		// search would hold here: that node is pruned, and everything
		// speculatively built under it is dropped.
		if (t == 0) {
			c_pr++;
			atomicAdd(&s_hist[stopper.depth], 1u);
		}
		for (int d = t; d <= n; d += NT)
			if (d >= stopper.depth)
				s_pend[d] = 0; // the pruned marker closes deeper blocks
		top -= 1;
		while (top >= 0) {
			int out_at = kChunkT;
#pragma unroll
			for (int i = 0; i < ITEMS; ++i) {
				const long long j = top - (long long)(ITEMS * t + i);
				const bool out = j < 0 || P.meta[j].depth <= stopper.depth;
				if (out && out_at == kChunkT)
					out_at = ITEMS * t + i;
			}
			const int s2 = block_reduce<NT>(out_at, MinOp(), kChunkT, s_int);
			if (t == 0)
				D->discarded += (unsigned long long)s2;
			top -= s2;
			if (s2 < kChunkT)
				break;
		}
	}

	// warp sums first: 1024 threads on one 64-bit shared counter serialise
	unsigned long long cv[6] = {c_br, c_pr, c_lf, c_im, c_bd, c_dead};
#pragma unroll
	for (int q = 0; q < 6; ++q) {
#pragma unroll
		for (int d = 16; d > 0; d >>= 1)
			cv[q] += __shfl_xor_sync(0xffffffffu, cv[q], d);
		if ((t & 31) == 0)
			atomicAdd(&s_cnt[q], cv[q]);
	}
	WSBB_BODY_SYNC();
	if (t == 0) {
		D->branched += s_cnt[0];
		D->pruned += s_cnt[1];
		D->leaves += s_cnt[2];
		D->improved += s_cnt[3];
		D->bounded += s_cnt[4];
		D->discarded += s_cnt[5];
		D->ub = ub;
		D->top = top;
		D->doom = ub < ub0 ? 1 : 0;
		if (ub < ub0) {
			D->win = D->win_min;
			D->win_cap = max(D->win_min, D->win_max >> 4);
			D->calm = 0;
		} else {
			if ((++D->calm & 127) == 0)
				D->win_cap = min(D->win_max, 2 * D->win_cap);
			D->win = min(D->win_cap, 2 * D->win);
		}
		D->iterations += 1;
		D->region_len = 0;
		D->region_slots = 0;
		D->n_fathers = 0;
		D->n_children = 0;
		D->n_unsettled = 0;
		if (reset_claims)
			D->fam_next = 0;
		if (top < 0)
			D->done = 1;
	}
	for (int i = t; i <= n; i += NT) {
		if (s_hist[i])
			D->hist[i] += s_hist[i];
		// the stack bottom closes every block
		D->pend[i] = top < 0 ? 0u : s_pend[i];
	}
}

__global__ void __launch_bounds__(kSelThreads) commit_kernel(ExParams P)
{
	__shared__ CommitShared sh;
	commit_body<kSelThreads, kItems>(P, sh, true);
}

// ---- doom: stop expanding under markers the new incumbent condemns ----------
// One warp walks the top region in DFS order carrying one value: the depth
// of the condemned marker whose subtree it is inside (or none). An entry at
// that depth or shallower ends the subtree (a subtree seen to its end
// settles its marker as CONDEMNED); entries inside it are marked dead so
// select never expands them. A marker outside any such subtree whose bound
// is not below the incumbent opens one. A marker whose subtree runs past
// the walk is left as it is: commit prunes it when it reaches the top (the
// sequential search prunes it on take, the incumbent never increases) and
// drops its whole subtree by depth.
// The walk takes 32 entries per step: the lane that closes the open subtree
// and the next marker that opens one are each found with one ballot, so a
// step costs a few instructions per subtree event instead of a pass per
// entry.
// Called by one warp.
__device__ void doom_body(const ExParams &P)
{
	ExDev *D = P.dev;
	if (halted(D) || !D->doom)
		return;
	const int lane = threadIdx.x & 31;
	const long long top = D->top;
	const int ub = D->ub;
	const long long stop = max(-1ll, top - P.region_cap);
	int dd = -1;              // depth of the open condemned subtree's marker (-1: none)
	long long dd_at = -1;     // its stack index
	// kDoomSteps steps of 32 entries are loaded at once (a step writes only
	// entries at or above its own, never the ones loaded for later steps)
	constexpr int kDoomSteps = 8;
	for (long long base0 = top; base0 > stop; base0 -= 32 * kDoomSteps) {
		Meta eb[kDoomSteps];
#pragma unroll
		for (int b = 0; b < kDoomSteps; ++b) {
			const long long idx = base0 - 32 * b - lane;
			eb[b] = idx > stop ? P.meta[idx] : Meta{0, 0, ST_DEAD, 0};
		}
#pragma unroll
		for (int b = 0; b < kDoomSteps; ++b) {
			const long long base = base0 - 32 * b;
			if (base <= stop)
				break; // uniform
			const long long idx = base - lane;
			const bool valid = idx > stop;
			const Meta e = eb[b];
			const int depth = e.depth;
			const unsigned condemned =
			    __ballot_sync(0xffffffffu, valid && e.state == ST_BRANCHED && e.lb >= ub);
			unsigned dead = 0;
			int from = 0; // lanes before `from` are settled for this step
			for (;;) {
				const unsigned rest = from >= 32 ? 0u : (0xffffffffu << from);
				if (dd >= 0) {
					const unsigned closer = __ballot_sync(0xffffffffu, valid && depth <= dd) & rest;
					if (!closer) {
						dead |= __ballot_sync(0xffffffffu, valid) & rest;
						break; // the subtree goes on past this step
					}
					const int c = __ffs(closer) - 1;
					dead |= rest & ~(0xffffffffu << c); // lanes [from, c)
					if (lane == 0)
						P.meta[dd_at].state = ST_CONDEMNED;
					dd = -1;
					from = c; // the closing entry may open a subtree itself
					continue;
				}
				const unsigned opener = condemned & rest;
				if (!opener)
					break;
				const int o = __ffs(opener) - 1;
				dd = __shfl_sync(0xffffffffu, depth, o);
				dd_at = base - o;
				from = o + 1;
			}
			if (valid && ((dead >> lane) & 1u))
				P.meta[idx].state = ST_DEAD;
		}
	}
	// a subtree that runs to the stack bottom also ended inside the walk
	if (dd >= 0 && stop < 0 && lane == 0)
		P.meta[dd_at].state = ST_CONDEMNED;
}

__global__ void doom_kernel(ExParams P) { doom_body(P); }

// ---- select ---------------------------------------------------------------
// Chunk c covers region entries [c * kSelChunk, (c + 1) * kSelChunk), region
// entry r being stack entry top - r.
// CTAs of kSelCtaThreads; CTA `bid` of `nblk` takes chunks bid, bid + nblk, ...
__device__ void select_count_body(const ExParams &P, int bid, int nblk, long long *s_ll)
{
	ExDev *D = P.dev;
	if (halted(D))
		return;
	const long long top = D->top;
	const int ub = D->ub;
	const long long scan_len = min(top + 1, P.region_cap);
	const int n = P.n;
	for (int c = bid; c < P.n_chunks; c += nblk) {
		long long cand = 0;
#pragma unroll
		for (int i = 0; i < kItems; ++i) {
			const long long r = (long long)c * kSelChunk + kItems * threadIdx.x + i;
			if (r >= scan_len)
				break;
			const long long idx = top - r;
			const Meta e = P.meta[idx];
			if (e.state == ST_UNPROC) {
				if (e.lb >= ub)
					P.meta[idx].state = ST_PRUNED; // final: the incumbent only decreases
				else
					cand += (1ll << kKidBits) + children_of_depth(e.depth, n);
			}
		}
		const long long total = block_reduce<kSelCtaThreads>(cand, SumOp(), 0ll, s_ll);
		if (threadIdx.x == 0)
			P.chunk_cnt[c] = total;
	}
}

__global__ void __launch_bounds__(kSelCtaThreads) select_count_kernel(ExParams P)
{
	__shared__ long long s_ll[32];
	select_count_body(P, blockIdx.x, gridDim.x, s_ll);
}

template <int NT>
__device__ void select_plan_body(const ExParams &P, long long *s_ll)
{
	ExDev *D = P.dev;
	if (halted(D))
		return;
	// each chunk's counts become the chunk's bases (both fields at once:
	// neither sum carries into the other)
	long long carry = 0;
	for (int base = 0; base < P.n_chunks; base += NT) {
		const int c = base + threadIdx.x;
		const long long v = c < P.n_chunks ? P.chunk_cnt[c] : 0;
		long long tot;
		const long long ex = block_excl_scan<NT>(v, SumOp(), 0ll, s_ll, &tot);
		if (c < P.n_chunks)
			P.chunk_cnt[c] = carry + ex;
		carry += tot;
	}
	if (threadIdx.x == 0)
		D->n_fathers = min(carry >> kKidBits, (long long)D->win);
}

__global__ void __launch_bounds__(kSelThreads) select_plan_kernel(ExParams P)
{
	__shared__ long long s_ll[32];
	select_plan_body<kSelThreads>(P, s_ll);
}

__device__ void select_write_body(const ExParams &P, int bid, int nblk, long long *s_ll)
{
	ExDev *D = P.dev;
	if (halted(D))
		return;
	const long long top = D->top;
	const long long nf = D->n_fathers;
	const int n = P.n;
	const long long scan_len = min(top + 1, P.region_cap);
	for (int c = bid; c < P.n_chunks; c += nblk) {
		const long long chunk_base = P.chunk_cnt[c];
		if ((long long)c * kSelChunk >= scan_len || (chunk_base >> kKidBits) >= nf)
			continue; // past the region (uniform per CTA)
		Meta e[kItems];
		long long cand = 0;
#pragma unroll
		for (int i = 0; i < kItems; ++i) {
			const long long r = (long long)c * kSelChunk + kItems * threadIdx.x + i;
			e[i] = r < scan_len ? P.meta[top - r] : Meta{0, 0, ST_DEAD, 0};
			if (e[i].state == ST_UNPROC)
				cand += (1ll << kKidBits) + children_of_depth(e[i].depth, n);
		}
		const long long ex = chunk_base + block_excl_scan<kSelCtaThreads>(cand, SumOp(), 0ll, s_ll,
		                                                                   (long long *)nullptr);
		long long order = ex >> kKidBits, kid = ex & kKidMask;
#pragma unroll
		for (int i = 0; i < kItems; ++i) {
			const long long r = (long long)c * kSelChunk + kItems * threadIdx.x + i;
			if (r >= scan_len)
				break;
			const bool take = e[i].state == ST_UNPROC && order < nf;
			P.fathers_before[r] = int(min(order, nf));
			P.father_of[r] = take ? int(order) : -1;
			if (e[i].state != ST_UNPROC)
				continue;
			const int kids = children_of_depth(e[i].depth, n);
			if (take) {
				// the father's first child: children of the fathers before it
				P.father_ridx[order] = r;
				P.child_off[order] = kid;
				if (order == nf - 1) {
					P.child_off[nf] = kid + kids;
					D->region_len = r + 1;
					D->n_children = kid + kids;
					D->evaluated += (unsigned long long)(kid + kids);
					D->scanned += (unsigned long long)(r + 1);
				}
			}
			order++;
			kid += kids;
		}
	}
}

__global__ void __launch_bounds__(kSelCtaThreads) select_write_kernel(ExParams P)
{
	__shared__ long long s_ll[32];
	select_write_body(P, blockIdx.x, gridDim.x, s_ll);
}

// Copy the region aside and, when a later step reads them (per-child
// bounds, the learned test, logging), write every father's child records.
__device__ void make_children_body(const ExParams &P, int write_children, long long gtid,
                                   long long gsz)
{
	ExDev *D = P.dev;
	if (D->done || D->error || D->n_fathers == 0)
		return;
	const long long top = D->top, rlen = D->region_len, nf = D->n_fathers;
	const int S = P.stride, n = P.n;
	// region copy, 16 bytes per thread step
	const long long words = rlen * (S / 16);
	for (long long w = gtid; w < words; w += gsz) {
		const long long r = w / (S / 16), c = w % (S / 16);
		reinterpret_cast<uint4 *>(P.tmp_rec + r * S)[c] =
		    reinterpret_cast<const uint4 *>(P.rec + (top - r) * S)[c];
	}
	for (long long r = gtid; r < rlen; r += gsz)
		P.tmp_meta[r] = P.meta[top - r];
	if (!write_children)
		return;
	// children: one thread per child record
	const long long total = D->n_children;
	for (long long c = gtid; c < total; c += gsz) {
		long long lo = 0, hi = nf - 1; // father with child_off[f] <= c
		while (lo < hi) {
			const long long mid = (lo + hi + 1) >> 1;
			if (P.child_off[mid] <= c)
				lo = mid;
			else
				hi = mid - 1;
		}
		const long long f = lo;
		const int k = int(c - P.child_off[f]);
		const long long fidx = top - P.father_ridx[f];
		const int16_t *fr = reinterpret_cast<const int16_t *>(P.rec + fidx * S);
		int16_t *cr = reinterpret_cast<int16_t *>(P.child_rec + c * S);
		const int l1 = fr[n], l2 = fr[n + 1], depth = fr[n + 2];
		for (int j = 0; j < n; ++j)
			cr[j] = fr[j];
		int nl1 = l1, nl2 = l2, slot, indice;
		if (depth == n - 2) { // simple: the two orders of the last two jobs
			indice = l1 + 1 + k;
			slot = l1 + 1;
			nl1 = l1 + 1;
		} else {
			const int u = l2 - l1 - 1;
			const bool end_side = k >= u;
			indice = l1 + 1 + (end_side ? k - u : k);
			slot = end_side ? l2 - 1 : l1 + 1;
			if (end_side)
				nl2 = l2 - 1;
			else
				nl1 = l1 + 1;
		}
		if (nl2 - nl1 == 2)
			nl1++; // the last free job goes in place (limites_set)
		const int16_t moved = fr[indice];
		cr[indice] = fr[slot];
		cr[slot] = moved;
		cr[n] = int16_t(nl1);
		cr[n + 1] = int16_t(nl2);
		cr[n + 2] = int16_t(depth == n - 2 ? n : depth + 1);
		cr[n + 3] = 0;
		for (int j = n + 4; j < S / 2; ++j)
			cr[j] = 0;
		P.child_job[c] = moved;
	}
}

__global__ void make_children_kernel(ExParams P, int write_children)
{
	make_children_body(P, write_children, (long long)blockIdx.x * blockDim.x + threadIdx.x,
	                   (long long)gridDim.x * blockDim.x);
}

// Per father (one warp): choise, ranks of the chosen side, and how many of
// the chosen children the incumbent already prunes.
__device__ void choose_body(const ExParams &P, long long warp, long long nwarps)
{
	ExDev *D = P.dev;
	if (D->done || D->error || D->n_fathers == 0)
		return;
	const int lane = threadIdx.x & 31;
	const long long nf = D->n_fathers;
	const int ub = D->ub, best = D->best;
	for (long long f = warp; f < nf; f += nwarps) {
		const long long c0 = P.child_off[f];
		const int nc = int(P.child_off[f + 1] - c0);
		const bool simple = nc == 2 && P.tmp_meta[P.father_ridx[f]].depth == P.n - 2;
		const int kept_all = simple ? 2 : nc / 2;
		int side_off = 0;
		if (!simple) {
			// choise: more children >= best wins; else the larger sum of the
			// bounds below best; ties go to the END side
			// (per side, in registers: a runtime-indexed array would live in
			// local memory)
			long long sum0 = 0, sum1 = 0;
			int cut0 = 0, cut1 = 0;
			for (int k = lane; k < nc; k += 32) {
				const int lb = P.child_lb[c0 + k];
				const bool end_side = k >= kept_all;
				const bool cut = lb >= best;
				cut0 += !end_side && cut;
				cut1 += end_side && cut;
				sum0 += !end_side && !cut ? lb : 0;
				sum1 += end_side && !cut ? lb : 0;
			}
#pragma unroll
			for (int d = 16; d > 0; d >>= 1) {
				sum0 += __shfl_xor_sync(0xffffffffu, sum0, d);
				sum1 += __shfl_xor_sync(0xffffffffu, sum1, d);
				cut0 += __shfl_xor_sync(0xffffffffu, cut0, d);
				cut1 += __shfl_xor_sync(0xffffffffu, cut1, d);
			}
			const bool begin = cut0 != cut1 ? cut0 > cut1 : sum0 > sum1;
			side_off = begin ? 0 : kept_all;
		}
		// rank 0 = smallest bound, ties to the smaller job (select_worst);
		// child k = lane + 32 i is held by its lane in slot i and the others'
		// keys arrive by shuffle
		constexpr int kSlots = (WSBB_MAX_JOBS + 31) / 32;
		int lbs[kSlots], jbs[kSlots];
#pragma unroll
		for (int i = 0; i < kSlots; ++i) {
			const int k = lane + 32 * i;
			const bool in = k < kept_all;
			lbs[i] = in ? P.child_lb[c0 + side_off + k] : INT_MAX;
			jbs[i] = in ? int(P.child_job[c0 + side_off + k]) : INT_MAX;
		}
		int rk[kSlots] = {};
		if (kept_all <= 32) {
			// one slot: the common case
			for (int q = 0; q < kept_all; ++q) {
				const int lq = __shfl_sync(0xffffffffu, lbs[0], q);
				const int jq = __shfl_sync(0xffffffffu, jbs[0], q);
				rk[0] += (lq < lbs[0]) || (lq == lbs[0] && jq < jbs[0]);
			}
		} else {
#pragma unroll
			for (int j = 0; j < kSlots; ++j) {
				const int qn = min(32, kept_all - 32 * j); // <= 0: slot j holds none
				for (int q = 0; q < qn; ++q) {
					const int lq = __shfl_sync(0xffffffffu, lbs[j], q);
					const int jq = __shfl_sync(0xffffffffu, jbs[j], q);
#pragma unroll
					for (int i = 0; i < kSlots; ++i)
						rk[i] += (lq < lbs[i]) || (lq == lbs[i] && jq < jbs[i]);
				}
			}
		}
		int open = 0;
#pragma unroll
		for (int i = 0; i < kSlots; ++i) {
			const int k = lane + 32 * i;
			if (k < kept_all) {
				P.child_rank[c0 + side_off + k] = rk[i];
				open += (simple || lbs[i] < ub) ? 1 : 0;
			}
		}
#pragma unroll
		for (int d = 16; d > 0; d >>= 1)
			open += __shfl_xor_sync(0xffffffffu, open, d);
		if (lane == 0) {
			P.father_side[f] = side_off;
			P.father_kept[f] = open;
			P.father_npr[f] = kept_all - open;
		}
	}
}

__global__ void choose_kernel(ExParams P)
{
	choose_body(P, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
	            ((long long)gridDim.x * blockDim.x) >> 5);
}

// Block sizes of the fathers in the rewritten region (one CTA).
template <int NT>
__device__ void kept_scan_body(const ExParams &P, long long *s_ll, int *tile)
{
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0)
		return;
	const long long nf = D->n_fathers;
	const long long carry = cta_scan<NT>(
	    nf, [&](long long f) { return 1 + P.father_kept[f]; },
	    [&](long long f, long long v) { P.kept_before[f] = v; }, s_ll, tile);
	if (threadIdx.x == 0) {
		P.kept_before[nf] = carry;
		const long long slots = (D->region_len - nf) + carry;
		const long long new_top = D->top - D->region_len + slots;
		if (new_top >= P.cap) {
			D->error = WSBB_ERR_CAPACITY;
			D->n_fathers = 0;
			D->region_len = 0;
		}
		D->region_slots = slots;
	}
}

__global__ void __launch_bounds__(kSelThreads) kept_scan_kernel(ExParams P)
{
	__shared__ long long s_ll[32];
	__shared__ int tile[kScanItems * kSelThreads + kScanItems * kSelThreads / 32];
	kept_scan_body<kSelThreads>(P, s_ll, tile);
}

// Half q (0-7) of a 16-byte record word set to v.
__device__ __forceinline__ void set_half(uint4 &w, int q, int16_t v)
{
	const int sh = (q & 1) * 16;
	const uint32_t keep = ~(0xffffu << sh), val = uint32_t(uint16_t(v)) << sh;
	const int i = q >> 1;
	w.x = i == 0 ? (w.x & keep) | val : w.x;
	w.y = i == 1 ? (w.y & keep) | val : w.y;
	w.z = i == 2 ? (w.z & keep) | val : w.z;
	w.w = i == 3 ? (w.w & keep) | val : w.w;
}

// Scatter the rewritten region. Work items, grid-strided: first one thread
// per 16-byte word of every region entry (region entry r moves to its new
// slot; fathers become BRANCHED markers), then one warp per father, which
// writes the father's open children — contiguous slots just above its
// marker, by rank — as one coalesced run of words. Region entry r has
// r - fb non-father entries above it (one slot each) and fb father blocks
// (kept_before[fb] slots), fb = fathers above it.
constexpr int kEmitThreads = 256;
// CTAs of kEmitThreads; s_inv: per warp, rank -> child
__device__ void emit_body(const ExParams &P, long long bid, long long nblk,
                          uint8_t (*s_inv)[WSBB_MAX_JOBS])
{
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0)
		return;
	const int S = P.stride, n = P.n, W = S / 16;
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	const long long rlen = D->region_len, nf = D->n_fathers;
	const long long new_top = D->top - rlen + D->region_slots;
	const long long words = rlen * W;
	const long long part2 = (words + 31) & ~31ll; // fathers start on a warp boundary
	const long long items = part2 + nf * 32;
	const long long gsz = nblk * kEmitThreads;
	for (long long w0 = bid * kEmitThreads; w0 < items; w0 += gsz) {
		const long long w = w0 + threadIdx.x;
		const long long wbase = w0 + (threadIdx.x & ~31); // the warp's first item
		if (wbase >= items)
			continue; // past the last father (warp-uniform)
		if (wbase < part2) {
			if (w >= words)
				continue;
			const long long r = w / W;
			const int c = int(w - r * W);
			const int fb = P.fathers_before[r];
			const long long hi_slot = new_top - ((r - fb) + P.kept_before[fb]);
			reinterpret_cast<uint4 *>(P.rec + hi_slot * S)[c] =
			    reinterpret_cast<const uint4 *>(P.tmp_rec + r * S)[c];
			if (c == 0) {
				Meta mm = P.tmp_meta[r];
				const int f = P.father_of[r];
				if (f >= 0) {
					mm.state = ST_BRANCHED;
					mm.npruned = uint16_t(P.father_npr[f]);
				}
				P.meta[hi_slot] = mm;
			}
			continue;
		}
		const long long f = (wbase - part2) >> 5; // < nf
		const long long r = P.father_ridx[f];
		const Meta fm = P.tmp_meta[r];
		const bool simple = fm.depth == n - 2;
		const int kept_all = simple ? 2 : int(P.child_off[f + 1] - P.child_off[f]) / 2;
		const int side_off = P.father_side[f];
		const long long c0 = P.child_off[f] + side_off;
		const int open = P.father_kept[f];
		for (int k = lane; k < kept_all; k += 32) {
			const int rank = P.child_rank[c0 + k];
			if (rank < open)
				s_inv[wib][rank] = uint8_t(k);
		}
		__syncwarp();
		// the child of rank q sits at slot hi_slot - 1 - q: the run starts
		// at the highest rank
		const long long lo_slot = new_top - ((r - f) + P.kept_before[f]) - open;
		const uint4 *src = reinterpret_cast<const uint4 *>(P.tmp_rec + r * S);
		const int16_t *fr16 = reinterpret_cast<const int16_t *>(src);
		const int fl1 = fr16[n], fl2 = fr16[n + 1];
		const int to = (simple || side_off == 0) ? fl1 + 1 : fl2 - 1;
		const int16_t at_to = fr16[to];
		const int16_t h_l1 = int16_t(simple ? fl1 + 2 : (side_off == 0 ? fl1 + 1 : fl1));
		const int16_t h_l2 = int16_t((simple || side_off == 0) ? fl2 : fl2 - 1);
		const int16_t h_depth = int16_t(simple ? n : fm.depth + 1);
		uint4 *dst = reinterpret_cast<uint4 *>(P.rec + lo_slot * S);
		for (int wi = lane; wi < open * W; wi += 32) {
			const int j = wi / W, c = wi - j * W; // run record j holds rank open - 1 - j
			const int k = s_inv[wib][open - 1 - j];
			const int indice = fl1 + 1 + k;
			uint4 word = src[c];
			const int lo = 8 * c;
			if ((indice >> 3) == c)
				set_half(word, indice - lo, at_to);
			if ((to >> 3) == c)
				set_half(word, to - lo, fr16[indice]);
			if ((n >> 3) == c)
				set_half(word, n - lo, h_l1);
			if (((n + 1) >> 3) == c)
				set_half(word, n + 1 - lo, h_l2);
			if (((n + 2) >> 3) == c)
				set_half(word, n + 2 - lo, h_depth);
			dst[wi] = word;
			if (c == 0) {
				Meta cm;
				cm.lb = P.child_lb[c0 + k];
				cm.depth = uint8_t(h_depth);
				cm.state = simple ? ST_LEAF : ST_UNPROC;
				cm.npruned = 0;
				P.meta[lo_slot + j] = cm;
			}
		}
		__syncwarp(); // s_inv is reused by the warp's next father
	}
}

__global__ void __launch_bounds__(kEmitThreads) emit_kernel(ExParams P)
{
	__shared__ uint8_t s_inv[kEmitThreads / 32][WSBB_MAX_JOBS];
	emit_body(P, blockIdx.x, gridDim.x, s_inv);
}

__device__ __forceinline__ void finish_body(const ExParams &P)
{
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0)
		return;
	D->top = D->top - D->region_len + D->region_slots;
}

__global__ void finish_iteration_kernel(ExParams P) { finish_body(P); }

__global__ void init_kernel(ExParams P, int ub0, int best, int win_min, int win_max,
                            int track_pend)
{
	ExDev *D = P.dev;
	const int n = P.n, S = P.stride;
	if (threadIdx.x == 0) {
		memset(D, 0, sizeof(ExDev));
		D->track_pend = track_pend;
		D->top = 0;
		D->ub = ub0;
		D->best = best;
		D->win = win_min;
		D->win_min = win_min;
		D->win_max = win_max;
		D->win_cap = win_max;
		D->calm = 0;
		Meta m0 = {0, 0, ST_UNPROC, 0};
		P.meta[0] = m0;
	}
	int16_t *r = reinterpret_cast<int16_t *>(P.rec);
	for (int j = threadIdx.x; j < S / 2; j += blockDim.x) {
		int16_t v = 0;
		if (j < n)
			v = int16_t(j);
		else if (j == n)
			v = -1;
		else if (j == n + 1)
			v = int16_t(n);
		r[j] = v;
		reinterpret_cast<int16_t *>(P.best_rec)[j] = int16_t(j < n ? -1 : 0);
	}
}

// A search state whose stack holds `count` given open nodes (records and
// meta already in place, entry 0 at the bottom).
__global__ void seed_kernel(ExParams P, long long count, int ub0, int best, int win_min,
                            int win_max)
{
	ExDev *D = P.dev;
	const int n = P.n, S = P.stride;
	if (threadIdx.x == 0) {
		memset(D, 0, sizeof(ExDev));
		D->track_pend = 1;
		D->top = count - 1;
		D->done = count == 0;
		D->ub = ub0;
		D->best = best;
		D->win = win_min;
		D->win_min = win_min;
		D->win_max = win_max;
		D->win_cap = win_max;
	}
	for (int j = threadIdx.x; j < S / 2; j += blockDim.x)
		reinterpret_cast<int16_t *>(P.best_rec)[j] = int16_t(j < n ? -1 : 0);
}

// Continue a stopped search: an incumbent found elsewhere may lower the
// cost (its permutation stays with whoever found it).
__global__ void resume_kernel(ExParams P, int ub0, int best)
{
	ExDev *D = P.dev;
	if (threadIdx.x == 0) {
		D->ub = min(D->ub, ub0);
		D->best = best;
		D->done = D->top < 0 ? 1 : 0;
	}
}

// Take up to max_count open nodes from the bottom of the stack (one CTA):
// each is copied to tmp_rec / tmp_meta in stack order and left EXPORTED.
// Open nodes the incumbent already prunes are not taken.
__global__ void __launch_bounds__(kSelThreads) export_kernel(ExParams P, long long max_count)
{
	__shared__ long long s_ll[32];
	ExDev *D = P.dev;
	const long long top = D->top;
	const int ub = D->ub, S = P.stride, t = threadIdx.x;
	long long taken = 0;
	for (long long base = 0; base <= top && taken < max_count; base += kChunk) {
		// thread t holds entries base + kItems t + i
		long long cand = 0;
#pragma unroll
		for (int i = 0; i < kItems; ++i) {
			const long long idx = base + (long long)kItems * t + i;
			if (idx <= top) {
				const Meta e = P.meta[idx];
				cand += e.state == ST_UNPROC && e.lb < ub;
			}
		}
		long long tot;
		long long order = taken + block_excl_scan<kSelThreads>(cand, SumOp(), 0ll, s_ll, &tot);
#pragma unroll
		for (int i = 0; i < kItems; ++i) {
			const long long idx = base + (long long)kItems * t + i;
			if (idx > top)
				break;
			Meta e = P.meta[idx];
			if (e.state != ST_UNPROC || e.lb >= ub)
				continue;
			if (order < max_count) {
				const uint4 *src = reinterpret_cast<const uint4 *>(P.rec + idx * S);
				uint4 *dst = reinterpret_cast<uint4 *>(P.tmp_rec + order * S);
				for (int c = 0; c < S / 16; ++c)
					dst[c] = src[c];
				P.tmp_meta[order] = e;
				e.state = ST_EXPORTED;
				P.meta[idx] = e;
			}
			++order;
		}
		taken = min(max_count, taken + tot);
	}
	if (t == 0)
		D->exported = taken;
}

// ---- learned mode ----------------------------------------------------------

// Features of every father (from the region copy), for the pair selector.
__global__ void father_features_kernel(ExParams P, BoundParams bp)
{
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0)
		return;
	const int n = P.n, m = bp.m;
	const uint8_t *tb = bp.t8.blob;
	const int32_t *pt = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pt);
	const int32_t *heads = reinterpret_cast<const int32_t *>(tb + bp.t8.off_heads);
	const int32_t *tails = reinterpret_cast<const int32_t *>(tb + bp.t8.off_tails);
	const long long nf = D->n_fathers;
	for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < nf;
	     f += (long long)gridDim.x * blockDim.x) {
		const int16_t *rec =
		    reinterpret_cast<const int16_t *>(P.tmp_rec + P.father_ridx[f] * P.stride);
		int32_t F[WSBB_MAX_MACHINES], G[WSBB_MAX_MACHINES], R[WSBB_MAX_MACHINES];
		node_times(rec, n, m, pt, F, G);
		const int l1 = rec[n], l2 = rec[n + 1];
		for (int k = 0; k < m; ++k) {
			F[k] = l1 >= 0 ? F[k] : heads[k];
			R[k] = l2 < n ? G[m - 1 - k] : tails[k];
		}
		uint32_t mask[4];
		free_mask(rec, n, mask);
		write_features(F, R, mask, n, m, pt, P.inv_scale, P.D, P.feat + f * P.D);
	}
}

constexpr int kPartialThreads = 256;

__device__ __forceinline__ bool job_free(const uint32_t (&mask)[4], int job)
{
	const uint32_t w01 = (job & 32) ? mask[1] : mask[0];
	const uint32_t w23 = (job & 32) ? mask[3] : mask[2];
	return ((((job & 64) ? w23 : w01) >> (job & 31)) & 1u) != 0;
}

// One warp per father, its children in passes of 32 lanes. Every child of
// a father is tried on the father's K ranked pairs (so all lanes read the
// same table entries: broadcasts). A child whose bound over those pairs
// already reaches max(best, incumbent) keeps that value; the others — and
// the leaves of simple fathers — go to the full-LB2 list.
template <int MAXM>
__global__ void __launch_bounds__(kPartialThreads) partial_kernel(ExParams P, BoundParams bp)
{
	extern __shared__ __align__(16) uint8_t smem[];
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0)
		return;
	{
		const uint4 *src = reinterpret_cast<const uint4 *>(bp.t8.blob);
		uint4 *dst = reinterpret_cast<uint4 *>(smem);
		for (uint32_t i = threadIdx.x; i < bp.t8.bytes / 16; i += blockDim.x)
			dst[i] = src[i];
	}
	WSBB_BODY_SYNC();
	const int n = P.n, m = bp.m, K = P.K;
	const uint2 *tj = reinterpret_cast<const uint2 *>(smem);
	const int32_t *pt = reinterpret_cast<const int32_t *>(smem + bp.t8.off_pt);
	const int32_t *pairs = reinterpret_cast<const int32_t *>(smem + bp.t8.off_pairs);
	const int32_t *heads = reinterpret_cast<const int32_t *>(smem + bp.t8.off_heads);
	const int32_t *tails = reinterpret_cast<const int32_t *>(smem + bp.t8.off_tails);
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	int32_t *colF = reinterpret_cast<int32_t *>(smem + bp.t8.bytes) + wib * 2 * MAXM * 32;
	int32_t *colR = colF + MAXM * 32;
	const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
	const long long nf = D->n_fathers;
	const int thr = max(D->best, D->ub);
	for (long long f = warp; f < nf; f += nwarps) {
		const long long c0 = P.child_off[f];
		const int nc = int(P.child_off[f + 1] - c0);
		const long long ridx = P.father_ridx[f];
		const int16_t *fr = reinterpret_cast<const int16_t *>(P.tmp_rec + ridx * P.stride);
		const int depth = P.tmp_meta[ridx].depth;
		if (depth == n - 2) { // leaves: makespans come from the full path
			const unsigned base = lane == 0 ? (unsigned)atomicAdd(
			                                      (unsigned long long *)&D->n_unsettled,
			                                      (unsigned long long)nc)
			                                : 0u;
			const unsigned b0 = __shfl_sync(0xffffffffu, base, 0);
			for (int k = lane; k < nc; k += 32)
				P.unsettled[b0 + k] = int32_t(c0 + k);
			continue;
		}
		const int l1 = fr[n], l2 = fr[n + 1];
		const int u = l2 - l1 - 1;
		// father's raw front / reversed back times (every lane, same values)
		int32_t Fr[MAXM], Gr[MAXM];
#pragma unroll
		for (int k = 0; k < MAXM; ++k)
			Fr[k] = Gr[k] = 0;
		for (int j = 0; j <= l1; ++j) {
			const int job = fr[j];
			Fr[0] += pt[job];
#pragma unroll
			for (int k = 1; k < MAXM; ++k)
				if (k < m)
					Fr[k] = max(Fr[k], Fr[k - 1]) + pt[k * n + job];
		}
		for (int j = n - 1; j >= l2; --j) {
			const int job = fr[j];
			Gr[0] += pt[(m - 1) * n + job];
#pragma unroll
			for (int q = 1; q < MAXM; ++q)
				if (q < m)
					Gr[q] = max(Gr[q], Gr[q - 1]) + pt[(m - 1 - q) * n + job];
		}
		uint32_t fmask[4] = {0, 0, 0, 0};
		for (int j = l1 + 1; j < l2; ++j)
			fmask[fr[j] >> 5] |= 1u << (fr[j] & 31);
		const int16_t *my_pairs = P.fpairs + f * K;
		for (int pass = 0; pass < nc; pass += 32) {
			const int k = pass + lane;
			const bool active = k < nc;
			const long long c = c0 + (active ? k : 0);
			const int job = active ? P.child_job[c] : fr[l1 + 1];
			const bool end_side = k >= u;
			// the child's front / back: the father's plus the moved job
			const int fcount = l1 + 1 + (end_side ? 0 : 1);
			const int bcount = n - l2 + (end_side ? 1 : 0);
			int32_t prevF = 0, prevG = 0;
#pragma unroll
			for (int q = 0; q < MAXM; ++q) {
				if (q >= m)
					break;
				int32_t fv = Fr[q], gv = Gr[q];
				if (!end_side) {
					fv = (q == 0 ? Fr[0] : max(prevF, Fr[q])) + pt[q * n + job];
					prevF = fv;
				} else {
					gv = (q == 0 ? Gr[0] : max(prevG, Gr[q])) + pt[(m - 1 - q) * n + job];
					prevG = gv;
				}
				colF[q * 32 + lane] = fcount > 0 ? fv : heads[q];
				colR[(m - 1 - q) * 32 + lane] = bcount > 0 ? gv : tails[m - 1 - q];
			}
			uint32_t mask[4] = {fmask[0], fmask[1], fmask[2], fmask[3]};
			mask[job >> 5] &= ~(1u << (job & 31));
			const int32_t tail_off = bcount > 0 ? 0 : -(1 << 30);
			int32_t part = 0;
			for (int i = 0; i < K; ++i) {
				const int pi = my_pairs[i];
				const int a = pairs[pi] & 0xff, b = pairs[pi] >> 8;
				int32_t t0 = colF[a * 32 + lane], t1 = colF[b * 32 + lane];
				const uint2 *e = tj + pi * n;
				for (int q = 0; q < n; ++q) {
					const uint2 v = e[q];
					if (job_free(mask, int(v.x & 0xffu))) {
						t0 += int32_t(v.x >> 16);
						t1 = max(t1, t0 + int32_t(v.y >> 16)) + int32_t(v.y & 0xffffu);
					}
				}
				part = max(part, max(t1 + colR[b * 32 + lane], t0 + colR[a * 32 + lane] + tail_off));
			}
			const bool settled = active && part >= thr;
			if (settled)
				P.child_lb[c] = part;
			const unsigned open = __ballot_sync(0xffffffffu, active && !settled);
			const unsigned done = __ballot_sync(0xffffffffu, settled);
			unsigned base = 0;
			if (lane == 0) {
				base = (unsigned)atomicAdd((unsigned long long *)&D->n_unsettled,
				                           (unsigned long long)__popc(open));
				if (done)
					atomicAdd(&D->early, (unsigned long long)__popc(done));
			}
			base = __shfl_sync(0xffffffffu, base, 0);
			if (active && !settled)
				P.unsettled[base + __popc(open & ((1u << lane) - 1u))] = int32_t(c);
			__syncwarp();
		}
	}
}

// Training records: a hashed sample of this iteration's bounded children.
__global__ void log_kernel(ExParams P)
{
	ExDev *D = P.dev;
	if (halted(D) || D->n_fathers == 0 || !P.log_rec)
		return;
	const long long total = D->n_children;
	const unsigned long long it = (unsigned long long)D->iterations;
	const int S = P.stride;
	for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < total;
	     c += (long long)gridDim.x * blockDim.x) {
		unsigned long long h = (unsigned long long)c * 0x9E3779B97F4A7C15ULL ^ (it << 32);
		h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9ULL;
		h ^= h >> 32;
		if (h % (unsigned long long)P.log_stride != 0)
			continue;
		const unsigned long long slot = atomicAdd(&D->log_count, 1ull);
		if (slot >= (unsigned long long)P.log_cap)
			continue;
		const uint4 *src = reinterpret_cast<const uint4 *>(P.child_rec + c * S);
		uint4 *dst = reinterpret_cast<uint4 *>(P.log_rec + slot * S);
		for (int q = 0; q < S / 16; ++q)
			dst[q] = src[q];
	}
}

// Lays the search buffers out from `base` (null: only sizes them).
size_t search_layout(uint8_t *base, long long cap, long long region_cap, int window, int n,
                     int S, ExParams &P)
{
	const long long child_cap = (long long)window * 2 * n;
	const int n_chunks = int((region_cap + kSelChunk - 1) / kSelChunk);
	auto a256 = [](size_t v) { return (v + 255) & ~size_t(255); };
	size_t off = 0;
	auto take = [&](size_t bytes) {
		const size_t at = off;
		off = a256(off + bytes);
		return base ? base + at : nullptr;
	};
	P.dev = reinterpret_cast<ExDev *>(take(sizeof(ExDev)));
	P.rec = take(size_t(cap) * S);
	P.meta = reinterpret_cast<Meta *>(take(size_t(cap) * sizeof(Meta)));
	P.tmp_rec = take(size_t(region_cap) * S);
	P.tmp_meta = reinterpret_cast<Meta *>(take(size_t(region_cap) * sizeof(Meta)));
	P.fathers_before = reinterpret_cast<int *>(take(size_t(region_cap) * 4));
	P.father_of = reinterpret_cast<int *>(take(size_t(region_cap) * 4));
	P.chunk_cnt = reinterpret_cast<long long *>(take(size_t(n_chunks) * 8));
	P.father_ridx = reinterpret_cast<long long *>(take(size_t(window) * 8));
	P.child_off = reinterpret_cast<long long *>(take(size_t(window + 1) * 8));
	P.father_side = reinterpret_cast<int *>(take(size_t(window) * 4));
	P.father_kept = reinterpret_cast<int *>(take(size_t(window) * 4));
	P.father_npr = reinterpret_cast<int *>(take(size_t(window) * 4));
	P.kept_before = reinterpret_cast<long long *>(take(size_t(window + 1) * 8));
	P.child_rec = take(size_t(child_cap) * S);
	P.child_lb = reinterpret_cast<int32_t *>(take(size_t(child_cap) * 4));
	P.child_job = reinterpret_cast<int16_t *>(take(size_t(child_cap) * 2));
	P.child_rank = reinterpret_cast<int32_t *>(take(size_t(child_cap) * 4));
	P.best_rec = take(size_t(S));
	P.cap = cap;
	P.region_cap = region_cap;
	P.child_cap = child_cap;
	P.window = window;
	P.n_chunks = n_chunks;
	P.n = n;
	P.stride = S;
	return off;
}

}  // namespace
}  // namespace wsbb
