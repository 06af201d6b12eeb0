// Exact begin-end DFS search, GPU-resident (wsbb_explore).
//
// The reference explores one node at a time: take the node with the
// smallest rank path (src/tree.cpp:37-46, 257-266); a leaf may improve the
// incumbent (src/solutions.cpp:45-65); a node whose bound is not below the
// incumbent is pruned; otherwise both sides of children are generated and
// bounded, the side is chosen (src/decompose_beginend.cpp:39-68) and the
// chosen children are inserted with their ranks (src/problems.cpp:46-62).
// The incumbent only changes at leaves, and only downwards, so a node's
// fate depends on the incumbent at the moment the sequential search would
// take it.
//
// Here the whole DFS stack lives in HBM, sorted by rank path (index 0 is
// the bottom, the top entry is the next node the sequential search takes).
// Every iteration is four stream-ordered kernels:
//
//   commit_select (1 CTA)  Commit, in DFS order, everything already decided
//                          at the top of the stack: leaves (incumbent
//                          updates), pruned markers, and markers of nodes
//                          that were branched ahead of their turn — each
//                          re-checked against the incumbent the sequential
//                          search would have at that point; a marker that
//                          fails is counted as pruned and its speculative
//                          subtree (contiguous just below it) is dropped.
//                          Then select the next `window` unprocessed nodes
//                          below the top: bound >= incumbent marks them
//                          pruned (final: the incumbent only decreases),
//                          the others become this iteration's fathers.
//   make_children          Copy the rewrite region aside and write every
//                          father's 2u children (both sides) or 2 leaves
//                          as pool records (create_raw_problem3,
//                          src/bb_problem_calculator.cpp:25-79).
//   lb2_pool_kernel        Bound the children (bound_kernels.cu).
//   emit                   Per father: side choice, ranks, and the
//                          rewritten region — chosen children (worst rank
//                          lowest) under a BRANCHED marker that keeps the
//                          father's bound for its commit-time check.
//
// Node counts, the incumbent trace and the optimum therefore equal the
// sequential search's exactly; work spent on markers that later fail is
// reported separately (evaluated vs bounded, discarded). No kernel waits
// on another CTA, so nothing can spin; an iteration cap and a capacity
// check end the search with a status instead.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include "wsbb_internal.h"

namespace wsbb {
namespace {

enum : uint8_t { ST_UNPROC = 0, ST_LEAF = 1, ST_PRUNED = 2, ST_BRANCHED = 3 };

struct Meta {
	int32_t lb;
	int16_t depth;
	uint8_t state;
	uint8_t pad;
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
	unsigned long long branched, pruned, leaves, improved, bounded;
	unsigned long long evaluated, discarded;
	unsigned long long hist[WSBB_MAX_JOBS + 1];
};

struct ExParams {
	ExDev *dev;
	uint8_t *rec;           // stack records [cap][stride]
	Meta *meta;             // stack meta [cap]
	uint8_t *tmp_rec;       // region copy [region_cap][stride]
	Meta *tmp_meta;         // [region_cap]
	long long *slot_from_top; // [region_cap] slots above the entry after rewrite
	int *father_of;         // [region_cap] father ordinal or -1
	long long *father_ridx; // [window] region index of each father
	long long *child_off;   // [window + 1] first child record of each father
	uint8_t *child_rec;     // [child_cap][stride]
	int32_t *child_lb;      // [child_cap]
	int16_t *child_job;     // [child_cap] job moved by the branching
	uint8_t *best_rec;      // [stride] incumbent permutation record
	long long cap, region_cap, child_cap;
	int window;
	int n, stride;
};

constexpr int kSelThreads = 1024;

__device__ __forceinline__ int children_of_depth(int depth, int n)
{
	// a non-leaf at depth d has n - d free jobs (a simple node: 2 leaves)
	return depth == n - 2 ? 2 : 2 * (n - depth);
}

__device__ __forceinline__ int kept_of_depth(int depth, int n)
{
	return depth == n - 2 ? 2 : (n - depth);
}

// Block-wide scans for kSelThreads threads. `scratch` holds 32 values.
template <typename T, typename Op>
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
	__syncthreads();
	if (warp == 0) {
		T w = lane < (kSelThreads / 32) ? scratch[lane] : identity;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			T y = __shfl_up_sync(0xffffffffu, w, d);
			if (lane >= d)
				w = op(w, y);
		}
		scratch[lane] = w; // inclusive over warps
	}
	__syncthreads();
	T warp_prefix = warp == 0 ? identity : scratch[warp - 1];
	T incl = op(warp_prefix, x);
	T excl_in_warp = __shfl_up_sync(0xffffffffu, x, 1);
	T excl = lane == 0 ? warp_prefix : op(warp_prefix, excl_in_warp);
	if (total)
		*total = scratch[kSelThreads / 32 - 1];
	__syncthreads();
	(void)incl;
	return excl;
}

template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T identity, T *scratch)
{
	T total;
	block_excl_scan(v, op, identity, scratch, &total);
	return total;
}

struct MinOp {
	__device__ int operator()(int a, int b) const { return a < b ? a : b; }
};
struct SumOp {
	__device__ long long operator()(long long a, long long b) const { return a + b; }
};
struct MaxOp {
	__device__ int operator()(int a, int b) const { return a > b ? a : b; }
};

__global__ void __launch_bounds__(kSelThreads) commit_select_kernel(ExParams P)
{
	__shared__ int s_int[32];
	__shared__ long long s_ll[32];
	__shared__ unsigned long long s_cnt[5];
	__shared__ unsigned long long s_hist[WSBB_MAX_JOBS + 1];
	ExDev *D = P.dev;
	if (D->done || D->error)
		return;
	const int t = threadIdx.x;
	const int n = P.n;
	if (t < 5)
		s_cnt[t] = 0;
	for (int i = t; i <= n; i += kSelThreads)
		s_hist[i] = 0;
	__syncthreads();

	long long top = D->top;
	int ub = D->ub;

	// ---- commit -------------------------------------------------------
	while (top >= 0) {
		const long long idx = top - t;
		Meta e = {INT_MAX, 0, ST_UNPROC, 0};
		if (idx >= 0)
			e = P.meta[idx];
		const int leaf_cost = (idx >= 0 && e.state == ST_LEAF) ? e.lb : INT_MAX;
		const int ub_before = min(ub, block_excl_scan(leaf_cost, MinOp(), INT_MAX, s_int,
		                                              (int *)nullptr));
		const bool stop = idx < 0 || e.state == ST_UNPROC ||
		                  (e.state == ST_BRANCHED && e.lb >= ub_before);
		const int s = block_reduce(stop ? t : kSelThreads, MinOp(), kSelThreads, s_int);
		if (t < s) {
			if (e.state == ST_BRANCHED) {
				atomicAdd(&s_cnt[0], 1ull);
				atomicAdd(&s_cnt[4], (unsigned long long)children_of_depth(e.depth, n));
			} else if (e.state == ST_PRUNED) {
				atomicAdd(&s_cnt[1], 1ull);
				atomicAdd(&s_hist[e.depth], 1ull);
			} else { // leaf
				atomicAdd(&s_cnt[2], 1ull);
				atomicAdd(&s_hist[n], 1ull);
				if (e.lb < ub_before)
					atomicAdd(&s_cnt[3], 1ull);
			}
		}
		const int chunk_min = block_reduce(t < s ? leaf_cost : INT_MAX, MinOp(), INT_MAX, s_int);
		if (chunk_min < ub) {
			// the first leaf reaching the new minimum is the one that set it
			const int first = block_reduce((t < s && leaf_cost == chunk_min) ? t : kSelThreads,
			                               MinOp(), kSelThreads, s_int);
			const long long src = top - first;
			for (int b = t; b < P.stride; b += kSelThreads)
				P.best_rec[b] = P.rec[src * P.stride + b];
			ub = chunk_min;
		}
		top -= s;
		if (s == kSelThreads)
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
			s_cnt[1] += 1;
			s_hist[stopper.depth] += 1;
		}
		__syncthreads();
		top -= 1;
		while (top >= 0) {
			const long long j = top - t;
			const bool out = j < 0 || P.meta[j].depth <= stopper.depth;
			const int s2 = block_reduce(out ? t : kSelThreads, MinOp(), kSelThreads, s_int);
			if (t == 0)
				D->discarded += (unsigned long long)s2;
			top -= s2;
			if (s2 < kSelThreads)
				break;
		}
	}

	// ---- select -------------------------------------------------------
	long long nf = 0, region = 0, slots = 0, nchild = 0;
	const long long scan_limit = P.region_cap;
	while (nf < P.window && top - region >= 0 && region < scan_limit) {
		const long long ridx = region + t;
		const long long idx = top - ridx;
		const bool valid = idx >= 0 && ridx < scan_limit;
		Meta e = {0, 0, ST_LEAF, 0};
		if (valid)
			e = P.meta[idx];
		const bool unproc = valid && e.state == ST_UNPROC;
		if (unproc && e.lb >= ub) {
			P.meta[idx].state = ST_PRUNED; // final: the incumbent only decreases
			e.state = ST_PRUNED;
		}
		const bool cand = unproc && e.lb < ub;
		long long ncand_chunk;
		const long long before = block_excl_scan<long long>(cand ? 1 : 0, SumOp(), 0ll, s_ll,
		                                                    &ncand_chunk);
		const bool take = cand && nf + before < P.window;
		// the region ends at the last father taken, or at the chunk's end
		int last;
		if (nf + ncand_chunk >= P.window)
			last = block_reduce((cand && nf + before == P.window - 1) ? t : -1, MaxOp(), -1,
			                    s_int);
		else
			last = block_reduce(valid ? t : -1, MaxOp(), -1, s_int);
		const bool in_region = t <= last;
		const long long my_slots =
		    in_region ? (take ? 1 + kept_of_depth(e.depth, n) : 1) : 0;
		long long chunk_slots;
		const long long slot_before =
		    block_excl_scan<long long>(my_slots, SumOp(), 0ll, s_ll, &chunk_slots);
		const long long my_children = take ? children_of_depth(e.depth, n) : 0;
		long long chunk_children;
		const long long child_before =
		    block_excl_scan<long long>(my_children, SumOp(), 0ll, s_ll, &chunk_children);
		if (in_region) {
			P.slot_from_top[ridx] = slots + slot_before;
			P.father_of[ridx] = take ? int(nf + before) : -1;
			if (take) {
				P.father_ridx[nf + before] = ridx;
				P.child_off[nf + before] = nchild + child_before;
			}
		}
		const long long taken = min(ncand_chunk, (long long)P.window - nf);
		nf += taken;
		slots += chunk_slots;
		nchild += chunk_children;
		region += last + 1;
		if (last + 1 < kSelThreads && nf < P.window)
			break; // reached the bottom of the stack
	}

	const long long new_top = top - region + slots;
	if (t == 0) {
		P.child_off[nf] = nchild;
		if (nf > 0 && (new_top >= P.cap || nchild > P.child_cap)) {
			D->error = WSBB_ERR_CAPACITY;
		}
		D->branched += s_cnt[0];
		D->pruned += s_cnt[1];
		D->leaves += s_cnt[2];
		D->improved += s_cnt[3];
		D->bounded += s_cnt[4];
		D->ub = ub;
		D->top = top;
		D->region_len = nf > 0 ? region : 0;
		D->region_slots = nf > 0 ? slots : 0;
		D->n_fathers = nf;
		D->n_children = nf > 0 ? nchild : 0;
		D->evaluated += nf > 0 ? nchild : 0;
		D->iterations += 1;
		if (top < 0)
			D->done = 1;
	}
	for (int i = t; i <= n; i += kSelThreads)
		if (s_hist[i])
			D->hist[i] += s_hist[i];
}

// Copy the region aside and write every father's child records.
__global__ void make_children_kernel(ExParams P)
{
	ExDev *D = P.dev;
	if (D->done || D->error || D->n_fathers == 0)
		return;
	const long long top = D->top, rlen = D->region_len, nf = D->n_fathers;
	const int S = P.stride, n = P.n;
	const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	const long long gsz = (long long)gridDim.x * blockDim.x;
	// region copy, 16 bytes per thread step
	const long long words = rlen * (S / 16);
	for (long long w = gtid; w < words; w += gsz) {
		const long long r = w / (S / 16), c = w % (S / 16);
		reinterpret_cast<uint4 *>(P.tmp_rec + r * S)[c] =
		    reinterpret_cast<const uint4 *>(P.rec + (top - r) * S)[c];
	}
	for (long long r = gtid; r < rlen; r += gsz)
		P.tmp_meta[r] = P.meta[top - r];
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

// Per father: choise, ranks, and the rewritten region. One warp per region
// entry; non-father entries are moved to their new slots.
__global__ void emit_kernel(ExParams P)
{
	ExDev *D = P.dev;
	if (D->done || D->error || D->n_fathers == 0)
		return;
	const int lane = threadIdx.x & 31;
	const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
	const int S = P.stride, n = P.n;
	const long long rlen = D->region_len;
	const long long new_top = D->top - rlen + D->region_slots;
	const int ub = D->ub, best = D->best;
	for (long long r = warp; r < rlen; r += nwarps) {
		const long long hi_slot = new_top - P.slot_from_top[r]; // top slot of this block
		const int f = P.father_of[r];
		const uint4 *src = reinterpret_cast<const uint4 *>(P.tmp_rec + r * S);
		if (f < 0) {
			for (int c = lane; c < S / 16; c += 32)
				reinterpret_cast<uint4 *>(P.rec + hi_slot * S)[c] = src[c];
			if (lane == 0)
				P.meta[hi_slot] = P.tmp_meta[r];
			continue;
		}
		const Meta fm = P.tmp_meta[r];
		const long long c0 = P.child_off[f];
		const int nc = int(P.child_off[f + 1] - c0);
		const bool simple = fm.depth == n - 2;
		const int kept = simple ? 2 : nc / 2;
		int side_off = 0;
		if (!simple) {
			// choise: more children >= best wins; else the larger sum of the
			// bounds below best; ties go to the END side
			long long sum[2] = {0, 0};
			int cut[2] = {0, 0};
			for (int k = lane; k < nc; k += 32) {
				const int lb = P.child_lb[c0 + k];
				const int sd = k >= kept;
				if (lb >= best)
					cut[sd]++;
				else
					sum[sd] += lb;
			}
#pragma unroll
			for (int d = 16; d > 0; d >>= 1) {
				sum[0] += __shfl_xor_sync(0xffffffffu, sum[0], d);
				sum[1] += __shfl_xor_sync(0xffffffffu, sum[1], d);
				cut[0] += __shfl_xor_sync(0xffffffffu, cut[0], d);
				cut[1] += __shfl_xor_sync(0xffffffffu, cut[1], d);
			}
			bool begin;
			if (cut[0] != cut[1])
				begin = cut[0] > cut[1];
			else
				begin = sum[0] > sum[1];
			side_off = begin ? 0 : kept;
		}
		// ranks: 0 = smallest bound, ties to the smaller job; rank 0 sits
		// right under the marker
		for (int k = lane; k < kept; k += 32) {
			const long long ck = c0 + side_off + k;
			const int lb = P.child_lb[ck];
			const int job = P.child_job[ck];
			int rank = 0;
			for (int q = 0; q < kept; ++q) {
				const int lq = P.child_lb[c0 + side_off + q];
				const int jq = P.child_job[c0 + side_off + q];
				rank += (lq < lb) || (lq == lb && jq < job);
			}
			const long long slot = hi_slot - 1 - rank;
			const uint4 *cs = reinterpret_cast<const uint4 *>(P.child_rec + ck * S);
			uint4 *dst = reinterpret_cast<uint4 *>(P.rec + slot * S);
			for (int c = 0; c < S / 16; ++c)
				dst[c] = cs[c];
			Meta cm;
			cm.lb = lb;
			cm.depth = int16_t(simple ? n : fm.depth + 1);
			cm.state = simple ? ST_LEAF : (lb >= ub ? ST_PRUNED : ST_UNPROC);
			cm.pad = 0;
			P.meta[slot] = cm;
		}
		for (int c = lane; c < S / 16; c += 32)
			reinterpret_cast<uint4 *>(P.rec + hi_slot * S)[c] = src[c];
		if (lane == 0) {
			Meta mm = fm;
			mm.state = ST_BRANCHED;
			P.meta[hi_slot] = mm;
		}
	}
	__syncthreads();
}

__global__ void finish_iteration_kernel(ExParams P)
{
	ExDev *D = P.dev;
	if (D->done || D->error || D->n_fathers == 0)
		return;
	D->top = D->top - D->region_len + D->region_slots;
	D->n_fathers = 0;
	D->n_children = 0;
}

__global__ void init_kernel(ExParams P, int ub0, int best)
{
	ExDev *D = P.dev;
	const int n = P.n, S = P.stride;
	if (threadIdx.x == 0) {
		memset(D, 0, sizeof(ExDev));
		D->top = 0;
		D->ub = ub0;
		D->best = best;
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

}  // namespace
}  // namespace wsbb

struct ExploreState {
	wsbb::ExParams P{};
	wsbb::BoundParams child_bp{};
	size_t bytes = 0;
	void *mem = nullptr;
	long long cap = 0, region_cap = 0, child_cap = 0;
	int window = 0;
	cudaGraphExec_t graph = nullptr;
	cudaStream_t graph_stream = nullptr;
	int graph_iters = 0;
};

void wsbb_explore_release(wsbb_ctx *ctx)
{
	if (!ctx || !ctx->ex)
		return;
	if (ctx->ex->graph)
		cudaGraphExecDestroy(ctx->ex->graph);
	if (ctx->ex->mem)
		cudaFree(ctx->ex->mem);
	delete ctx->ex;
	ctx->ex = nullptr;
}

namespace {

int ex_fail(wsbb_ctx *ctx, cudaError_t e, const char *what)
{
	return wsbb_set_error(ctx, WSBB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// One iteration: four stream-ordered launches (captured into a graph).
cudaError_t enqueue_iteration(wsbb_ctx *ctx, ExploreState &X, cudaStream_t s)
{
	using namespace wsbb;
	commit_select_kernel<<<1, kSelThreads, 0, s>>>(X.P);
	const int grid = ctx->num_sms * 4;
	make_children_kernel<<<grid, 256, 0, s>>>(X.P);
	cudaError_t e = launch_pool_bounds(X.child_bp, X.P.child_rec, X.child_cap, X.P.child_lb, 0,
	                                   ctx->num_sms, s);
	if (e != cudaSuccess)
		return e;
	emit_kernel<<<grid, 256, 0, s>>>(X.P);
	finish_iteration_kernel<<<1, 32, 0, s>>>(X.P);
	return cudaGetLastError();
}

}  // namespace

extern "C" int wsbb_explore(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, wsbb_stats *st,
                            void *stream_v)
{
	using namespace wsbb;
	if (!ctx || !cfg || !st)
		return WSBB_ERR_ARG;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	const int n = ctx->inst.n;
	const int window = cfg->window > 0 ? cfg->window : 4096;
	const long long cap = cfg->capacity > 0 ? cfg->capacity : (1ll << 22);
	const long long region_cap = 4ll * window + 4096;
	const long long child_cap = (long long)window * 2 * n;
	const int S = ctx->bp.stride;
	if (window > (1 << 20) || cap < region_cap)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "window / capacity out of range");

	ExploreState *X = ctx->ex;
	if (!X || X->cap != cap || X->window != window) {
		wsbb_explore_release(ctx);
		X = new ExploreState();
		X->cap = cap;
		X->region_cap = region_cap;
		X->child_cap = child_cap;
		X->window = window;
		auto a16 = [](size_t v) { return (v + 255) & ~size_t(255); };
		size_t off = 0;
		const size_t o_dev = off; off = a16(off + sizeof(ExDev));
		const size_t o_rec = off; off = a16(off + size_t(cap) * S);
		const size_t o_meta = off; off = a16(off + size_t(cap) * sizeof(Meta));
		const size_t o_trec = off; off = a16(off + size_t(region_cap) * S);
		const size_t o_tmeta = off; off = a16(off + size_t(region_cap) * sizeof(Meta));
		const size_t o_sft = off; off = a16(off + size_t(region_cap) * 8);
		const size_t o_fof = off; off = a16(off + size_t(region_cap) * 4);
		const size_t o_fr = off; off = a16(off + size_t(window) * 8);
		const size_t o_co = off; off = a16(off + size_t(window + 1) * 8);
		const size_t o_crec = off; off = a16(off + size_t(child_cap) * S);
		const size_t o_clb = off; off = a16(off + size_t(child_cap) * 4);
		const size_t o_cjob = off; off = a16(off + size_t(child_cap) * 2);
		const size_t o_best = off; off = a16(off + size_t(S));
		X->bytes = off;
		e = cudaMalloc(&X->mem, X->bytes);
		if (e != cudaSuccess) {
			delete X;
			return wsbb_set_error(ctx, WSBB_ERR_NOMEM, "search pool allocation failed");
		}
		uint8_t *b = static_cast<uint8_t *>(X->mem);
		ExParams &P = X->P;
		P.dev = reinterpret_cast<ExDev *>(b + o_dev);
		P.rec = b + o_rec;
		P.meta = reinterpret_cast<Meta *>(b + o_meta);
		P.tmp_rec = b + o_trec;
		P.tmp_meta = reinterpret_cast<Meta *>(b + o_tmeta);
		P.slot_from_top = reinterpret_cast<long long *>(b + o_sft);
		P.father_of = reinterpret_cast<int *>(b + o_fof);
		P.father_ridx = reinterpret_cast<long long *>(b + o_fr);
		P.child_off = reinterpret_cast<long long *>(b + o_co);
		P.child_rec = b + o_crec;
		P.child_lb = reinterpret_cast<int32_t *>(b + o_clb);
		P.child_job = reinterpret_cast<int16_t *>(b + o_cjob);
		P.best_rec = b + o_best;
		P.cap = cap;
		P.region_cap = region_cap;
		P.child_cap = child_cap;
		P.window = window;
		P.n = n;
		P.stride = S;
		X->child_bp = ctx->bp;
		X->child_bp.count_dev = &P.dev->n_children;
		ctx->ex = X;
	}

	cudaStream_t s = stream_v ? static_cast<cudaStream_t>(stream_v) : ctx->stream;
	const int ub0 = cfg->ub0;
	const int best = cfg->best;
	init_kernel<<<1, 128, 0, s>>>(X->P, ub0, best);
	e = cudaGetLastError();
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search init");

	const int G = cfg->graph_iters > 0 ? cfg->graph_iters : 16;
	const bool use_graph = !(cfg->flags & WSBB_EXPLORE_NO_GRAPH);
	if (use_graph && (!X->graph || X->graph_iters != G || X->graph_stream != s)) {
		if (X->graph)
			cudaGraphExecDestroy(X->graph);
		X->graph = nullptr;
		cudaGraph_t g;
		e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
		if (e != cudaSuccess)
			return ex_fail(ctx, e, "graph capture");
		for (int i = 0; i < G && e == cudaSuccess; ++i)
			e = enqueue_iteration(ctx, *X, s);
		cudaError_t e2 = cudaStreamEndCapture(s, &g);
		if (e != cudaSuccess || e2 != cudaSuccess)
			return ex_fail(ctx, e != cudaSuccess ? e : e2, "graph capture");
		e = cudaGraphInstantiate(&X->graph, g, 0);
		cudaGraphDestroy(g);
		if (e != cudaSuccess)
			return ex_fail(ctx, e, "graph instantiate");
		X->graph_iters = G;
		X->graph_stream = s;
	}

	cudaEvent_t ev0, ev1;
	cudaEventCreate(&ev0);
	cudaEventCreate(&ev1);
	cudaEventRecord(ev0, s);
	ExDev h{};
	long long launched = 0;
	const long long max_iters = cfg->max_iters > 0 ? cfg->max_iters : LLONG_MAX;
	int status = 0;
	for (;;) {
		if (use_graph) {
			e = cudaGraphLaunch(X->graph, s);
			launched += G;
		} else {
			for (int i = 0; i < G && e == cudaSuccess; ++i)
				e = enqueue_iteration(ctx, *X, s);
			launched += G;
		}
		if (e != cudaSuccess)
			break;
		e = cudaMemcpyAsync(&h, X->P.dev, sizeof(ExDev), cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(s);
		if (e != cudaSuccess || h.done || h.error)
			break;
		if (launched >= max_iters) {
			status = 1;
			break;
		}
	}
	cudaEventRecord(ev1, s);
	cudaEventSynchronize(ev1);
	float ms = 0;
	cudaEventElapsedTime(&ms, ev0, ev1);
	cudaEventDestroy(ev0);
	cudaEventDestroy(ev1);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search");
	std::vector<int16_t> best_rec(S / 2);
	e = cudaMemcpy(best_rec.data(), X->P.best_rec, S, cudaMemcpyDeviceToHost);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "incumbent download");

	std::memset(st, 0, sizeof(*st));
	st->branched = (int64_t)h.branched;
	st->pruned = (int64_t)h.pruned;
	st->leaves = (int64_t)h.leaves;
	st->improved = (int64_t)h.improved;
	st->bounded = (int64_t)h.bounded;
	st->evaluated = (int64_t)h.evaluated;
	st->discarded = (int64_t)h.discarded;
	st->iterations = (int64_t)h.iterations;
	st->best_cost = h.ub;
	st->status = h.error ? h.error : status;
	for (int d = 0; d <= n; ++d)
		st->depth_hist[d] = h.hist[d];
	for (int j = 0; j < n; ++j)
		st->best_perm[j] = best_rec[j];
	st->seconds = ms * 1e-3;
	if (h.error)
		return wsbb_set_error(ctx, h.error, "search pool capacity exceeded");
	return WSBB_OK;
}

// ---------------------------------------------------------------------------
// wsbb_explore_noalloc: the search above with its whole state in one fixed
// file-scope device array instead of memory it allocates, for callers that
// must not allocate GPU memory. The kernels are the same; only where their
// buffers live differs.

namespace {

__device__ __align__(256) uint8_t g_noalloc_scratch[WSBB_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch, looked up once per device. In host
// code the symbol itself is only a host-side stand-in, never a device
// address, so it is never handed to a kernel directly.
std::mutex g_noalloc_mu;
void *g_noalloc_addr[64];

int noalloc_scratch(wsbb_ctx *ctx, uint8_t **out)
{
	if (ctx->device < 0 || ctx->device >= 64)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "device ordinal out of range");
	std::lock_guard<std::mutex> lock(g_noalloc_mu);
	if (!g_noalloc_addr[ctx->device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p)
			return ex_fail(ctx, e != cudaSuccess ? e : cudaErrorInvalidSymbol,
			               "cudaGetSymbolAddress(no-alloc scratch)");
		g_noalloc_addr[ctx->device] = p;
	}
	*out = static_cast<uint8_t *>(g_noalloc_addr[ctx->device]);
	return WSBB_OK;
}

// Lays the search buffers out from `base` (null: only sizes them).
size_t noalloc_layout(uint8_t *base, long long cap, int window, int n, int S,
                      wsbb::ExParams &P)
{
	using wsbb::ExDev;
	using wsbb::Meta;
	const long long region_cap = 4ll * window + 4096;
	const long long child_cap = (long long)window * 2 * n;
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
	P.slot_from_top = reinterpret_cast<long long *>(take(size_t(region_cap) * 8));
	P.father_of = reinterpret_cast<int *>(take(size_t(region_cap) * 4));
	P.father_ridx = reinterpret_cast<long long *>(take(size_t(window) * 8));
	P.child_off = reinterpret_cast<long long *>(take(size_t(window + 1) * 8));
	P.child_rec = take(size_t(child_cap) * S);
	P.child_lb = reinterpret_cast<int32_t *>(take(size_t(child_cap) * 4));
	P.child_job = reinterpret_cast<int16_t *>(take(size_t(child_cap) * 2));
	P.best_rec = take(size_t(S));
	P.cap = cap;
	P.region_cap = region_cap;
	P.child_cap = child_cap;
	P.window = window;
	P.n = n;
	P.stride = S;
	return off;
}

}  // namespace

extern "C" int wsbb_explore_noalloc(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg,
                                    wsbb_stats *st, void *stream_v)
{
	using namespace wsbb;
	if (!ctx || !cfg || !st)
		return WSBB_ERR_ARG;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	uint8_t *scratch = nullptr;
	int rc = noalloc_scratch(ctx, &scratch);
	if (rc != WSBB_OK)
		return rc;

	const int n = ctx->inst.n;
	const int S = ctx->bp.stride;
	const int window = cfg->window > 0 ? cfg->window : 1024;
	const size_t limit = WSBB_NOALLOC_SCRATCH_BYTES;
	ExploreState X; // host-side view only: no graph, no allocation
	if (window > (1 << 20))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "window out of range");
	long long cap = cfg->capacity;
	if (cap <= 0) {
		const size_t fixed = noalloc_layout(nullptr, 0, window, n, S, X.P);
		cap = fixed < limit ? (long long)((limit - fixed) / (S + sizeof(Meta))) : 0;
		while (cap > 0 && noalloc_layout(nullptr, cap, window, n, S, X.P) > limit)
			cap -= 256;
	}
	const long long region_cap = 4ll * window + 4096;
	if (cap < region_cap || noalloc_layout(nullptr, cap, window, n, S, X.P) > limit)
		return wsbb_set_error(ctx, WSBB_ERR_CAPACITY,
		                      "window / capacity do not fit the fixed no-alloc scratch of " +
		                          std::to_string(limit >> 20) + " MiB");
	noalloc_layout(scratch, cap, window, n, S, X.P);
	X.cap = cap;
	X.region_cap = region_cap;
	X.child_cap = X.P.child_cap;
	X.window = window;
	X.child_bp = ctx->bp;
	X.child_bp.count_dev = &X.P.dev->n_children;

	cudaStream_t s = stream_v ? static_cast<cudaStream_t>(stream_v) : ctx->stream;
	const auto t0 = std::chrono::steady_clock::now();
	init_kernel<<<1, 128, 0, s>>>(X.P, cfg->ub0, cfg->best);
	e = cudaGetLastError();
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search init");
	const int G = cfg->graph_iters > 0 ? cfg->graph_iters : 16;
	const long long max_iters = cfg->max_iters > 0 ? cfg->max_iters : LLONG_MAX;
	ExDev h{};
	long long launched = 0;
	int status = 0;
	for (;;) {
		for (int i = 0; i < G && e == cudaSuccess; ++i)
			e = enqueue_iteration(ctx, X, s);
		launched += G;
		if (e != cudaSuccess)
			break;
		e = cudaMemcpyAsync(&h, X.P.dev, sizeof(ExDev), cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(s);
		if (e != cudaSuccess || h.done || h.error)
			break;
		if (launched >= max_iters) {
			status = 1;
			break;
		}
	}
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "no-alloc search");
	int16_t best_rec[WSBB_MAX_JOBS + 8];
	e = cudaMemcpyAsync(best_rec, X.P.best_rec, S, cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "incumbent download");
	const double secs =
	    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

	std::memset(st, 0, sizeof(*st));
	st->branched = (int64_t)h.branched;
	st->pruned = (int64_t)h.pruned;
	st->leaves = (int64_t)h.leaves;
	st->improved = (int64_t)h.improved;
	st->bounded = (int64_t)h.bounded;
	st->evaluated = (int64_t)h.evaluated;
	st->discarded = (int64_t)h.discarded;
	st->iterations = (int64_t)h.iterations;
	st->best_cost = h.ub;
	st->status = h.error ? h.error : status;
	for (int d = 0; d <= n; ++d)
		st->depth_hist[d] = h.hist[d];
	for (int j = 0; j < n; ++j)
		st->best_perm[j] = best_rec[j];
	st->seconds = secs;
	if (h.error)
		return wsbb_set_error(ctx, h.error, "search outgrew the no-alloc scratch capacity");
	return WSBB_OK;
}
