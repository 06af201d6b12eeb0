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
// Every iteration is a fixed sequence of stream-ordered kernels (replayed
// from a CUDA graph):
//
//   commit (1 CTA)      Commit, in DFS order, everything already decided at
//                       the top of the stack: leaves (incumbent updates),
//                       pruned entries, and markers of nodes that were
//                       branched ahead of their turn — each re-checked
//                       against the incumbent the sequential search holds at
//                       that point; a marker that fails is counted as pruned
//                       and its speculative subtree (contiguous just below
//                       it) is dropped.
//   doom (1 warp)       Only after the incumbent improved: walk the top of
//                       the stack and settle markers that the new incumbent
//                       already condemns — the sequential search will prune
//                       them whenever it reaches them, since the incumbent
//                       never increases — so their subtrees are marked dead
//                       and never expanded further.
//   select (3 kernels)  Count the unprocessed nodes of the top region and
//                       their children per chunk (bound >= incumbent prunes
//                       them, final), plan the first `window` of them, and
//                       mark those fathers with their first child's offset.
//   make_children       Copy the rewrite region aside and write every
//                       father's 2u children (both sides) or 2 leaves as pool
//                       records (create_raw_problem3,
//                       src/bb_problem_calculator.cpp:25-79).
//   lb2 pool kernel     Bound the children (bound_kernels.cu).
//   choose              Per father: side choice with threshold `best`, ranks
//                       of the kept side by (bound, job), and how many of
//                       them the incumbent already prunes.
//   kept scan           Block sizes of the fathers in the rewritten region.
//   emit                Scatter: the chosen children still open (their lowest
//                       ranks) under a BRANCHED marker that keeps the
//                       father's bound for its commit-time check and the
//                       count of its children pruned at birth (the highest
//                       ranks, which never need an entry); other region
//                       entries move to their new slots.
//
// Counts are only taken at commit, in the sequential order, so node counts,
// the incumbent trace and the optimum equal the sequential search's
// exactly; work on markers that later fail is reported separately
// (evaluated vs bounded, discarded). The number of fathers per iteration
// adapts: it drops to its minimum when the incumbent improves (speculation
// made then is the kind that gets discarded) and doubles while it does not.
// No kernel waits on another CTA, so nothing can spin; an iteration cap and
// a capacity check end the search with a status instead.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <string>

#include "search_host.h"

void wsbb_explore_release(wsbb_ctx *ctx)
{
	if (!ctx || !ctx->ex)
		return;
	if (ctx->ex->graph)
		cudaGraphExecDestroy(ctx->ex->graph);
	if (ctx->ex->mem)
		cudaFree(ctx->ex->mem);
	if (ctx->ex->learned_mem)
		cudaFree(ctx->ex->learned_mem);
	delete ctx->ex;
	ctx->ex = nullptr;
}

namespace wsbb {
namespace host {

int ex_fail(wsbb_ctx *ctx, cudaError_t e, const char *what)
{
	return wsbb_set_error(ctx, WSBB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// One iteration: a fixed sequence of stream-ordered launches (captured
// into a graph). The learned mode bounds children in two steps (K ranked
// pairs for all, full LB2 for the ones left open); the logging mode copies
// a sample of the children out before bounding them.
cudaError_t enqueue_iteration(wsbb_ctx *ctx, ExploreState &X, cudaStream_t s)
{
	using namespace wsbb;
	const int grid = ctx->num_sms * 4;
	const int sel_grid = std::min(X.P.n_chunks, ctx->num_sms * 8);
	commit_kernel<<<1, kSelThreads, 0, s>>>(X.P);
	doom_kernel<<<1, 32, 0, s>>>(X.P);
	select_count_kernel<<<sel_grid, kSelCtaThreads, 0, s>>>(X.P);
	select_plan_kernel<<<1, kSelThreads, 0, s>>>(X.P);
	select_write_kernel<<<sel_grid, kSelCtaThreads, 0, s>>>(X.P);
	make_children_kernel<<<grid, 256, 0, s>>>(X.P, X.mode == 2 || X.child_lb2);
	cudaError_t e = cudaSuccess;
	if (X.mode == 1) {
		father_features_kernel<<<grid, 128, 0, s>>>(X.P, ctx->bp);
		e = launch_mlp_topk(X.model, X.P.feat, X.window, &X.P.dev->n_fathers, X.P.K, X.P.fpairs,
		                    nullptr, ctx->num_sms, s);
		if (e != cudaSuccess)
			return e;
		if (X.child_lb2) {
			// per child: the K ranked pairs, then full LB2 for the children
			// they do not settle
			const size_t smem = size_t(ctx->bp.t8.bytes) +
			                    size_t(kPartialThreads / 32) * 2 * 20 * 32 * 4;
			auto kern = ctx->bp.m <= 8
			                ? partial_kernel<8>
			                : (ctx->bp.m <= 16 ? partial_kernel<16> : partial_kernel<20>);
			e = allow_max_dynamic_smem(kern);
			if (e != cudaSuccess)
				return e;
			kern<<<ctx->num_sms, kPartialThreads, smem, s>>>(X.P, ctx->bp);
			BoundParams gbp = X.child_bp;
			gbp.count_dev = &X.P.dev->n_unsettled;
			gbp.gather = X.P.unsettled;
			e = launch_pool_bounds(gbp, X.P.child_rec, X.child_cap, X.P.child_lb, 0,
			                       ctx->num_sms, s);
		} else {
			FamilyArgs fa;
			fa.fathers = X.P.tmp_rec;
			fa.ridx = X.P.father_ridx;
			fa.count_dev = &X.P.dev->n_fathers;
			fa.child_off = X.P.child_off;
			fa.child_lb = X.P.child_lb;
			fa.child_job = X.P.child_job;
			fa.stride = X.P.stride;
			fa.next = &X.P.dev->fam_next;
			fa.fpairs = X.P.fpairs;
			fa.K = X.P.K;
			fa.ub_dev = &X.P.dev->ub;
			fa.best_dev = &X.P.dev->best;
			fa.early = &X.P.dev->early;
			fa.settled_fathers = &X.P.dev->settled_fathers;
			e = launch_family_lb2(ctx->bp, ctx->tables, fa, X.window, ctx->num_sms,
			                      s, X.fam_kb);
		}
	} else {
		if (X.mode == 2)
			log_kernel<<<grid, 256, 0, s>>>(X.P);
		if (X.child_lb2) {
			e = launch_pool_bounds(X.child_bp, X.P.child_rec, X.child_cap, X.P.child_lb, 0,
			                       ctx->num_sms, s);
		} else {
			FamilyArgs fa;
			fa.fathers = X.P.tmp_rec;
			fa.ridx = X.P.father_ridx;
			fa.count_dev = &X.P.dev->n_fathers;
			fa.child_off = X.P.child_off;
			fa.child_lb = X.P.child_lb;
			fa.child_job = X.P.child_job;
			fa.stride = X.P.stride;
			fa.next = &X.P.dev->fam_next;
			e = launch_family_lb2(ctx->bp, ctx->tables, fa, X.window, ctx->num_sms, s,
			                      X.fam_kb);
		}
	}
	if (e != cudaSuccess)
		return e;
	choose_kernel<<<grid, 256, 0, s>>>(X.P);
	kept_scan_kernel<<<1, kSelThreads, 0, s>>>(X.P);
	emit_kernel<<<2 * grid, kEmitThreads, 0, s>>>(X.P);
	finish_iteration_kernel<<<1, 32, 0, s>>>(X.P);
	return cudaGetLastError();
}

// Window bounds: at most `window` fathers per iteration, shrinking to
// window / 64 (at least 64) after an incumbent improvement, then doubling
// per iteration up to a ceiling that is window / 16 right after the
// improvement and doubles every 128 iterations without one.
int window_min_of(int window) { return std::min(window, std::max(64, window / 64)); }

void fill_stats(const wsbb::ExDev &h, const int16_t *best_rec, int n, int status,
                double seconds, long long reads, int S, wsbb_stats *st)
{
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
	st->seconds = seconds;
	st->scanned = (int64_t)h.scanned;
	st->committed = (int64_t)h.committed;
	st->early = (int64_t)h.early;
	st->settled_fathers = (int64_t)h.settled_fathers;
	st->d2h_bytes = (int64_t)(reads * (long long)sizeof(wsbb::ExDev) + S);
	long long pending = 0;
	for (int d = 0; d < n; ++d) {
		st->pending_hist[d + 1] = h.pend[d];
		pending += h.pend[d];
	}
	st->pending = pending;
	st->takes = st->branched + st->pruned + st->leaves - pending;
}

struct SearchMode {
	int mode = 0;                 // 0 plain, 1 learned, 2 logging
	const wsbb_model *model = nullptr;
	int K = 0;
	uint8_t *log_rec = nullptr;
	long long log_cap = 0;
	int log_stride = 1;
};

// Stack capacity and window of a search configuration.
int search_shape(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, int &window, long long &cap,
                 long long &region_cap)
{
	using namespace wsbb;
	const int n = ctx->inst.n;
	const int S = ctx->bp.stride;
	window = cfg->window > 0 ? cfg->window : 16384;
	cap = cfg->capacity;
	if (cap <= 0) {
		// A `window`-wide DFS keeps up to about window * u entries per level
		// live: 2 * window * n^2 covers it, within half the free memory.
		cap = std::max(1ll << 22, 2ll * window * n * n);
		size_t free_b = 0, total_b = 0;
		if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
			const long long fit = (long long)(free_b / 2 / (S + sizeof(Meta)));
			cap = std::min(cap, std::max(fit, 1ll << 20));
		}
	}
	// Scanning past pruned entries to fill the window is cheap next to an
	// under-filled iteration; the region copy grows with it.
	region_cap = 16ll * window + 8192;
	if (window > (1 << 20) || cap < region_cap)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "window / capacity out of range");
	return WSBB_OK;
}

// The context's search state for this shape (allocated, or reallocated when
// the shape changed, which drops any stopped search).
int search_state(wsbb_ctx *ctx, int window, long long cap, long long region_cap)
{
	using namespace wsbb;
	const int n = ctx->inst.n;
	const int S = ctx->bp.stride;
	ExploreState *X = ctx->ex;
	if (!X || X->cap != cap || X->window != window) {
		wsbb_explore_release(ctx);
		X = new ExploreState();
		X->bytes = search_layout(nullptr, cap, region_cap, window, n, S, X->P);
		const cudaError_t e = cudaMalloc(&X->mem, X->bytes);
		if (e != cudaSuccess) {
			delete X;
			return wsbb_set_error(ctx, WSBB_ERR_NOMEM, "search pool allocation failed");
		}
		search_layout(static_cast<uint8_t *>(X->mem), cap, region_cap, window, n, S, X->P);
		X->cap = cap;
		X->region_cap = region_cap;
		X->child_cap = X->P.child_cap;
		X->window = window;
		X->child_bp = ctx->bp;
		X->child_bp.count_dev = &X->P.dev->n_children;
		ctx->ex = X;
	}
	return WSBB_OK;
}

int run_search(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, const SearchMode &M, wsbb_stats *st,
               void *stream_v, long long *logged)
{
	using namespace wsbb;
	if (!ctx || !cfg || !st)
		return WSBB_ERR_ARG;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	const int n = ctx->inst.n;
	const int S = ctx->bp.stride;
	int window = 0;
	long long cap = 0, region_cap = 0;
	int rc = search_shape(ctx, cfg, window, cap, region_cap);
	if (rc != WSBB_OK)
		return rc;
	const bool resume = (cfg->flags & WSBB_EXPLORE_RESUME) != 0;
	if (resume && (!ctx->ex || ctx->ex->cap != cap || ctx->ex->window != window))
		return wsbb_set_error(ctx, WSBB_ERR_ARG,
		                      "no stopped search of this window and capacity to resume");
	if ((rc = search_state(ctx, window, cap, region_cap)) != WSBB_OK)
		return rc;
	ExploreState *X = ctx->ex;
	if (M.mode == 1) {
		int D = 0;
		wsbb_model_dims(M.model, &D, nullptr, nullptr);
		const size_t need = size_t(window) * D * 4 + size_t(window) * M.K * 2 + 256 +
		                    size_t(X->child_cap) * 4 + 256;
		if (X->learned_bytes < need) {
			if (X->learned_mem)
				cudaFree(X->learned_mem);
			X->learned_mem = nullptr;
			X->learned_bytes = 0;
			if (cudaMalloc(&X->learned_mem, need) != cudaSuccess)
				return wsbb_set_error(ctx, WSBB_ERR_NOMEM, "learned buffers");
			X->learned_bytes = need;
		}
		uint8_t *b = static_cast<uint8_t *>(X->learned_mem);
		X->P.feat = reinterpret_cast<float *>(b);
		X->P.fpairs = reinterpret_cast<int16_t *>(b + size_t(window) * D * 4);
		X->P.unsettled = reinterpret_cast<int32_t *>(
		    b + ((size_t(window) * D * 4 + size_t(window) * M.K * 2 + 255) & ~size_t(255)));
		X->P.K = M.K;
		X->P.D = D;
		X->P.inv_scale = wsbb_feature_scale(ctx);
	}
	X->P.log_rec = M.mode == 2 ? M.log_rec : nullptr;
	X->P.log_cap = M.mode == 2 ? M.log_cap : 0;
	X->P.log_stride = M.mode == 2 ? std::max(1, M.log_stride) : 1;

	cudaStream_t s = stream_v ? static_cast<cudaStream_t>(stream_v) : ctx->stream;
	// no caller stream: the training-record buffer may still be in use by
	// work queued on the legacy default stream
	if (!stream_v && (e = wait_for_legacy(s, ctx->legacy_ev)) != cudaSuccess)
		return ex_fail(ctx, e, "stream ordering");
	if (resume)
		resume_kernel<<<1, 32, 0, s>>>(X->P, cfg->ub0, cfg->best);
	else
		init_kernel<<<1, 128, 0, s>>>(X->P, cfg->ub0, cfg->best, window_min_of(window), window,
		                              cfg->max_iters > 0 || cfg->max_bounded > 0);
	e = cudaGetLastError();
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search init");

	const int G = cfg->graph_iters > 0 ? cfg->graph_iters : 16;
	const bool use_graph = !(cfg->flags & WSBB_EXPLORE_NO_GRAPH);
	// kernel arguments are captured by value: any change of mode, model, K,
	// learned buffers or log target needs a new graph
	X->child_lb2 = (cfg->flags & WSBB_EXPLORE_CHILD_LB2) != 0;
	X->fam_kb = cfg->family_smem_kb;
	const bool stale = X->graph_iters != G || X->graph_stream != s || X->mode != M.mode ||
	                   X->graph_child_lb2 != X->child_lb2 || X->graph_fam_kb != X->fam_kb ||
	                   X->model != M.model || X->graph_K != X->P.K ||
	                   X->graph_learned != X->learned_mem || X->graph_log != X->P.log_rec ||
	                   X->graph_log_cap != X->P.log_cap || X->graph_log_stride != X->P.log_stride;
	X->mode = M.mode;
	X->model = M.model;
	X->graph_K = X->P.K;
	X->graph_learned = X->learned_mem;
	X->graph_log = X->P.log_rec;
	X->graph_log_cap = X->P.log_cap;
	X->graph_log_stride = X->P.log_stride;
	X->graph_child_lb2 = X->child_lb2;
	X->graph_fam_kb = X->fam_kb;
	if (use_graph && (!X->graph || stale)) {
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
	long long reads = 0;
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
		++reads;
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(s);
		if (e != cudaSuccess || h.done || h.error)
			break;
		if (launched >= max_iters || (M.mode == 2 && (long long)h.log_count >= M.log_cap) ||
		    (cfg->max_bounded > 0 && (long long)h.bounded >= cfg->max_bounded)) {
			status = 1; // iteration cap, or the training-record buffer is full
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
	fill_stats(h, best_rec.data(), n, status, ms * 1e-3, reads, S, st);
	if (logged)
		*logged = std::min((long long)h.log_count, M.log_cap);
	if (h.error)
		return wsbb_set_error(ctx, h.error, "search pool capacity exceeded");
	return WSBB_OK;
}

}  // namespace host
}  // namespace wsbb

using namespace wsbb::host;

extern "C" int wsbb_explore(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, wsbb_stats *st,
                            void *stream)
{
	if (cfg && (cfg->flags & WSBB_EXPLORE_RESIDENT))
		return wsbb_explore_resident(&ctx, 1, cfg, nullptr, st, stream);
	return run_search(ctx, cfg, SearchMode(), st, stream, nullptr);
}

extern "C" int wsbb_explore_seed(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, const void *recs,
                                 const int32_t *lbs, int64_t count, void *stream)
{
	using namespace wsbb;
	if (!ctx || !cfg || count < 0 || (count > 0 && (!recs || !lbs)))
		return WSBB_ERR_ARG;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	const int n = ctx->inst.n, S = ctx->bp.stride;
	int window = 0;
	long long cap = 0, region_cap = 0;
	int rc = search_shape(ctx, cfg, window, cap, region_cap);
	if (rc != WSBB_OK)
		return rc;
	if (count > cap - region_cap)
		return wsbb_set_error(ctx, WSBB_ERR_CAPACITY, "more seed nodes than the stack holds");
	// records are checked on the host: the search indexes its tables by them
	const int16_t *r16 = static_cast<const int16_t *>(recs);
	std::vector<Meta> meta((size_t)count);
	for (int64_t i = 0; i < count; ++i) {
		const int16_t *r = r16 + i * (S / 2);
		const int l1 = r[n], l2 = r[n + 1], depth = r[n + 2];
		unsigned seen[(WSBB_MAX_JOBS + 31) / 32] = {};
		bool ok = l1 >= -1 && l2 <= n && l2 - l1 >= 3 && depth == n - (l2 - l1 - 1);
		for (int j = 0; ok && j < n; ++j) {
			const int v = r[j];
			ok = v >= 0 && v < n && !(seen[v >> 5] >> (v & 31) & 1u);
			if (ok)
				seen[v >> 5] |= 1u << (v & 31);
		}
		if (!ok)
			return wsbb_set_error(ctx, WSBB_ERR_ARG, "seed record is not an open node");
		meta[size_t(i)] = Meta{lbs[i], uint8_t(depth), ST_UNPROC, 0};
	}
	if ((rc = search_state(ctx, window, cap, region_cap)) != WSBB_OK)
		return rc;
	ExploreState *X = ctx->ex;
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	if (count > 0)
		e = cudaMemcpyAsync(X->P.rec, recs, size_t(count) * S, cudaMemcpyHostToDevice, s);
	if (e == cudaSuccess && count > 0)
		e = cudaMemcpyAsync(X->P.meta, meta.data(), size_t(count) * sizeof(Meta),
		                    cudaMemcpyHostToDevice, s);
	if (e == cudaSuccess) {
		seed_kernel<<<1, 128, 0, s>>>(X->P, count, cfg->ub0, cfg->best, window_min_of(window),
		                              window);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s); // the host meta buffer goes out of scope
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search seed");
	return WSBB_OK;
}

extern "C" int wsbb_explore_export(wsbb_ctx *ctx, int64_t max_count, void *recs_out,
                                   int32_t *lbs_out, int64_t *count_out, void *stream)
{
	using namespace wsbb;
	if (!ctx || max_count < 0 || !count_out || (max_count > 0 && (!recs_out || !lbs_out)))
		return WSBB_ERR_ARG;
	*count_out = 0;
	if (!ctx->ex)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "no search state to export from");
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	ExploreState *X = ctx->ex;
	const int S = ctx->bp.stride;
	// the region copy stages the exported nodes
	const long long take = std::min<long long>(max_count, X->region_cap);
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	export_kernel<<<1, kSelThreads, 0, s>>>(X->P, take);
	e = cudaGetLastError();
	long long got = 0;
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(&got, &X->P.dev->exported, sizeof(got), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s);
	std::vector<Meta> meta(size_t(std::max(got, 0ll)));
	if (e == cudaSuccess && got > 0)
		e = cudaMemcpyAsync(recs_out, X->P.tmp_rec, size_t(got) * S, cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && got > 0)
		e = cudaMemcpyAsync(meta.data(), X->P.tmp_meta, size_t(got) * sizeof(Meta),
		                    cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search export");
	for (long long i = 0; i < got; ++i)
		lbs_out[i] = meta[size_t(i)].lb;
	*count_out = got;
	return WSBB_OK;
}

extern "C" int wsbb_explore_learned(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg,
                                    wsbb_model *model, int K, wsbb_stats *st, void *stream)
{
	if (!ctx || !model)
		return WSBB_ERR_ARG;
	int D = 0, O = 0;
	wsbb_model_dims(model, &D, &O, nullptr);
	if (K < 1 || K > 32 || K > ctx->inst.P || ctx->inst.m > 20 ||
	    D != (3 * ctx->inst.m + ctx->inst.n + 15) / 16 * 16 ||
	    O != (ctx->inst.P + 7) / 8 * 8)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "model does not match the instance or K");
	SearchMode M;
	M.mode = 1;
	M.model = model;
	M.K = K;
	return run_search(ctx, cfg, M, st, stream, nullptr);
}

extern "C" int wsbb_explore_log(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, void *recs_out,
                                int64_t cap, int stride, int64_t *logged, wsbb_stats *st,
                                void *stream)
{
	if (!ctx || !recs_out || cap <= 0 || stride < 1)
		return WSBB_ERR_ARG;
	SearchMode M;
	M.mode = 2;
	M.log_rec = static_cast<uint8_t *>(recs_out);
	M.log_cap = cap;
	M.log_stride = stride;
	long long got = 0;
	const int rc = run_search(ctx, cfg, M, st, stream, &got);
	if (logged)
		*logged = got;
	return rc;
}

// ---------------------------------------------------------------------------
// wsbb_explore_noalloc: the search above with its whole state in one fixed
// file-scope device array instead of memory it allocates, for callers that
// must not allocate GPU memory. The kernels are the same; only where their
// buffers live differs.

namespace {

__device__ __align__(256) uint8_t g_noalloc_scratch[WSBB_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch on the current device. In host code
// the symbol itself is only a host-side stand-in, never a device address,
// so it is never handed to a kernel directly. The address is looked up on
// every call (a cheap query once the module is loaded), so a primary
// context that was torn down and re-created never leaves a stale pointer.
int noalloc_scratch(wsbb_ctx *ctx, uint8_t **out)
{
	void *p = nullptr;
	const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
	if (e != cudaSuccess || !p)
		return ex_fail(ctx, e != cudaSuccess ? e : cudaErrorInvalidSymbol,
		               "cudaGetSymbolAddress(no-alloc scratch)");
	*out = static_cast<uint8_t *>(p);
	return WSBB_OK;
}

// Stack capacity (nodes) that fits the fixed array with the given window
// and the region reserve of the no-alloc search (0: none).
long long noalloc_capacity(int window, long long region_cap, int n, int S)
{
	const size_t limit = WSBB_NOALLOC_SCRATCH_BYTES;
	wsbb::ExParams P{};
	const size_t fixed = wsbb::search_layout(nullptr, 0, region_cap, window, n, S, P);
	long long cap = fixed < limit ? (long long)((limit - fixed) / (S + sizeof(wsbb::Meta))) : 0;
	while (cap > 0 && wsbb::search_layout(nullptr, cap, region_cap, window, n, S, P) > limit)
		cap -= 256;
	return std::max(cap, 0ll);
}

long long noalloc_region(int window) { return 4ll * window + 4096; }

// Default window: the widest of 1024, 512, ..., 64 that leaves the stack
// room for at least 8 iterations of `window` fathers with n children each
// (n = 20: 1024 and ~397k nodes; n = 50: 256 and ~178k; n = 100: 64 and
// ~99k).
int noalloc_default_window(int n, int S)
{
	for (int w = 1024; w > 64; w >>= 1)
		if (noalloc_capacity(w, noalloc_region(w), n, S) >= 8ll * w * n)
			return w;
	return 64;
}

}  // namespace

extern "C" int wsbb_explore_noalloc(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg,
                                    wsbb_stats *st, void *stream_v)
{
	using namespace wsbb;
	if (!ctx || !cfg || !st)
		return WSBB_ERR_ARG;
	// the shared array holds no search between calls
	if (cfg->flags & WSBB_EXPLORE_RESUME)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "the no-alloc search cannot resume");
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "cudaSetDevice");
	uint8_t *scratch = nullptr;
	int rc = noalloc_scratch(ctx, &scratch);
	if (rc != WSBB_OK)
		return rc;

	const int n = ctx->inst.n;
	const int S = ctx->bp.stride;
	const int window = cfg->window > 0 ? cfg->window : noalloc_default_window(n, S);
	const size_t limit = WSBB_NOALLOC_SCRATCH_BYTES;
	ExploreState X; // host-side view only: no graph, no allocation
	if (window > (1 << 20))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "window out of range");
	const long long region_cap = noalloc_region(window);
	long long cap = cfg->capacity;
	if (cap <= 0)
		cap = noalloc_capacity(window, region_cap, n, S);
	if (cap < region_cap || search_layout(nullptr, cap, region_cap, window, n, S, X.P) > limit)
		return wsbb_set_error(ctx, WSBB_ERR_CAPACITY,
		                      "window / capacity do not fit the fixed no-alloc scratch of " +
		                          std::to_string(limit >> 20) + " MiB");
	search_layout(scratch, cap, region_cap, window, n, S, X.P);
	X.cap = cap;
	X.region_cap = region_cap;
	X.child_cap = X.P.child_cap;
	X.window = window;
	X.child_bp = ctx->bp;
	X.child_bp.count_dev = &X.P.dev->n_children;
	X.child_lb2 = (cfg->flags & WSBB_EXPLORE_CHILD_LB2) != 0;
	X.fam_kb = cfg->family_smem_kb;

	cudaStream_t s = stream_v ? static_cast<cudaStream_t>(stream_v) : ctx->stream;
	// no caller stream: the search runs on the context's stream after the
	// work queued on the legacy default stream so far (the context's own
	// event, so nothing is created here)
	if (!stream_v && (e = wait_for_legacy(s, ctx->legacy_ev)) != cudaSuccess)
		return ex_fail(ctx, e, "stream ordering");
	const auto t0 = std::chrono::steady_clock::now();
	init_kernel<<<1, 128, 0, s>>>(X.P, cfg->ub0, cfg->best, window_min_of(window), window,
	                              cfg->max_iters > 0 || cfg->max_bounded > 0);
	e = cudaGetLastError();
	if (e != cudaSuccess)
		return ex_fail(ctx, e, "search init");
	const int G = cfg->graph_iters > 0 ? cfg->graph_iters : 16;
	const long long max_iters = cfg->max_iters > 0 ? cfg->max_iters : LLONG_MAX;
	ExDev h{};
	long long reads = 0;
	long long launched = 0;
	int status = 0;
	for (;;) {
		for (int i = 0; i < G && e == cudaSuccess; ++i)
			e = enqueue_iteration(ctx, X, s);
		launched += G;
		if (e != cudaSuccess)
			break;
		e = cudaMemcpyAsync(&h, X.P.dev, sizeof(ExDev), cudaMemcpyDeviceToHost, s);
		++reads;
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(s);
		if (e != cudaSuccess || h.done || h.error)
			break;
		if (launched >= max_iters ||
		    (cfg->max_bounded > 0 && (long long)h.bounded >= cfg->max_bounded)) {
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
	fill_stats(h, best_rec, n, status, secs, reads, S, st);
	if (h.error)
		return wsbb_set_error(ctx, h.error, "search outgrew the no-alloc scratch capacity");
	return WSBB_OK;
}
