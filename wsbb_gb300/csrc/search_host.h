// Host side of the exact search shared by explore.cu (the graph-launched
// search and its entry points) and resident.cu (the resident search): the
// per-context search state and the helpers that shape, allocate and report
// it.
#pragma once

#include "search_kernels.cuh"


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
	// mode of the captured graph: 0 plain, 1 learned, 2 logging
	int mode = 0;
	const wsbb_model *model = nullptr;
	void *learned_mem = nullptr; // features, ranked pairs, unsettled list
	size_t learned_bytes = 0;
	int graph_K = 0;
	void *graph_learned = nullptr;
	uint8_t *graph_log = nullptr;
	long long graph_log_cap = 0;
	int graph_log_stride = 0;
	// children bounded one record at a time (pool LB2 kernel) instead of
	// per father (family bounds)
	bool child_lb2 = false;
	bool graph_child_lb2 = false;
	int fam_kb = 0, graph_fam_kb = 0; // family bounds' shared-memory budget
};


namespace wsbb {
namespace host {

int ex_fail(wsbb_ctx *ctx, cudaError_t e, const char *what);
// Window bounds: at most `window` fathers per iteration, shrinking to
// window / 64 (at least 64) after an incumbent improvement.
int window_min_of(int window);
void fill_stats(const wsbb::ExDev &h, const int16_t *best_rec, int n, int status,
                double seconds, long long reads, int S, wsbb_stats *st);
// Stack capacity and window of a search configuration.
int search_shape(wsbb_ctx *ctx, const wsbb_explore_cfg *cfg, int &window, long long &cap,
                 long long &region_cap);
// The context's search state for this shape (allocated, or reallocated when
// the shape changed, which drops any stopped search).
int search_state(wsbb_ctx *ctx, int window, long long cap, long long region_cap);

}  // namespace host
}  // namespace wsbb
