// Internal declarations shared by the host precompute (instance.cpp), the
// bound kernels (bound_kernels.cu), the search (explore.cu) and the C-ABI
// layer (capi.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/wsbb_gb300.h"

namespace wsbb {

// Host precompute of one instance (the reference's initialiserVar,
// src/bound_flowshop.cpp:556-576, restricted to what LB2 reads).
struct Instance {
	int n = 0, m = 0, P = 0;
	std::vector<int32_t> p;        // m x n, machine-major
	std::vector<int32_t> mach0;    // P: first machine of pair i
	std::vector<int32_t> mach1;    // P: second machine of pair i
	std::vector<int32_t> lag;      // P x n
	std::vector<int32_t> johnson;  // P x n: job order of pair i
	std::vector<int32_t> heads;    // m: minTempsArr
	std::vector<int32_t> tails;    // m: minTempsDep
};

// Fills `inst` from p (m x n). Returns an error message, empty on success.
std::string build_instance(const int32_t *p_mxn, int n, int m, Instance &inst);

// Device image of the bound tables. Each CTA stages one image into shared
// memory with a single linear copy, so an image is one contiguous blob:
//   johnson[P * n]   pair-major, each pair's jobs in Johnson order, as
//     8-byte entries (generic path, any n <= 128):
//       x = job | p[m1][job] << 16,  y = p[m2][job] | lag << 16
//     16-byte entries (fast path, n <= 32):
//       x = 1 << job, y = p[m1][job], z = p[m2][job], w = lag + p[m2][job]
//   int32 pt[m * n]  p, machine-major
//   int32 pairs[P]   m1 | m2 << 8
//   int32 heads[m], tails[m]
struct TableView {
	const uint8_t *blob = nullptr;
	uint32_t bytes = 0; // multiple of 16
	uint32_t off_pt = 0, off_pairs = 0, off_heads = 0, off_tails = 0;
};

struct DeviceTables {
	void *mem = nullptr; // all images in one allocation
	size_t bytes = 0;
	TableView t8, t16;   // t16.blob is null when n > 32
	// Johnson entries position-major, johnsonT[q * P + i] = entry q of pair
	// i, so that threads walking consecutive pairs read consecutive entries
	// (family bounds): x = job | p1 << 16, y = p2 | (p1 + lag + p2) << 16.
	const uint2 *johnsonT = nullptr;
	// jobposT[j * P + i] = position of job j in pair i's Johnson order
	const uint8_t *jobposT = nullptr;
	// The same entries packed in 32 bits, position-major with rows of Pp
	// (P rounded up to 64) words: tpack[q * Pp + i] = job | p1 << 7 |
	// p2 << 14 | (p1 + lag + p2) << 21. Null when an instance's values do
	// not fit (n > 128, a time > 127 or p1 + lag + p2 > 2047).
	const uint32_t *tpack = nullptr;
	int Pp = 0;
};

// Host images of the tables; offsets are relative to each image.
struct HostTables {
	std::vector<uint8_t> img8, img16, imgT, imgPos, imgPack;
	int Pp = 0;
	TableView t8, t16;
};
HostTables pack_tables(const Instance &inst, std::string &err);

struct BoundParams {
	TableView t8, t16;
	int n, m, P;
	int stride; // record stride in bytes
	int col16;  // 1: every front/back time fits int16 (total work < 32768)
	// 1: (n + m - 1) * max p <= 65535. Every time a bound of this instance
	// produces is the length of a staircase path through the machine x job
	// grid of some permutation (n + m - 1 operations), so it fits uint16.
	int span16 = 0;
	// When set, the kernels read the record count from device memory and
	// the host-side count only sizes the grid (graph-captured launches).
	const long long *count_dev = nullptr;
	// When set, record i of a launch is record gather[i] of the pool and its
	// result goes to out[gather[i]].
	const int32_t *gather = nullptr;
};

// Kernel launchers (bound_kernels.cu). `mode`: 0 = LB2, 1 = LB1,
// 2 = makespan of the full permutation.
cudaError_t launch_pool_bounds(const BoundParams &bp, const void *recs,
                               int64_t count, int32_t *out, int mode,
                               int num_sms, cudaStream_t stream);
size_t pool_bounds_smem(const BoundParams &bp, int threads);

// Family bounds (family.cu): LB2 of every child of each father, in the
// search's child order (the father's u BEGIN children, then its u END
// children; two leaves when it has two free jobs).
struct FamilyArgs {
	const uint8_t *fathers = nullptr;    // father records
	const long long *ridx = nullptr;     // father f is record ridx[f] (null: f)
	long long count = 0;                 // fathers, when count_dev is null
	const long long *count_dev = nullptr;
	const long long *child_off = nullptr; // [count + 1] first child of each father
	int32_t *child_lb = nullptr;
	int16_t *child_job = nullptr;        // the job each child moves
	int stride = 0;                      // record stride in bytes
	// learned form (fpairs set): father f's K ranked pairs fpairs[f * K ..];
	// a child whose bound over them reaches max(*best_dev, *ub_dev) keeps
	// that value (counted in *early), the others get their full LB2
	const int16_t *fpairs = nullptr;
	int K = 0;
	const int *ub_dev = nullptr, *best_dev = nullptr;
	unsigned long long *early = nullptr;
	unsigned long long *settled_fathers = nullptr; // fathers with every child settled
	// fathers are claimed from this device counter (zero at launch); null:
	// round-robin by CTA
	unsigned long long *next = nullptr;
};
// smem_kb: shared-memory budget per CTA in KB (0: 56), which sets the
// pair-chunk length and how many CTAs share an SM.
cudaError_t launch_family_lb2(const BoundParams &bp, const DeviceTables &T, const FamilyArgs &A,
                              long long max_fathers, int num_sms, cudaStream_t s,
                              int smem_kb = 0);
size_t family_smem(const BoundParams &bp, int smem_kb = 0);

// Learned selector inference (learned.cu): top-K pairs of `rows` feature
// rows (rows_dev, when set, holds the row count on the device).
cudaError_t launch_mlp_topk(const wsbb_model *md, const float *X, long long rows,
                            const long long *rows_dev, int K, int16_t *topk, float *logits,
                            int num_sms, cudaStream_t s);

// Raises a kernel's dynamic shared-memory ceiling to the device's opt-in
// maximum, once per (device, kernel). The ceiling is process-wide per
// function, so setting it to each launch's own size would let one host
// thread lower it under another thread's launch (which then fails); the
// ceiling itself changes neither occupancy nor the launch.
cudaError_t allow_max_dynamic_smem_fn(const void *kernel);
template <typename K>
cudaError_t allow_max_dynamic_smem(K kernel)
{
	return allow_max_dynamic_smem_fn(reinterpret_cast<const void *>(kernel));
}

// Orders the library's own stream `s` after the work already queued on the
// legacy default stream, where a caller given no stream (PyTorch's default
// stream among them) writes the buffers it passes in. A non-blocking
// stream does not wait on the legacy stream by itself.
// `s` waits for the work queued on the legacy default stream so far, with
// an event of the caller's (`ev`), or one made for the call when ev is null.
inline cudaError_t wait_for_legacy(cudaStream_t s, cudaEvent_t ev_given = nullptr)
{
	if (s == nullptr || s == cudaStreamLegacy)
		return cudaSuccess;
	if (ev_given) {
		const cudaError_t e = cudaEventRecord(ev_given, cudaStreamLegacy);
		return e == cudaSuccess ? cudaStreamWaitEvent(s, ev_given, 0) : e;
	}
	cudaEvent_t ev;
	cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
	if (e != cudaSuccess)
		return e;
	e = cudaEventRecord(ev, cudaStreamLegacy);
	if (e == cudaSuccess)
		e = cudaStreamWaitEvent(s, ev, 0);
	cudaEventDestroy(ev);
	return e;
}

}  // namespace wsbb

struct wsbb_ctx {
	int device = 0;
	int num_sms = 0;
	wsbb::Instance inst;
	wsbb::DeviceTables tables;
	wsbb::BoundParams bp;
	std::string last_error;
	// host-buffer path scratch (grown on demand)
	void *d_recs = nullptr;
	int32_t *d_out = nullptr;
	int64_t host_cap = 0;
	unsigned long long *d_claim = nullptr; // family bounds' father counter
	cudaStream_t stream = nullptr;
	// recorded on the legacy default stream when a call given no stream runs
	// on `stream` (created with the context, so such calls make no event)
	cudaEvent_t legacy_ev = nullptr;
	// search state (explore.cu)
	struct ExploreState *ex = nullptr;
};

int wsbb_set_error(wsbb_ctx *ctx, int code, const std::string &msg);
