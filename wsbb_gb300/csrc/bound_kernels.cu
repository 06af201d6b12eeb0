// Pool bound kernels for sm_103a: LB2 (Johnson two-machine bound over every
// machine pair), LB1 and full-permutation makespan, one record per lane.
//
// Layout of the work. A CTA stages one instance-table image (Johnson-ordered
// pair tables, p, pairs, heads, tails; see TableView) into shared memory
// once. Each warp then takes 32 consecutive records, copies them into
// shared memory with coalesced 16-byte loads, and each lane bounds one
// record:
//   front times  F[k]  over job[0..limite1]   (max-plus, registers)
//   back times   R[k]  over job[limite2..n-1] for every start machine k,
//                      in one reversed pass: the makespan of a sequence on
//                      machines k..m-1 equals that of the reversed sequence
//                      on the reversed machines, so one O(b*m) sweep gives
//                      all m values the reference gets in O(b*m^2)
//                      (src/bound_flowshop.cpp:876-895)
//   pair loop    for every pair, the Johnson recurrence of
//                src/bound_flowshop.cpp:64-77 over the pair's job order,
//                skipping fixed jobs, then the tail rule of :92-100 /
//                :140-149; LB = max over pairs (:150-153).
// All lanes walk the same pair and the same position at the same time, so
// every table read is a shared-memory broadcast; the per-lane state is the
// record's unscheduled-job mask and its F / R vectors (kept in shared
// memory, one column per lane, so the pair loop can index them by machine).
// Everything is exact int32 arithmetic.
//
// Two LB2 variants:
//   lb2_fast_kernel   n <= 32: 16-byte table entries {1<<job, p1, p2,
//                     lag+p2}, so a Johnson step is one broadcast load, one
//                     mask test, an add and one fused add-max
//                     (max(t1 + p2, t0 + lag + p2) == max(t1, t0 + lag) + p2);
//                     two pairs are interleaved per lane for ILP; the record
//                     staging rows and the F / R columns share one per-warp
//                     buffer (F / R in int16 when the instance's total work
//                     fits); 512-thread CTAs, two per SM.
//   lb2_pool_kernel   any n <= 128: 8-byte packed entries, 1-4 mask words.
#include <algorithm>

#include "wsbb_internal.h"

namespace wsbb {
namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kFastThreads = 512;
constexpr int kFastWarps = kFastThreads / 32;

__device__ __forceinline__ int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

// Bit `x & (32*NW - 1)` of the unscheduled-job mask.
template <int NW>
__device__ __forceinline__ uint32_t mask_bit(const uint32_t (&mask)[NW], uint32_t x)
{
	uint32_t w;
	if (NW == 1) {
		w = mask[0];
	} else if (NW == 2) {
		w = (x & 32u) ? mask[NW - 1] : mask[0];
	} else {
		const uint32_t sel = (x >> 5) & 3u;
		const uint32_t lo = (sel & 1u) ? mask[1] : mask[0];
		const uint32_t hi = (sel & 1u) ? mask[NW - 1] : mask[NW > 2 ? 2 : 0];
		w = (sel & 2u) ? hi : lo;
	}
	return __funnelshift_r(w, 0u, x) & 1u;
}

struct Staged {
	const void *johnson;
	const int32_t *pt;
	const int32_t *pairs;
	const int32_t *heads;
	const int32_t *tails;
	uint8_t *rest; // first byte after the table image
};

__device__ __forceinline__ Staged stage_tables(const TableView &tv, uint8_t *smem)
{
	const uint4 *src = reinterpret_cast<const uint4 *>(tv.blob);
	uint4 *dst = reinterpret_cast<uint4 *>(smem);
	for (uint32_t i = threadIdx.x; i < tv.bytes / 16; i += blockDim.x)
		dst[i] = src[i];
	Staged s;
	s.johnson = smem;
	s.pt = reinterpret_cast<const int32_t *>(smem + tv.off_pt);
	s.pairs = reinterpret_cast<const int32_t *>(smem + tv.off_pairs);
	s.heads = reinterpret_cast<const int32_t *>(smem + tv.off_heads);
	s.tails = reinterpret_cast<const int32_t *>(smem + tv.off_tails);
	s.rest = smem + tv.bytes;
	return s;
}

__host__ __device__ __forceinline__ int rec_words_of(int stride) { return (stride / 4) | 1; }

// Copy records [base, base + nrec) of the pool — or, with `gather`, the
// records gather[base..base + nrec) — into this warp's staging rows (odd
// word stride: lanes reading their own row hit distinct banks).
__device__ __forceinline__ void stage_records(int stride, const uint8_t *recs, int64_t base,
                                              int nrec, uint32_t *rows, int rec_words, int lane,
                                              const int32_t *gather)
{
	const int chunks_per_rec = stride / 16;
	const int nchunks = nrec * chunks_per_rec;
	for (int c = lane; c < nchunks; c += 32) {
		const int r = c / chunks_per_rec;
		const int k = c - r * chunks_per_rec;
		const int64_t rid = gather ? int64_t(gather[base + r]) : base + r;
		const uint4 v = __ldg(reinterpret_cast<const uint4 *>(recs + rid * stride) + k);
		uint32_t *d = rows + r * rec_words + k * 4;
		d[0] = v.x;
		d[1] = v.y;
		d[2] = v.z;
		d[3] = v.w;
	}
}

template <int MAXM>
__device__ __forceinline__ void front_times(const int16_t *rec, int upto, int n, int m,
                                            const int32_t *pt, int32_t (&F)[MAXM])
{
#pragma unroll
	for (int k = 0; k < MAXM; ++k)
		F[k] = 0;
	for (int j = 0; j <= upto; ++j) {
		const int job = rec[j];
		F[0] += pt[job];
#pragma unroll
		for (int k = 1; k < MAXM; ++k)
			if (k < m)
				F[k] = imax(F[k], F[k - 1]) + pt[k * n + job];
	}
}

// Back times in reversed machine order: G[r] = makespan of job[from..n-1]
// on machines m-1-r .. m-1.
template <int MAXM>
__device__ __forceinline__ void back_times(const int16_t *rec, int from, int n, int m,
                                           const int32_t *pt, int32_t (&G)[MAXM])
{
#pragma unroll
	for (int r = 0; r < MAXM; ++r)
		G[r] = 0;
	for (int j = n - 1; j >= from; --j) {
		const int job = rec[j];
		G[0] += pt[(m - 1) * n + job];
#pragma unroll
		for (int r = 1; r < MAXM; ++r)
			if (r < m)
				G[r] = imax(G[r], G[r - 1]) + pt[(m - 1 - r) * n + job];
	}
}

template <int MAXM>
__device__ __forceinline__ int32_t last_of(const int32_t (&F)[MAXM], int m)
{
	int32_t v = 0;
#pragma unroll
	for (int k = 0; k < MAXM; ++k)
		if (k == m - 1)
			v = F[k];
	return v;
}

// ---------------------------------------------------------------- fast path

// Per-warp buffer: [colF | colR], with the record staging rows placed
// right after colF, so F can be stored while the rows are still read and
// only colR overwrites them (after the warp is done with the rows).
template <typename ColT>
__host__ __device__ __forceinline__ int fast_col_bytes(int m)
{
	return (m * 32 * int(sizeof(ColT)) + 15) & ~15;
}

template <typename ColT>
__host__ __device__ __forceinline__ int fast_warp_bytes(int stride, int m)
{
	const int staging = 32 * rec_words_of(stride) * 4;
	const int col = fast_col_bytes<ColT>(m);
	return col + ((staging > col ? staging : col) + 15 & ~15);
}

// One Johnson step of one pair for a lane whose unscheduled-job mask is
// `mask`: skip the job when it is fixed.
__device__ __forceinline__ void johnson_step(uint32_t mask, const uint4 &v, int32_t &t0,
                                             int32_t &t1)
{
	if (mask & v.x) {
		t0 += int32_t(v.y);
		t1 = __viaddmax_s32(t0, int32_t(v.w), t1 + int32_t(v.z));
	}
}

template <int MAXM, typename ColT>
__global__ void __launch_bounds__(kFastThreads, 2)
    lb2_fast_kernel(BoundParams bp, const uint8_t *__restrict__ recs, int64_t count,
                    int32_t *__restrict__ out)
{
	extern __shared__ __align__(16) uint8_t smem[];
	if (bp.count_dev)
		count = *bp.count_dev;
	const Staged s = stage_tables(bp.t16, smem);
	__syncthreads();

	const int n = bp.n, m = bp.m, P = bp.P;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int rec_words = rec_words_of(bp.stride);
	uint8_t *wbuf = s.rest + warp * fast_warp_bytes<ColT>(bp.stride, m);
	ColT *colF = reinterpret_cast<ColT *>(wbuf);
	ColT *colR = reinterpret_cast<ColT *>(wbuf + fast_col_bytes<ColT>(m));
	uint32_t *rows = reinterpret_cast<uint32_t *>(colR);
	const uint4 *tj = reinterpret_cast<const uint4 *>(s.johnson);
	const int64_t step = int64_t(gridDim.x) * kFastWarps * 32;

	for (int64_t base = (int64_t(blockIdx.x) * kFastWarps + warp) * 32; base < count;
	     base += step) {
		const int nrec = count - base < 32 ? int(count - base) : 32;
		stage_records(bp.stride, recs, base, nrec, rows, rec_words, lane, bp.gather);
		__syncwarp();
		bool work = false;
		int32_t lb = 0;
		uint32_t mask = 0;
		int32_t G[MAXM];
		int l1 = 0, l2 = 0;
		if (lane < nrec) {
			const int16_t *rec = reinterpret_cast<const int16_t *>(rows + lane * rec_words);
			l1 = rec[n];
			l2 = rec[n + 1];
			int32_t F[MAXM];
			if (l2 - l1 == 1) {
				front_times<MAXM>(rec, n - 1, n, m, s.pt, F);
				lb = last_of<MAXM>(F, m);
			} else {
				work = true;
				mask = n == 32 ? 0xffffffffu : (1u << n) - 1u;
				for (int j = 0; j <= l1; ++j)
					mask &= ~(1u << rec[j]);
				for (int j = l2; j < n; ++j)
					mask &= ~(1u << rec[j]);
				front_times<MAXM>(rec, l1, n, m, s.pt, F);
#pragma unroll
				for (int k = 0; k < MAXM; ++k)
					if (k < m)
						colF[k * 32 + lane] = ColT(l1 >= 0 ? F[k] : s.heads[k]);
				back_times<MAXM>(rec, l2, n, m, s.pt, G);
			}
		}
		__syncwarp(); // the staging rows are overwritten by colR below
		if (work) {
#pragma unroll
			for (int r = 0; r < MAXM; ++r)
				if (r < m) {
					const int k = m - 1 - r;
					colR[k * 32 + lane] = ColT(l2 < n ? G[r] : s.tails[k]);
				}
			// With no back jobs the tail is the static tail of the pair's
			// second machine alone (src/bound_flowshop.cpp:147-148).
			const int32_t first_tail_off = l2 < n ? 0 : -(1 << 30);
			int i = 0;
			for (; i + 1 < P; i += 2) {
				const int32_t ma = s.pairs[i], mb = s.pairs[i + 1];
				const int a0 = ma & 0xff, a1 = ma >> 8, b0 = mb & 0xff, b1 = mb >> 8;
				int32_t ta0 = colF[a0 * 32 + lane], ta1 = colF[a1 * 32 + lane];
				int32_t tb0 = colF[b0 * 32 + lane], tb1 = colF[b1 * 32 + lane];
				const uint4 *ea = tj + i * n;
				const uint4 *eb = ea + n;
#pragma unroll 4
				for (int q = 0; q < n; ++q) {
					const uint4 va = ea[q];
					const uint4 vb = eb[q];
					johnson_step(mask, va, ta0, ta1);
					johnson_step(mask, vb, tb0, tb1);
				}
				const int32_t va = imax(ta1 + colR[a1 * 32 + lane],
				                        ta0 + colR[a0 * 32 + lane] + first_tail_off);
				const int32_t vb = imax(tb1 + colR[b1 * 32 + lane],
				                        tb0 + colR[b0 * 32 + lane] + first_tail_off);
				lb = imax(lb, imax(va, vb));
			}
			if (i < P) {
				const int32_t ma = s.pairs[i];
				const int a0 = ma & 0xff, a1 = ma >> 8;
				int32_t t0 = colF[a0 * 32 + lane], t1 = colF[a1 * 32 + lane];
				const uint4 *ea = tj + i * n;
#pragma unroll 4
				for (int q = 0; q < n; ++q)
					johnson_step(mask, ea[q], t0, t1);
				lb = imax(lb, imax(t1 + colR[a1 * 32 + lane],
				                   t0 + colR[a0 * 32 + lane] + first_tail_off));
			}
		}
		if (lane < nrec)
			out[bp.gather ? int64_t(bp.gather[base + lane]) : base + lane] = lb;
		__syncwarp(); // the next batch's staging overwrites the columns
	}
}

// ------------------------------------------------------------- generic path

template <int NW, int MAXM>
__global__ void __launch_bounds__(kThreads) lb2_pool_kernel(BoundParams bp,
                                                           const uint8_t *__restrict__ recs,
                                                           int64_t count,
                                                           int32_t *__restrict__ out)
{
	extern __shared__ __align__(16) uint8_t smem[];
	if (bp.count_dev)
		count = *bp.count_dev;
	const Staged s = stage_tables(bp.t8, smem);
	__syncthreads();

	const int n = bp.n, m = bp.m, P = bp.P;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int32_t *colF = reinterpret_cast<int32_t *>(s.rest);
	int32_t *colR = colF + m * kThreads;
	const int rec_words = rec_words_of(bp.stride);
	uint32_t *rows = reinterpret_cast<uint32_t *>(colR + m * kThreads) + warp * 32 * rec_words;
	const uint2 *tj = reinterpret_cast<const uint2 *>(s.johnson);
	const int64_t step = int64_t(gridDim.x) * kWarps * 32;

	for (int64_t base = (int64_t(blockIdx.x) * kWarps + warp) * 32; base < count;
	     base += step) {
		const int nrec = count - base < 32 ? int(count - base) : 32;
		stage_records(bp.stride, recs, base, nrec, rows, rec_words, lane, bp.gather);
		__syncwarp();
		if (lane < nrec) {
			const int16_t *rec = reinterpret_cast<const int16_t *>(rows + lane * rec_words);
			const int l1 = rec[n], l2 = rec[n + 1];
			int32_t lb;
			if (l2 - l1 == 1) {
				int32_t F[MAXM];
				front_times<MAXM>(rec, n - 1, n, m, s.pt, F);
				lb = last_of<MAXM>(F, m);
			} else {
				uint32_t mask[NW];
#pragma unroll
				for (int w = 0; w < NW; ++w) {
					const int lo = 32 * w;
					mask[w] = n >= lo + 32 ? 0xffffffffu
					                       : (n > lo ? (1u << (n - lo)) - 1u : 0u);
				}
				for (int j = 0; j < n; ++j) {
					if (j > l1 && j < l2)
						continue;
					const int job = rec[j];
#pragma unroll
					for (int w = 0; w < NW; ++w)
						if ((job >> 5) == w)
							mask[w] &= ~(1u << (job & 31));
				}
				{
					int32_t F[MAXM];
					front_times<MAXM>(rec, l1, n, m, s.pt, F);
#pragma unroll
					for (int k = 0; k < MAXM; ++k)
						if (k < m)
							colF[k * kThreads + tid] = l1 >= 0 ? F[k] : s.heads[k];
				}
				{
					int32_t G[MAXM];
					back_times<MAXM>(rec, l2, n, m, s.pt, G);
#pragma unroll
					for (int r = 0; r < MAXM; ++r)
						if (r < m) {
							const int k = m - 1 - r;
							colR[k * kThreads + tid] = l2 < n ? G[r] : s.tails[k];
						}
				}
				const int32_t first_tail_off = l2 < n ? 0 : -(1 << 30);
				const int32_t *cF = colF + tid;
				const int32_t *cR = colR + tid;
				lb = 0;
				for (int i = 0; i < P; ++i) {
					const int32_t mm = s.pairs[i];
					const int a = mm & 0xff, c = mm >> 8;
					int32_t t0 = cF[a * kThreads], t1 = cF[c * kThreads];
					const uint2 *e = tj + i * n;
#pragma unroll 4
					for (int q = 0; q < n; ++q) {
						const uint2 v = e[q];
						if (mask_bit<NW>(mask, v.x)) {
							t0 += int32_t(v.x >> 16);
							t1 = imax(t1, t0 + int32_t(v.y >> 16)) + int32_t(v.y & 0xffffu);
						}
					}
					const int32_t v1 =
					    imax(t1 + cR[c * kThreads], t0 + cR[a * kThreads] + first_tail_off);
					lb = imax(lb, v1);
				}
			}
			out[bp.gather ? int64_t(bp.gather[base + lane]) : base + lane] = lb;
		}
		__syncwarp();
	}
}

// LB1 (mode 1) and makespan (mode 2): not on the hot path; generic shapes.
template <int MODE>
__global__ void __launch_bounds__(kThreads) aux_pool_kernel(BoundParams bp,
                                                           const uint8_t *__restrict__ recs,
                                                           int64_t count,
                                                           int32_t *__restrict__ out)
{
	extern __shared__ __align__(16) uint8_t smem[];
	if (bp.count_dev)
		count = *bp.count_dev;
	const Staged s = stage_tables(bp.t8, smem);
	__syncthreads();
	const int n = bp.n, m = bp.m;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int rec_words = rec_words_of(bp.stride);
	uint32_t *rows = reinterpret_cast<uint32_t *>(s.rest + 2 * m * kThreads * 4) +
	                 warp * 32 * rec_words;
	const int64_t step = int64_t(gridDim.x) * kWarps * 32;
	for (int64_t base = (int64_t(blockIdx.x) * kWarps + warp) * 32; base < count;
	     base += step) {
		const int nrec = count - base < 32 ? int(count - base) : 32;
		stage_records(bp.stride, recs, base, nrec, rows, rec_words, lane, bp.gather);
		__syncwarp();
		if (lane < nrec) {
			const int16_t *rec = reinterpret_cast<const int16_t *>(rows + lane * rec_words);
			const int l1 = rec[n], l2 = rec[n + 1];
			int32_t F[WSBB_MAX_MACHINES];
			int32_t res;
			if (MODE == 2 || l2 - l1 == 1) {
				front_times<WSBB_MAX_MACHINES>(rec, n - 1, n, m, s.pt, F);
				res = last_of<WSBB_MAX_MACHINES>(F, m);
			} else {
				int32_t G[WSBB_MAX_MACHINES];
				front_times<WSBB_MAX_MACHINES>(rec, l1, n, m, s.pt, F);
				back_times<WSBB_MAX_MACHINES>(rec, l2, n, m, s.pt, G);
				res = 0;
				for (int k = 0; k < m; ++k) {
					int32_t work = 0;
					for (int j = l1 + 1; j < l2; ++j)
						work += s.pt[k * n + rec[j]];
					int32_t head = s.heads[k], tail = s.tails[k];
#pragma unroll
					for (int q = 0; q < WSBB_MAX_MACHINES; ++q) {
						if (q == k && l1 >= 0)
							head = F[q];
						if (q == m - 1 - k && l2 < n)
							tail = G[q];
					}
					res = imax(res, head + work + tail);
				}
			}
			out[bp.gather ? int64_t(bp.gather[base + lane]) : base + lane] = res;
		}
		__syncwarp();
	}
}

// ---------------------------------------------------------------- launchers

template <typename K>
cudaError_t launch(K kernel, int threads, size_t smem, const BoundParams &bp, const void *recs,
                   int64_t count, int32_t *out, int num_sms, cudaStream_t stream)
{
	cudaError_t e = allow_max_dynamic_smem(kernel);
	if (e != cudaSuccess)
		return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
	if (e != cudaSuccess)
		return e;
	if (per_sm < 1)
		return cudaErrorInvalidConfiguration;
	const int warps_per_block = threads / 32;
	const int64_t warps_needed = (count + 31) / 32;
	const int64_t blocks_needed = (warps_needed + warps_per_block - 1) / warps_per_block;
	const int grid = int(std::max<int64_t>(
	    1, std::min<int64_t>(blocks_needed, int64_t(num_sms) * per_sm)));
	kernel<<<grid, threads, smem, stream>>>(bp, static_cast<const uint8_t *>(recs), count, out);
	return cudaGetLastError();
}

size_t generic_smem(const BoundParams &bp)
{
	return size_t(bp.t8.bytes) + 2 * size_t(bp.m) * kThreads * 4 +
	       size_t(kThreads) * rec_words_of(bp.stride) * 4;
}

template <typename ColT>
size_t fast_smem(const BoundParams &bp)
{
	return size_t(bp.t16.bytes) + size_t(kFastWarps) * fast_warp_bytes<ColT>(bp.stride, bp.m);
}

template <int NW>
cudaError_t launch_lb2_nw(const BoundParams &bp, const void *recs, int64_t count, int32_t *out,
                          int num_sms, cudaStream_t stream)
{
	const size_t sm = generic_smem(bp);
	if (bp.m <= 8)
		return launch(lb2_pool_kernel<NW, 8>, kThreads, sm, bp, recs, count, out, num_sms,
		              stream);
	if (bp.m <= 16)
		return launch(lb2_pool_kernel<NW, 16>, kThreads, sm, bp, recs, count, out, num_sms,
		              stream);
	if (bp.m <= 20)
		return launch(lb2_pool_kernel<NW, 20>, kThreads, sm, bp, recs, count, out, num_sms,
		              stream);
	return launch(lb2_pool_kernel<NW, 32>, kThreads, sm, bp, recs, count, out, num_sms,
	              stream);
}

template <typename ColT>
cudaError_t launch_fast(const BoundParams &bp, const void *recs, int64_t count, int32_t *out,
                        int num_sms, cudaStream_t stream)
{
	const size_t sm = fast_smem<ColT>(bp);
	if (bp.m <= 8)
		return launch(lb2_fast_kernel<8, ColT>, kFastThreads, sm, bp, recs, count, out,
		              num_sms, stream);
	if (bp.m <= 16)
		return launch(lb2_fast_kernel<16, ColT>, kFastThreads, sm, bp, recs, count, out,
		              num_sms, stream);
	if (bp.m <= 20)
		return launch(lb2_fast_kernel<20, ColT>, kFastThreads, sm, bp, recs, count, out,
		              num_sms, stream);
	return launch(lb2_fast_kernel<32, ColT>, kFastThreads, sm, bp, recs, count, out, num_sms,
	              stream);
}

cudaError_t launch_generic(const BoundParams &bp, const void *recs, int64_t count,
                           int32_t *out, int num_sms, cudaStream_t stream)
{
	if (bp.n <= 32)
		return launch_lb2_nw<1>(bp, recs, count, out, num_sms, stream);
	if (bp.n <= 64)
		return launch_lb2_nw<2>(bp, recs, count, out, num_sms, stream);
	return launch_lb2_nw<4>(bp, recs, count, out, num_sms, stream);
}

}  // namespace

bool fast_path_fits(const BoundParams &bp)
{
	if (!bp.t16.blob || bp.n > 32)
		return false;
	const size_t sm = bp.col16 ? fast_smem<int16_t>(bp) : fast_smem<int32_t>(bp);
	return sm <= 227 * 1024;
}

size_t pool_bounds_smem(const BoundParams &bp, int threads)
{
	(void)threads;
	return generic_smem(bp);
}

// mode: 0 = LB2 (fast path when it fits), 1 = LB1, 2 = makespan,
// 3 = LB2 on the generic path only.
cudaError_t launch_pool_bounds(const BoundParams &bp, const void *recs, int64_t count,
                               int32_t *out, int mode, int num_sms, cudaStream_t stream)
{
	if (count <= 0)
		return cudaSuccess;
	if (mode == 1)
		return launch(aux_pool_kernel<1>, kThreads, generic_smem(bp), bp, recs, count, out,
		              num_sms, stream);
	if (mode == 2)
		return launch(aux_pool_kernel<2>, kThreads, generic_smem(bp), bp, recs, count, out,
		              num_sms, stream);
	if (mode == 0 && fast_path_fits(bp))
		return bp.col16 ? launch_fast<int16_t>(bp, recs, count, out, num_sms, stream)
		                : launch_fast<int32_t>(bp, recs, count, out, num_sms, stream);
	return launch_generic(bp, recs, count, out, num_sms, stream);
}

}  // namespace wsbb
