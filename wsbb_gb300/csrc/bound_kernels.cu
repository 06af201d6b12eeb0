// Pool bound kernels for sm_103a: LB2 (Johnson two-machine bound over every
// machine pair), LB1 and full-permutation makespan, one record per lane.
//
// Layout of the work. A CTA stages the instance tables (Johnson-ordered
// pair tables, p, pairs, heads, tails; see DeviceTables) into shared
// memory once. Each warp then takes 32 consecutive records, copies them
// into shared memory with coalesced 16-byte loads, and each lane bounds
// one record:
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
// every table read is a shared-memory broadcast. The only per-lane state is
// the record's unscheduled-job mask and its F / R vectors (kept in shared
// memory, one column per thread, so the pair loop can index them).
// Everything is exact int32 arithmetic.
#include <algorithm>

#include "wsbb_internal.h"

namespace wsbb {
namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

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
	const uint2 *johnson;
	const int32_t *pt;
	const int32_t *pairs;
	const int32_t *heads;
	const int32_t *tails;
	int32_t *colF; // [m][kThreads]
	int32_t *colR; // [m][kThreads]
	uint32_t *recs; // [kWarps][32][rec_words]
	int rec_words;
};

__device__ __forceinline__ Staged stage_tables(const BoundParams &bp, uint8_t *smem)
{
	const uint4 *src = reinterpret_cast<const uint4 *>(bp.tables);
	uint4 *dst = reinterpret_cast<uint4 *>(smem);
	for (uint32_t i = threadIdx.x; i < bp.table_bytes / 16; i += blockDim.x)
		dst[i] = src[i];
	Staged s;
	s.johnson = reinterpret_cast<const uint2 *>(smem);
	s.pt = reinterpret_cast<const int32_t *>(smem + bp.off_pt);
	s.pairs = reinterpret_cast<const int32_t *>(smem + bp.off_pairs);
	s.heads = reinterpret_cast<const int32_t *>(smem + bp.off_heads);
	s.tails = reinterpret_cast<const int32_t *>(smem + bp.off_tails);
	s.colF = reinterpret_cast<int32_t *>(smem + bp.table_bytes);
	s.colR = s.colF + bp.m * kThreads;
	s.recs = reinterpret_cast<uint32_t *>(s.colR + bp.m * kThreads);
	s.rec_words = (bp.stride / 4) | 1; // odd word stride: conflict-free rows
	return s;
}

// Copy records [base, base + nrec) of the pool into this warp's staging rows.
__device__ __forceinline__ void stage_records(const BoundParams &bp, const uint8_t *recs,
                                              int64_t base, int nrec, uint32_t *rows,
                                              int rec_words, int lane)
{
	const int chunks_per_rec = bp.stride / 16;
	const uint4 *src = reinterpret_cast<const uint4 *>(recs + base * bp.stride);
	const int nchunks = nrec * chunks_per_rec;
	for (int c = lane; c < nchunks; c += 32) {
		const uint4 v = __ldg(src + c);
		const int r = c / chunks_per_rec;
		uint32_t *d = rows + r * rec_words + (c - r * chunks_per_rec) * 4;
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

template <int NW, int MAXM>
__global__ void __launch_bounds__(kThreads) lb2_pool_kernel(BoundParams bp,
                                                           const uint8_t *__restrict__ recs,
                                                           int64_t count,
                                                           int32_t *__restrict__ out)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const Staged s = stage_tables(bp, smem);
	__syncthreads();

	const int n = bp.n, m = bp.m, P = bp.P;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	uint32_t *rows = s.recs + warp * 32 * s.rec_words;
	const int64_t step = int64_t(gridDim.x) * kWarps * 32;

	for (int64_t base = (int64_t(blockIdx.x) * kWarps + warp) * 32; base < count;
	     base += step) {
		const int nrec = count - base < 32 ? int(count - base) : 32;
		stage_records(bp, recs, base, nrec, rows, s.rec_words, lane);
		__syncwarp();
		if (lane < nrec) {
			const int16_t *rec = reinterpret_cast<const int16_t *>(rows + lane * s.rec_words);
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
							s.colF[k * kThreads + tid] = l1 >= 0 ? F[k] : s.heads[k];
				}
				{
					int32_t G[MAXM];
					back_times<MAXM>(rec, l2, n, m, s.pt, G);
#pragma unroll
					for (int r = 0; r < MAXM; ++r)
						if (r < m) {
							const int k = m - 1 - r;
							s.colR[k * kThreads + tid] = l2 < n ? G[r] : s.tails[k];
						}
				}
				// With no back jobs the tail is the static tail of the
				// pair's second machine alone (src/bound_flowshop.cpp:147-148).
				const int32_t first_tail_off = l2 < n ? 0 : -(1 << 30);
				const int32_t *cF = s.colF + tid;
				const int32_t *cR = s.colR + tid;
				lb = 0;
				for (int i = 0; i < P; ++i) {
					const int32_t mm = s.pairs[i];
					const int a = mm & 0xff, c = mm >> 8;
					int32_t t0 = cF[a * kThreads], t1 = cF[c * kThreads];
					const uint2 *e = s.johnson + i * n;
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
			out[base + lane] = lb;
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
	const Staged s = stage_tables(bp, smem);
	__syncthreads();
	const int n = bp.n, m = bp.m;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	uint32_t *rows = s.recs + warp * 32 * s.rec_words;
	const int64_t step = int64_t(gridDim.x) * kWarps * 32;
	for (int64_t base = (int64_t(blockIdx.x) * kWarps + warp) * 32; base < count;
	     base += step) {
		const int nrec = count - base < 32 ? int(count - base) : 32;
		stage_records(bp, recs, base, nrec, rows, s.rec_words, lane);
		__syncwarp();
		if (lane < nrec) {
			const int16_t *rec = reinterpret_cast<const int16_t *>(rows + lane * s.rec_words);
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
			out[base + lane] = res;
		}
		__syncwarp();
	}
}

template <typename K>
cudaError_t launch(K kernel, const BoundParams &bp, const void *recs, int64_t count,
                   int32_t *out, int num_sms, cudaStream_t stream)
{
	const size_t smem = pool_bounds_smem(bp, kThreads);
	cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     int(smem));
	if (e != cudaSuccess)
		return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
	if (e != cudaSuccess)
		return e;
	if (per_sm < 1)
		return cudaErrorInvalidConfiguration;
	const int64_t warps_needed = (count + 31) / 32;
	const int64_t blocks_needed = (warps_needed + kWarps - 1) / kWarps;
	const int grid = int(std::max<int64_t>(
	    1, std::min<int64_t>(blocks_needed, int64_t(num_sms) * per_sm)));
	kernel<<<grid, kThreads, smem, stream>>>(bp, static_cast<const uint8_t *>(recs), count,
	                                         out);
	return cudaGetLastError();
}

template <int NW>
cudaError_t launch_lb2_nw(const BoundParams &bp, const void *recs, int64_t count, int32_t *out,
                          int num_sms, cudaStream_t stream)
{
	if (bp.m <= 8)
		return launch(lb2_pool_kernel<NW, 8>, bp, recs, count, out, num_sms, stream);
	if (bp.m <= 16)
		return launch(lb2_pool_kernel<NW, 16>, bp, recs, count, out, num_sms, stream);
	if (bp.m <= 20)
		return launch(lb2_pool_kernel<NW, 20>, bp, recs, count, out, num_sms, stream);
	return launch(lb2_pool_kernel<NW, 32>, bp, recs, count, out, num_sms, stream);
}

}  // namespace

size_t pool_bounds_smem(const BoundParams &bp, int threads)
{
	const size_t rec_words = size_t((bp.stride / 4) | 1);
	return size_t(bp.table_bytes) + 2 * size_t(bp.m) * threads * 4 +
	       size_t(threads) * rec_words * 4;
}

cudaError_t launch_pool_bounds(const BoundParams &bp, const void *recs, int64_t count,
                               int32_t *out, int mode, int num_sms, cudaStream_t stream)
{
	if (count <= 0)
		return cudaSuccess;
	if (mode == 1)
		return launch(aux_pool_kernel<1>, bp, recs, count, out, num_sms, stream);
	if (mode == 2)
		return launch(aux_pool_kernel<2>, bp, recs, count, out, num_sms, stream);
	if (bp.n <= 32)
		return launch_lb2_nw<1>(bp, recs, count, out, num_sms, stream);
	if (bp.n <= 64)
		return launch_lb2_nw<2>(bp, recs, count, out, num_sms, stream);
	return launch_lb2_nw<4>(bp, recs, count, out, num_sms, stream);
}

}  // namespace wsbb
