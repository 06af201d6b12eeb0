// Family bounds: LB2 of every child of a batch of begin-end fathers, one
// father at a time per CTA, from the father alone.
//
// The reference generates both sides of a father and bounds each child
// from scratch (decompose_beginend::operator(),
// src/decompose_beginend.cpp:91-107, calling bound_flowshop::bornes_calculer,
// src/bound_flowshop.cpp:929-951): per child and machine pair a walk over
// the pair's Johnson order of all n jobs (borneInfMakespan, 121-168).
//
// Here the walk is shared by the family. One step of the two-machine
// recurrence on pair (m1, m2),
//     t0 += a_j;  t1 = max(t1, t0 + lag_j) + b_j,
// is the max-plus linear map (t0, t1) -> (t0 + a_j, max(t1 + b_j, t0 + c_j))
// with c_j = a_j + lag_j + b_j, i.e. the lower-triangular max-plus matrix
// [[a_j, -inf], [c_j, b_j]]. A product of such matrices is again
// [[A, -inf], [C, B]] with A = sum a, B = sum b. A child of the father
// frees every job the father frees except the one it moves, so its walk is
// the father's walk with job j left out: suffix(j) x prefix(j), whose C is
//     X_j = max(Csuf + Apre, Bsuf + Cpre).
// One forward and one backward pass over the pair's Johnson order give X_j
// for every free job j. Then the child that moves j, starting from
// (v1, v2) = its front times on m1, m2, ends the walk at
//     t0 = v1 + A - a_j,    t1 = max(v2 + B - b_j, v1 + X_j),
// and the pair's bound is max(t1 + back[m2], t0 + back[m1]) (t1 +
// tails[m2] without back jobs), exactly as the sequential walk gives it:
// max and + are exact on int32 and max-plus products are associative.
// Per child and pair that is a handful of integer operations instead of a
// walk over n jobs.
//
// Fronts and backs: a BEGIN child's front is the father's front followed by
// j, an END child's back is j followed by the father's back; both are one
// max-plus step (over the m machines) from the father's times, which one
// warp computes as a wavefront (lane = machine). A father with two free
// jobs has two leaf children (both orders of the last two jobs), bounded
// by their makespans, max_k(front_k + back_k).
//
// Child order (the search's, make_children_kernel): the u BEGIN children
// (free position l1+1+k moved to the front) then the u END children
// (position l1+1+k moved to the back); two leaves for a simple father.
#include <algorithm>

#include "wsbb_internal.h"

namespace wsbb {
namespace {

constexpr int kFamThreads = 256;
constexpr int32_t kNeg = -(1 << 28); // max-plus -inf, far from any sum of times

__device__ __forceinline__ bool free_bit(const uint32_t (&mask)[4], int job)
{
	return (mask[job >> 5] >> (job & 31)) & 1u;
}

struct FamLayout {
	int xs;        // X row stride (odd: rows of consecutive pairs start in different banks)
	int pc;        // pairs per chunk
	size_t off_pairs, off_V, off_W, off_X, off_AB, off_red, off_F, off_G, off_fr, off_mask, bytes;
};

FamLayout fam_layout(int n, int m, int P, size_t budget)
{
	FamLayout L;
	L.xs = n | 1;
	auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
	size_t off = a16(size_t(m) * n * 4); // pt
	L.off_pairs = off;
	off = a16(off + size_t(P) * 4);
	L.off_V = off;
	off = a16(off + size_t(m) * (n + 1) * 4);
	L.off_W = off;
	off = a16(off + size_t(m) * (n + 1) * 4);
	const size_t fixed_after = a16(kFamThreads * 4) + a16(32 * 4) * 2 + a16((n + 4) * 2) + 16;
	const size_t per_pair = size_t(L.xs) * 4 + 8;
	long long pc = budget > off + fixed_after ? (long long)((budget - off - fixed_after) / per_pair)
	                                          : 0;
	pc = std::max<long long>(pc, 32);
	L.pc = int(std::min<long long>(pc, P));
	L.off_X = off;
	off = a16(off + size_t(L.pc) * L.xs * 4);
	L.off_AB = off;
	off = a16(off + size_t(L.pc) * 8);
	L.off_red = off;
	off = a16(off + kFamThreads * 4);
	L.off_F = off;
	off = a16(off + 32 * 4);
	L.off_G = off;
	off = a16(off + 32 * 4);
	L.off_fr = off;
	off = a16(off + size_t(n + 4) * 2);
	L.off_mask = off;
	off += 16;
	L.bytes = a16(off);
	return L;
}

__global__ void __launch_bounds__(kFamThreads) family_lb2_kernel(FamilyArgs A, BoundParams bp,
                                                                 const uint2 *__restrict__ tjT,
                                                                 FamLayout L)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const long long nf = A.count_dev ? *A.count_dev : A.count;
	if ((long long)blockIdx.x >= nf)
		return;
	const int n = bp.n, m = bp.m, P = bp.P, xs = L.xs;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int32_t *s_pt = reinterpret_cast<int32_t *>(smem);
	int32_t *s_pairs = reinterpret_cast<int32_t *>(smem + L.off_pairs);
	int32_t *s_V = reinterpret_cast<int32_t *>(smem + L.off_V); // [m][n+1] child fronts
	int32_t *s_W = reinterpret_cast<int32_t *>(smem + L.off_W); // [m][n+1] child backs
	int32_t *s_X = reinterpret_cast<int32_t *>(smem + L.off_X); // [pc][xs]
	int2 *s_AB = reinterpret_cast<int2 *>(smem + L.off_AB);     // [pc] (A, B)
	int32_t *s_red = reinterpret_cast<int32_t *>(smem + L.off_red);
	int32_t *s_F = reinterpret_cast<int32_t *>(smem + L.off_F); // father's raw front
	int32_t *s_G = reinterpret_cast<int32_t *>(smem + L.off_G); // father's reversed back
	int16_t *s_fr = reinterpret_cast<int16_t *>(smem + L.off_fr);
	uint32_t *s_mask = reinterpret_cast<uint32_t *>(smem + L.off_mask);
	const uint8_t *tb = bp.t8.blob;
	{
		const int32_t *g_pt = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pt);
		const int32_t *g_pairs = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pairs);
		for (int i = tid; i < m * n; i += kFamThreads)
			s_pt[i] = g_pt[i];
		for (int i = tid; i < P; i += kFamThreads)
			s_pairs[i] = g_pairs[i];
	}
	const int32_t *heads = reinterpret_cast<const int32_t *>(tb + bp.t8.off_heads);
	const int32_t *tails = reinterpret_cast<const int32_t *>(tb + bp.t8.off_tails);

	for (long long f = blockIdx.x; f < nf; f += gridDim.x) {
		const long long ri = A.ridx ? A.ridx[f] : f;
		const int16_t *g_fr = reinterpret_cast<const int16_t *>(A.fathers + ri * A.stride);
		// job ids clamped to [0, n): a malformed record gives wrong bounds,
		// never an access outside the tables
		for (int i = tid; i < n + 2; i += kFamThreads)
			s_fr[i] = i < n ? int16_t(min(max(int(g_fr[i]), 0), n - 1)) : g_fr[i];
		if (tid < 4)
			s_mask[tid] = 0;
		__syncthreads();
		const int l1 = s_fr[n], l2 = s_fr[n + 1];
		const int u = l2 - l1 - 1;
		const long long c0 = A.child_off[f];
		// cursors outside -1 <= l1, l2 <= n with two free jobs or more, or a
		// child range of another size: the father is skipped
		if (l1 < -1 || l2 > n || u < 2 || A.child_off[f + 1] - c0 != (u == 2 ? 2 : 2 * u)) {
			__syncthreads();
			continue;
		}
		if (tid < u)
			atomicOr(&s_mask[s_fr[l1 + 1 + tid] >> 5], 1u << (s_fr[l1 + 1 + tid] & 31));
		// the father's raw front (warp 0) and reversed back (warp 1): a
		// wavefront, lane = machine, lane k takes job s - k at step s
		if (warp == 0) {
			int32_t Fk = 0;
			const int nj = l1 + 1;
			for (int s = 0; s < nj + m - 1; ++s) {
				const int32_t left = __shfl_up_sync(0xffffffffu, Fk, 1);
				const int i = s - lane;
				if (lane < m && i >= 0 && i < nj)
					Fk = max(Fk, lane > 0 ? left : 0) + s_pt[lane * n + s_fr[i]];
			}
			if (lane < m)
				s_F[lane] = Fk;
		} else if (warp == 1) {
			int32_t Gq = 0;
			const int nj = n - l2;
			for (int s = 0; s < nj + m - 1; ++s) {
				const int32_t left = __shfl_up_sync(0xffffffffu, Gq, 1);
				const int i = s - lane;
				if (lane < m && i >= 0 && i < nj)
					Gq = max(Gq, lane > 0 ? left : 0) + s_pt[(m - 1 - lane) * n + s_fr[n - 1 - i]];
			}
			if (lane < m)
				s_G[lane] = Gq;
		}
		__syncthreads();
		if (u == 2) {
			// two leaves: makespan of front + (x, y) + back for both orders
			if (tid < 2) {
				const int x = s_fr[l1 + 1 + tid], y = s_fr[l1 + 2 - tid];
				int32_t v1 = 0, v2 = 0, mk = 0;
				for (int k = 0; k < m; ++k) {
					v1 = max(v1, s_F[k]) + s_pt[k * n + x];
					v2 = max(v2, v1) + s_pt[k * n + y];
					mk = max(mk, v2 + s_G[m - 1 - k]);
				}
				A.child_lb[c0 + tid] = mk;
				A.child_job[c0 + tid] = int16_t(x);
			}
			__syncthreads();
			continue;
		}
		uint32_t mask[4];
#pragma unroll
		for (int w = 0; w < 4; ++w)
			mask[w] = s_mask[w];
		// column n: what the children inherit (front for END children, back
		// for BEGIN children, the static heads / tails when empty); column
		// j: the BEGIN child's front / END child's back that moves job j
		if (tid < m) {
			s_V[tid * (n + 1) + n] = l1 >= 0 ? s_F[tid] : heads[tid];
			s_W[tid * (n + 1) + n] = l2 < n ? s_G[m - 1 - tid] : tails[tid];
		}
		if (tid < u) {
			const int j = s_fr[l1 + 1 + tid];
			int32_t v = 0;
			for (int k = 0; k < m; ++k) {
				v = max(v, s_F[k]) + s_pt[k * n + j];
				s_V[k * (n + 1) + j] = v;
			}
		} else if (tid >= 128 && tid - 128 < u) {
			const int j = s_fr[l1 + 1 + tid - 128];
			int32_t g = 0;
			for (int q = 0; q < m; ++q) {
				g = max(g, s_G[q]) + s_pt[(m - 1 - q) * n + j];
				s_W[(m - 1 - q) * (n + 1) + j] = g;
			}
		}
		// this thread's child and pair slice
		const int nc = 2 * u, nc32 = (nc + 31) & ~31;
		const int S = kFamThreads / nc32;
		const int my_c = tid % nc32, my_s = tid / nc32;
		const bool active = my_s < S && my_c < nc;
		const bool begin = my_c < u;
		const int my_j = active ? s_fr[l1 + 1 + (begin ? my_c : my_c - u)] : 0;
		const int vcol = begin ? my_j : n, rcol = begin ? n : my_j;
		const int32_t toff = (begin && l2 == n) ? kNeg : 0;
		int32_t acc = kNeg;
		for (int p_lo = 0; p_lo < P; p_lo += L.pc) {
			const int len = min(L.pc, P - p_lo);
			__syncthreads(); // fronts / backs written; previous chunk consumed
			for (int t = tid; t < len; t += kFamThreads) {
				const uint2 *e = tjT + p_lo + t;
				int32_t *xrow = s_X + t * xs;
				int32_t a_sum = 0, b_sum = 0, c = kNeg;
				for (int q = 0; q < n; ++q) {
					const uint2 v = __ldg(e + (size_t)q * P);
					const int job = int(v.x & 0xffu);
					if (free_bit(mask, job)) {
						const int32_t a = int32_t(v.x >> 16), b = int32_t(v.y & 0xffffu);
						const int32_t cj = a + int32_t(v.y >> 16) + b;
						xrow[job] = c; // C of the prefix before job
						c = max(c + b, a_sum + cj);
						a_sum += a;
						b_sum += b;
					}
				}
				s_AB[t] = make_int2(a_sum, b_sum);
				int32_t as = 0, bs = 0, cs = kNeg;
				for (int q = n - 1; q >= 0; --q) {
					const uint2 v = __ldg(e + (size_t)q * P);
					const int job = int(v.x & 0xffu);
					if (free_bit(mask, job)) {
						const int32_t a = int32_t(v.x >> 16), b = int32_t(v.y & 0xffffu);
						const int32_t cj = a + int32_t(v.y >> 16) + b;
						const int32_t apre = a_sum - as - a;
						xrow[job] = max(xrow[job] + bs, apre + cs);
						cs = max(cs + a, bs + cj);
						as += a;
						bs += b;
					}
				}
			}
			__syncthreads();
			if (active) {
				const int lo = p_lo + my_s * len / S, hi = p_lo + (my_s + 1) * len / S;
				for (int p = lo; p < hi; ++p) {
					const int pr = s_pairs[p];
					const int m1 = pr & 0xff, m2 = pr >> 8;
					const int2 ab = s_AB[p - p_lo];
					const int32_t x = s_X[(p - p_lo) * xs + my_j];
					const int32_t a = s_pt[m1 * n + my_j], b = s_pt[m2 * n + my_j];
					const int32_t v1 = s_V[m1 * (n + 1) + vcol], v2 = s_V[m2 * (n + 1) + vcol];
					const int32_t r1 = s_W[m1 * (n + 1) + rcol], r2 = s_W[m2 * (n + 1) + rcol];
					const int32_t t0 = v1 + ab.x - a;
					const int32_t t1 = max(v2 + ab.y - b, v1 + x);
					acc = max(acc, max(t1 + r2, t0 + r1 + toff));
				}
			}
		}
		s_red[tid] = acc;
		__syncthreads();
		if (tid < nc) {
			int32_t lb = s_red[tid];
			for (int s = 1; s < S; ++s)
				lb = max(lb, s_red[s * nc32 + tid]);
			A.child_lb[c0 + tid] = lb;
			A.child_job[c0 + tid] = int16_t(s_fr[l1 + 1 + (tid < u ? tid : tid - u)]);
		}
		__syncthreads();
	}
}

}  // namespace

size_t family_smem(const BoundParams &bp)
{
	return fam_layout(bp.n, bp.m, bp.P, 56 * 1024).bytes;
}

cudaError_t launch_family_lb2(const BoundParams &bp, const uint2 *johnsonT, const FamilyArgs &A,
                              long long max_fathers, int num_sms, cudaStream_t s)
{
	if (max_fathers <= 0)
		return cudaSuccess;
	const FamLayout L = fam_layout(bp.n, bp.m, bp.P, 56 * 1024);
	cudaError_t e = cudaFuncSetAttribute(family_lb2_kernel,
	                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.bytes));
	if (e != cudaSuccess)
		return e;
	int occ = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, family_lb2_kernel, kFamThreads,
	                                                  L.bytes);
	if (e != cudaSuccess)
		return e;
	const long long grid = std::min<long long>(max_fathers, (long long)num_sms * std::max(occ, 1));
	family_lb2_kernel<<<unsigned(grid), kFamThreads, L.bytes, s>>>(A, bp, johnsonT, L);
	return cudaGetLastError();
}

}  // namespace wsbb

extern "C" int wsbb_decompose_lb2(wsbb_ctx *ctx, const void *fathers, int64_t count,
                                  const int64_t *child_off, int32_t *child_lb,
                                  int16_t *child_job, void *stream)
{
	if (!ctx)
		return WSBB_ERR_ARG;
	if (count < 0 || (count > 0 && (!fathers || !child_off || !child_lb || !child_job)))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "null buffer or negative count");
	if (count == 0)
		return WSBB_OK;
	cudaError_t e = cudaSetDevice(ctx->device);
	wsbb::FamilyArgs A;
	A.fathers = static_cast<const uint8_t *>(fathers);
	A.count = count;
	A.child_off = reinterpret_cast<const long long *>(child_off);
	A.child_lb = child_lb;
	A.child_job = child_job;
	A.stride = ctx->bp.stride;
	if (e == cudaSuccess)
		e = wsbb::launch_family_lb2(ctx->bp, ctx->tables.johnsonT, A, count, ctx->num_sms,
		                            static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess)
		return wsbb_set_error(ctx, WSBB_ERR_CUDA,
		                      std::string("family bound launch: ") + cudaGetErrorString(e));
	return WSBB_OK;
}
