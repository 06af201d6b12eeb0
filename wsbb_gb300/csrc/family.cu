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
constexpr int kFrontThreads = 64; // warps 0-1: fronts and backs, while the rest walk pairs
constexpr int32_t kNeg = -(1 << 28); // max-plus -inf, far from any sum of times

struct FamLayout {
	int xs; // X row stride (odd: rows of consecutive pairs start in different banks)
	int pc; // pairs per chunk
	size_t off_pairs, off_V, off_W, off_PF, off_PR, off_X, off_PI, off_red, off_F, off_G, off_fr,
	    off_list, off_misc, bytes;
};

FamLayout fam_layout(int n, int m, int P, size_t budget)
{
	FamLayout L;
	L.xs = n | 1;
	auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
	// pt as uint16 (the tables cap times at 65535), rows of n + 1 like V and W
	size_t off = a16(size_t(m) * (n + 1) * 2);
	L.off_pairs = off;
	off = a16(off + size_t(P) * 4);
	L.off_V = off;
	off = a16(off + size_t(m) * (n + 1) * 4);
	L.off_W = off;
	off = a16(off + size_t(m) * (n + 1) * 4);
	L.off_PF = off;
	off = a16(off + size_t(P) * 8);
	L.off_PR = off;
	off = a16(off + size_t(P) * 8);
	const size_t fixed_after = a16(32 * 4) * 2 + a16(size_t(n + 4) * 2) + a16(size_t(2 * n) * 2) + 32;
	const size_t per_pair = size_t(L.xs) * 4 + 16;
	long long pc = budget > off + fixed_after ? (long long)((budget - off - fixed_after) / per_pair)
	                                          : 0;
	pc = std::max<long long>(pc, 32);
	// as few chunks as the budget allows, of equal length (a short last
	// chunk costs a full round of walks and barriers for a few pairs)
	const long long chunks = (P + pc - 1) / pc;
	L.pc = int((P + chunks - 1) / chunks);
	// the per-thread reduction reuses the X rows once the pairs are consumed
	L.off_X = off;
	L.off_red = off;
	off = a16(off + std::max(size_t(L.pc) * L.xs * 4, size_t(2 * kFamThreads * 4)));
	L.off_PI = off;
	off = a16(off + size_t(L.pc) * 16);
	L.off_F = off;
	off = a16(off + 32 * 4);
	L.off_G = off;
	off = a16(off + 32 * 4);
	L.off_fr = off;
	off = a16(off + size_t(n + 4) * 2);
	L.off_list = off;
	off = a16(off + size_t(2 * n) * 2);
	L.off_misc = off;
	off += 32;
	L.bytes = a16(off);
	return L;
}

struct FamSmem {
	uint16_t *pt;
	int32_t *pairs, *V, *W, *X, *red, *F, *G;
	int2 *PF, *PR;
	int4 *PI;
	int16_t *fr, *list;
	uint32_t *mask; // [4] free jobs (scan walks)
	int *cnt;       // [1]
};

__device__ __forceinline__ FamSmem carve(uint8_t *smem, const FamLayout &L)
{
	FamSmem S;
	S.pt = reinterpret_cast<uint16_t *>(smem);
	S.pairs = reinterpret_cast<int32_t *>(smem + L.off_pairs);
	S.V = reinterpret_cast<int32_t *>(smem + L.off_V);
	S.W = reinterpret_cast<int32_t *>(smem + L.off_W);
	S.PF = reinterpret_cast<int2 *>(smem + L.off_PF);
	S.PR = reinterpret_cast<int2 *>(smem + L.off_PR);
	S.X = reinterpret_cast<int32_t *>(smem + L.off_X);
	S.PI = reinterpret_cast<int4 *>(smem + L.off_PI);
	S.red = reinterpret_cast<int32_t *>(smem + L.off_red);
	S.F = reinterpret_cast<int32_t *>(smem + L.off_F);
	S.G = reinterpret_cast<int32_t *>(smem + L.off_G);
	S.fr = reinterpret_cast<int16_t *>(smem + L.off_fr);
	S.list = reinterpret_cast<int16_t *>(smem + L.off_list);
	S.mask = reinterpret_cast<uint32_t *>(smem + L.off_misc);
	S.cnt = reinterpret_cast<int *>(smem + L.off_misc + 16);
	return S;
}

// Warp 0: the father's raw front F (a wavefront, lane = machine: lane k
// takes job s - k at step s), the children's inherited front (column n of
// V: F or the static heads), every BEGIN child's front (column j: F
// followed by job j) and the per-pair (F[m1], F[m2]). Warp 1: the same for
// the reversed back G, W and (back[m1] or -inf without back jobs, back[m2]).
// With `leaves_only`, F and G only.
__device__ __forceinline__ void fronts_and_backs(const FamSmem &S, int warp, int lane, int n,
                                                 int m, int P, int l1, int l2, int u,
                                                 const int32_t *heads, const int32_t *tails,
                                                 bool leaves_only)
{
	const int ld = n + 1;
	if (warp == 0) {
		int32_t Fk = 0;
		const int nj = l1 + 1;
		// the time added at step s is loaded one step ahead, off the chain
		int32_t add = (lane < m && lane == 0 && nj > 0) ? S.pt[S.fr[0]] : 0;
		for (int s = 0; s < nj + m - 1; ++s) {
			const int i = s - lane, i1 = i + 1;
			const int32_t next = (lane < m && i1 >= 0 && i1 < nj) ? S.pt[lane * ld + S.fr[i1]] : 0;
			const int32_t left = __shfl_up_sync(0xffffffffu, Fk, 1);
			if (lane < m && i >= 0 && i < nj)
				Fk = max(Fk, lane > 0 ? left : 0) + add;
			add = next;
		}
		if (lane < m) {
			S.F[lane] = Fk;
			S.V[lane * ld + n] = l1 >= 0 ? Fk : heads[lane];
		}
		if (leaves_only)
			return;
		__syncwarp();
		for (int i = lane; i < u; i += 32) {
			const int j = S.fr[l1 + 1 + i];
			int32_t v = 0;
			for (int k = 0; k < m; ++k) {
				v = max(v, S.F[k]) + S.pt[k * ld + j];
				S.V[k * ld + j] = v;
			}
		}
		for (int p = lane; p < P; p += 32) {
			const int pr = S.pairs[p];
			S.PF[p] = make_int2(S.V[(pr & 0xff) * ld + n], S.V[(pr >> 8) * ld + n]);
		}
	} else if (warp == 1) {
		int32_t Gq = 0;
		const int nj = n - l2;
		int32_t add = (lane < m && lane == 0 && nj > 0) ? S.pt[(m - 1) * ld + S.fr[n - 1]] : 0;
		for (int s = 0; s < nj + m - 1; ++s) {
			const int i = s - lane, i1 = i + 1;
			const int32_t next =
			    (lane < m && i1 >= 0 && i1 < nj) ? S.pt[(m - 1 - lane) * ld + S.fr[n - 1 - i1]] : 0;
			const int32_t left = __shfl_up_sync(0xffffffffu, Gq, 1);
			if (lane < m && i >= 0 && i < nj)
				Gq = max(Gq, lane > 0 ? left : 0) + add;
			add = next;
		}
		if (lane < m)
			S.G[lane] = Gq;
		if (leaves_only)
			return;
		__syncwarp();
		if (lane < m)
			S.W[lane * ld + n] = l2 < n ? S.G[m - 1 - lane] : tails[lane];
		for (int i = lane; i < u; i += 32) {
			const int j = S.fr[l1 + 1 + i];
			int32_t g = 0;
			for (int q = 0; q < m; ++q) {
				g = max(g, S.G[q]) + S.pt[(m - 1 - q) * ld + j];
				S.W[(m - 1 - q) * ld + j] = g;
			}
		}
		__syncwarp();
		for (int p = lane; p < P; p += 32) {
			const int pr = S.pairs[p];
			const int32_t r1 = S.W[(pr & 0xff) * ld + n];
			S.PR[p] = make_int2(l2 < n ? r1 : kNeg, S.W[(pr >> 8) * ld + n]);
		}
	}
}

constexpr int kWalkBatch = 4;

// The next free position of a pair's Johnson order (ascending or
// descending) from its free-position mask (w0: positions 0-63, w1: 64-127);
// -1 when none is left.
template <bool kWide>
__device__ __forceinline__ int next_up(uint64_t &w0, uint64_t &w1)
{
	if (w0) {
		const int q = __ffsll((long long)w0) - 1;
		w0 &= w0 - 1;
		return q;
	}
	if (kWide && w1) {
		const int q = __ffsll((long long)w1) - 1;
		w1 &= w1 - 1;
		return 64 + q;
	}
	return -1;
}

template <bool kWide>
__device__ __forceinline__ int next_down(uint64_t &w0, uint64_t &w1)
{
	if (kWide && w1) {
		const int q = 63 - __clzll((long long)w1);
		w1 ^= 1ull << q;
		return 64 + q;
	}
	if (w0) {
		const int q = 63 - __clzll((long long)w0);
		w0 ^= 1ull << q;
		return q;
	}
	return -1;
}

template <bool kWide>
__device__ __forceinline__ bool free_bit(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3,
                                         int job)
{
	const uint32_t lo = (job & 32) ? w1 : w0;
	if (!kWide) // n <= 64
		return ((lo >> (job & 31)) & 1u) != 0;
	const uint32_t hi = (job & 32) ? w3 : w2;
	return ((((job & 64) ? hi : lo) >> (job & 31)) & 1u) != 0;
}

constexpr int kScanBatch = 8;

// The same passes as walk_pair below, scanning all n positions of the
// order and skipping the fixed jobs (free-job mask w0..w3): cheaper than
// the position-table walk when almost every job is free.
template <bool kWide>
__device__ __forceinline__ void scan_pair(const FamSmem &S, const uint2 *__restrict__ tjT, int p,
                                          int slot, int n, int P, int xs, uint32_t w0,
                                          uint32_t w1, uint32_t w2, uint32_t w3)
{
	const uint2 *e = tjT + p;
	int32_t *xrow = S.X + slot * xs;
	int32_t a_sum = 0, b_sum = 0, c = kNeg;
	for (int q0 = 0; q0 < n; q0 += kScanBatch) {
		uint2 v[kScanBatch];
#pragma unroll
		for (int k = 0; k < kScanBatch; ++k)
			v[k] = q0 + k < n ? __ldg(e + (size_t)(q0 + k) * P) : make_uint2(0u, 0u);
#pragma unroll
		for (int k = 0; k < kScanBatch; ++k) {
			const int job = int(v[k].x & 0xffu);
			if (q0 + k < n && free_bit<kWide>(w0, w1, w2, w3, job)) {
				const int32_t a = int32_t(v[k].x >> 16), b = int32_t(v[k].y & 0xffffu);
				const int32_t cj = int32_t(v[k].y >> 16);
				xrow[job] = c;
				c = max(c + b, a_sum + cj);
				a_sum += a;
				b_sum += b;
			}
		}
	}
	const int pr = S.pairs[p], ld = n + 1;
	S.PI[slot] = make_int4((pr & 0xff) * ld | ((pr >> 8) * ld) << 16, a_sum, b_sum, p);
	int32_t as = 0, bs = 0, cs = kNeg;
	for (int q0 = n - 1; q0 >= 0; q0 -= kScanBatch) {
		uint2 v[kScanBatch];
#pragma unroll
		for (int k = 0; k < kScanBatch; ++k)
			v[k] = q0 - k >= 0 ? __ldg(e + (size_t)(q0 - k) * P) : make_uint2(0u, 0u);
#pragma unroll
		for (int k = 0; k < kScanBatch; ++k) {
			const int job = int(v[k].x & 0xffu);
			if (q0 - k >= 0 && free_bit<kWide>(w0, w1, w2, w3, job)) {
				const int32_t a = int32_t(v[k].x >> 16), b = int32_t(v[k].y & 0xffffu);
				const int32_t cj = int32_t(v[k].y >> 16);
				const int32_t apre = a_sum - as - a;
				xrow[job] = max(xrow[job] + bs, apre + cs);
				cs = max(cs + a, bs + cj);
				as += a;
				bs += b;
			}
		}
	}
}

// Pair p's forward and backward max-plus passes over its Johnson order,
// restricted to the father's u free jobs `fj`: X[slot][j] = C of (suffix
// after j) x (prefix before j), and PI[slot] = (m1 (n+1) | m2 (n+1) << 16,
// A, B, p): the row offsets of the pair's machines in pt, V and W. The
// free positions come from the job-position table (u lookups, not a scan
// of all n positions), so both passes touch only the u free entries.
template <bool kWide>
__device__ __forceinline__ void walk_pair(const FamSmem &S, const uint2 *__restrict__ tjT,
                                          const uint8_t *__restrict__ jobposT, int p, int slot,
                                          int n, int P, int xs, const int16_t *fj, int u)
{
	uint64_t m0 = 0, m1 = 0;
#pragma unroll 8
	for (int i = 0; i < u; ++i) {
		const int q = __ldg(jobposT + (size_t)fj[i] * P + p);
		if (kWide) {
			const uint64_t bit = 1ull << (q & 63);
			m0 |= q < 64 ? bit : 0ull;
			m1 |= q < 64 ? 0ull : bit;
		} else {
			m0 |= 1ull << q;
		}
	}
	const uint2 *e = tjT + p;
	int32_t *xrow = S.X + slot * xs;
	int32_t a_sum = 0, b_sum = 0, c = kNeg;
	uint64_t w0 = m0, w1 = m1;
	for (int left = u; left > 0; left -= kWalkBatch) {
		int q[kWalkBatch];
		uint2 v[kWalkBatch];
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k)
			q[k] = next_up<kWide>(w0, w1);
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k)
			v[k] = q[k] >= 0 ? __ldg(e + (size_t)q[k] * P) : make_uint2(0u, 0u);
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k) {
			if (q[k] >= 0) {
				const int job = int(v[k].x & 0xffu);
				const int32_t a = int32_t(v[k].x >> 16), b = int32_t(v[k].y & 0xffffu);
				const int32_t cj = int32_t(v[k].y >> 16); // a + lag + b
				xrow[job] = c; // C of the prefix before job
				c = max(c + b, a_sum + cj);
				a_sum += a;
				b_sum += b;
			}
		}
	}
	const int pr = S.pairs[p], ld = n + 1;
	S.PI[slot] = make_int4((pr & 0xff) * ld | ((pr >> 8) * ld) << 16, a_sum, b_sum, p);
	int32_t as = 0, bs = 0, cs = kNeg;
	w0 = m0;
	w1 = m1;
	for (int left = u; left > 0; left -= kWalkBatch) {
		int q[kWalkBatch];
		uint2 v[kWalkBatch];
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k)
			q[k] = next_down<kWide>(w0, w1);
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k)
			v[k] = q[k] >= 0 ? __ldg(e + (size_t)q[k] * P) : make_uint2(0u, 0u);
#pragma unroll
		for (int k = 0; k < kWalkBatch; ++k) {
			if (q[k] >= 0) {
				const int job = int(v[k].x & 0xffu);
				const int32_t a = int32_t(v[k].x >> 16), b = int32_t(v[k].y & 0xffffu);
				const int32_t cj = int32_t(v[k].y >> 16);
				const int32_t apre = a_sum - as - a;
				xrow[job] = max(xrow[job] + bs, apre + cs);
				cs = max(cs + a, bs + cj);
				as += a;
				bs += b;
			}
		}
	}
}

// Both children that move job j (BEGIN and END) over chunk slots [lo, hi).
__device__ __forceinline__ void job_pairs(const FamSmem &S, int lo, int hi, int j, int xs,
                                          int32_t &accB, int32_t &accE)
{
	const int32_t *xp = S.X + lo * xs + j;
	for (int t = lo; t < hi; ++t, xp += xs) {
		const int4 pi = S.PI[t];
		const int o1 = (pi.x & 0xffff) + j, o2 = (int(unsigned(pi.x) >> 16)) + j;
		const int2 pf = S.PF[pi.w], pr = S.PR[pi.w];
		const int32_t x = *xp;
		const int32_t aa = pi.y - int32_t(S.pt[o1]), bb = pi.z - int32_t(S.pt[o2]);
		// BEGIN child: front V[.][j], the father's back
		const int32_t v1 = S.V[o1], v2 = S.V[o2];
		const int32_t t0 = v1 + aa, t1 = max(v2 + bb, v1 + x);
		accB = max(accB, max(t1 + pr.y, t0 + pr.x));
		// END child: the father's front, back W[.][j]
		const int32_t w1 = S.W[o1], w2 = S.W[o2];
		const int32_t e0 = pf.x + aa, e1 = max(pf.y + bb, pf.x + x);
		accE = max(accE, max(e1 + w2, e0 + w1));
	}
}

// One child (c < u: BEGIN, else END) over chunk slots [lo, hi).
__device__ __forceinline__ int32_t child_pairs(const FamSmem &S, int lo, int hi, int j,
                                               bool begin, int xs, int32_t acc)
{
	const int32_t *xp = S.X + lo * xs + j;
	for (int t = lo; t < hi; ++t, xp += xs) {
		const int4 pi = S.PI[t];
		const int o1 = (pi.x & 0xffff) + j, o2 = (int(unsigned(pi.x) >> 16)) + j;
		const int32_t x = *xp;
		const int32_t aa = pi.y - int32_t(S.pt[o1]), bb = pi.z - int32_t(S.pt[o2]);
		const int2 pf = S.PF[pi.w], pr = S.PR[pi.w];
		// BEGIN: own front, the father's back; END: the father's front, own back
		const int32_t v1 = begin ? S.V[o1] : pf.x, v2 = begin ? S.V[o2] : pf.y;
		const int32_t r1 = begin ? pr.x : S.W[o1], r2 = begin ? pr.y : S.W[o2];
		const int32_t t0 = v1 + aa, t1 = max(v2 + bb, v1 + x);
		acc = max(acc, max(t1 + r2, t0 + r1));
	}
	return acc;
}

// kLearned: the father's K ranked pairs first; a child whose bound over
// them reaches max(best, incumbent) is settled with that value (the search
// only compares such bounds with the thresholds, never ranks or sums
// them); fathers with children left walk every pair for those children.
template <bool kLearned, bool kWide>
__global__ void __launch_bounds__(kFamThreads, 4) family_kernel(FamilyArgs A, BoundParams bp,
                                                             const uint2 *__restrict__ tjT,
                                                             const uint8_t *__restrict__ jobposT,
                                                             FamLayout L)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const long long nf = A.count_dev ? *A.count_dev : A.count;
	if ((long long)blockIdx.x >= nf)
		return;
	const int n = bp.n, m = bp.m, P = bp.P, xs = L.xs;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const FamSmem S = carve(smem, L);
	const uint8_t *tb = bp.t8.blob;
	{
		const int32_t *g_pt = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pt);
		const int32_t *g_pairs = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pairs);
		for (int i = tid; i < m * n; i += kFamThreads)
			S.pt[(i / n) * (n + 1) + i % n] = uint16_t(g_pt[i]);
		for (int i = tid; i < P; i += kFamThreads)
			S.pairs[i] = g_pairs[i];
	}
	const int32_t *heads = reinterpret_cast<const int32_t *>(tb + bp.t8.off_heads);
	const int32_t *tails = reinterpret_cast<const int32_t *>(tb + bp.t8.off_tails);
	const int thr = kLearned ? max(*A.best_dev, *A.ub_dev) : 0;
	const int K = kLearned ? min(A.K, P) : 0;

	// fathers: the CTA's own first, then the next unclaimed one from the
	// device counter (A.next, zero at launch), so CTAs that drew light
	// fathers take more and none idles at the tail; without a counter,
	// every gridDim.x-th father
	__shared__ long long s_next;
	for (long long f = blockIdx.x; f < nf;) {
		do {
			const long long ri = A.ridx ? A.ridx[f] : f;
			const int16_t *g_fr = reinterpret_cast<const int16_t *>(A.fathers + ri * A.stride);
			// job ids clamped to [0, n): a malformed record gives wrong bounds,
			// never an access outside the tables
			for (int i = tid; i < n + 2; i += kFamThreads)
				S.fr[i] = i < n ? int16_t(min(max(int(g_fr[i]), 0), n - 1)) : g_fr[i];
			if (tid == 4)
				*S.cnt = 0;
			__syncthreads();
			const int l1 = S.fr[n], l2 = S.fr[n + 1];
			const int u = l2 - l1 - 1;
			const long long c0 = A.child_off[f];
			// cursors outside -1 <= l1, l2 <= n with two free jobs or more, or a
			// child range of another size: the father is skipped
			if (l1 < -1 || l2 > n || u < 2 || A.child_off[f + 1] - c0 != (u == 2 ? 2 : 2 * u)) {
				__syncthreads();
				continue;
			}
			if (u == 2) {
				// two leaves: makespans of front + (x, y) + back, both orders
				fronts_and_backs(S, warp, lane, n, m, P, l1, l2, u, heads, tails, true);
				__syncthreads();
				if (tid < 2) {
					const int x = S.fr[l1 + 1 + tid], y = S.fr[l1 + 2 - tid];
					int32_t v1 = 0, v2 = 0, mk = 0;
					for (int k = 0; k < m; ++k) {
						v1 = max(v1, S.F[k]) + S.pt[k * (n + 1) + x];
						v2 = max(v2, v1) + S.pt[k * (n + 1) + y];
						mk = max(mk, v2 + S.G[m - 1 - k]);
					}
					A.child_lb[c0 + tid] = mk;
					A.child_job[c0 + tid] = int16_t(x);
				}
				__syncthreads();
				continue;
			}
			const int16_t *fj = S.fr + l1 + 1; // the father's free jobs
			// walks: scan all n positions when most jobs are free (more than
			// 3/4, or half for n > 64 where the position masks take two
			// words), else follow the position table over the free ones only
			const bool scan = kWide ? 2 * u > n : 4 * u > 3 * n;
			if (scan) {
				if (tid < 4)
					S.mask[tid] = 0;
				__syncthreads();
				if (tid < u)
					atomicOr(&S.mask[fj[tid] >> 5], 1u << (fj[tid] & 31));
				__syncthreads();
			}
			const uint32_t w0 = S.mask[0], w1 = S.mask[1], w2 = S.mask[2], w3 = S.mask[3];
			// first chunk: the K ranked pairs (learned) or pairs [0, pc); its
			// walks overlap the fronts and backs
			const int len0 = kLearned ? K : min(L.pc, P);
			if (tid < kFrontThreads) {
				fronts_and_backs(S, warp, lane, n, m, P, l1, l2, u, heads, tails, false);
			} else {
				for (int t = tid - kFrontThreads; t < len0; t += kFamThreads - kFrontThreads) {
					int p = t;
					if (kLearned)
						p = min(max(int(A.fpairs[f * A.K + t]), 0), P - 1);
					if (scan)
						scan_pair<kWide>(S, tjT, p, t, n, P, xs, w0, w1, w2, w3);
					else
						walk_pair<kWide>(S, tjT, jobposT, p, t, n, P, xs, fj, u);
				}
			}
			// per job: one thread per (job, slice of the chunk's pairs) takes
			// both children that move the job
			const int u32 = (u + 31) & ~31, NS = kFamThreads / u32;
			const int my_i = tid % u32, my_s = tid / u32;
			const bool active = my_s < NS && my_i < u;
			const int my_j = active ? S.fr[l1 + 1 + my_i] : 0;
			int32_t accB = kNeg, accE = kNeg;
			__syncthreads();
			if (active)
				job_pairs(S, my_s * len0 / NS, (my_s + 1) * len0 / NS, my_j, xs, accB, accE);
			if (!kLearned) {
				for (int p_lo = len0; p_lo < P; p_lo += L.pc) {
					const int len = min(L.pc, P - p_lo);
					__syncthreads(); // previous chunk consumed
					for (int t = tid; t < len; t += kFamThreads)
						{
						if (scan)
							scan_pair<kWide>(S, tjT, p_lo + t, t, n, P, xs, w0, w1, w2, w3);
						else
							walk_pair<kWide>(S, tjT, jobposT, p_lo + t, t, n, P, xs, fj, u);
					}
					__syncthreads();
					if (active)
						job_pairs(S, my_s * len / NS, (my_s + 1) * len / NS, my_j, xs, accB, accE);
				}
			}
			__syncthreads(); // the reduction overwrites the X rows
			S.red[2 * tid] = accB;
			S.red[2 * tid + 1] = accE;
			__syncthreads();
			if (tid < u) {
				int32_t lbB = S.red[2 * tid], lbE = S.red[2 * tid + 1];
				for (int s = 1; s < NS; ++s) {
					lbB = max(lbB, S.red[2 * (s * u32 + tid)]);
					lbE = max(lbE, S.red[2 * (s * u32 + tid) + 1]);
				}
				const int16_t job = S.fr[l1 + 1 + tid];
				A.child_job[c0 + tid] = job;
				A.child_job[c0 + u + tid] = job;
				if (!kLearned) {
					A.child_lb[c0 + tid] = lbB;
					A.child_lb[c0 + u + tid] = lbE;
				} else {
					// settled children keep the bound over the K pairs
					if (lbB >= thr)
						A.child_lb[c0 + tid] = lbB;
					else
						S.list[atomicAdd(S.cnt, 1)] = int16_t(tid);
					if (lbE >= thr)
						A.child_lb[c0 + u + tid] = lbE;
					else
						S.list[atomicAdd(S.cnt, 1)] = int16_t(u + tid);
				}
			}
			if (kLearned) {
				__syncthreads();
				const int nu = *S.cnt;
				if (tid == 0 && 2 * u - nu > 0)
					atomicAdd(A.early, (unsigned long long)(2 * u - nu));
				if (tid == 0 && nu == 0 && A.settled_fathers)
					atomicAdd(A.settled_fathers, 1ull);
				if (nu > 0) {
					// the children left: every pair
					const int nu32 = (nu + 31) & ~31, NS2 = kFamThreads / nu32;
					const int ci = tid % nu32, cs = tid / nu32;
					const bool act2 = cs < NS2 && ci < nu;
					const int c = act2 ? S.list[ci] : 0;
					const bool begin = c < u;
					const int j = S.fr[l1 + 1 + (begin ? c : c - u)];
					int32_t acc = kNeg;
					for (int p_lo = 0; p_lo < P; p_lo += L.pc) {
						const int len = min(L.pc, P - p_lo);
						__syncthreads();
						for (int t = tid; t < len; t += kFamThreads)
							{
						if (scan)
							scan_pair<kWide>(S, tjT, p_lo + t, t, n, P, xs, w0, w1, w2, w3);
						else
							walk_pair<kWide>(S, tjT, jobposT, p_lo + t, t, n, P, xs, fj, u);
					}
						__syncthreads();
						if (act2)
							acc = child_pairs(S, cs * len / NS2, (cs + 1) * len / NS2, j, begin, xs,
							                  acc);
					}
					__syncthreads();
					S.red[tid] = acc;
					__syncthreads();
					if (tid < nu) {
						int32_t lb = S.red[tid];
						for (int s = 1; s < NS2; ++s)
							lb = max(lb, S.red[s * nu32 + tid]);
						A.child_lb[c0 + S.list[tid]] = lb;
					}
				}
			}
			__syncthreads();
		} while (0);
		// claim the next father (every thread reads the same value)
		if (tid == 0)
			s_next = A.next ? (long long)gridDim.x + (long long)atomicAdd(A.next, 1ull)
			                : f + gridDim.x;
		__syncthreads();
		f = s_next;
		__syncthreads();
	}
}

}  // namespace

size_t family_smem(const BoundParams &bp, int smem_kb)
{
	return fam_layout(bp.n, bp.m, bp.P, size_t(smem_kb > 0 ? smem_kb : 56) * 1024).bytes;
}

cudaError_t launch_family_lb2(const BoundParams &bp, const DeviceTables &T, const FamilyArgs &A,
                              long long max_fathers, int num_sms, cudaStream_t s, int smem_kb)
{
	if (max_fathers <= 0)
		return cudaSuccess;
	const size_t budget = size_t(std::min(std::max(smem_kb > 0 ? smem_kb : 56, 16), 220)) * 1024;
	const FamLayout L = fam_layout(bp.n, bp.m, bp.P, budget);
	const bool learned = A.fpairs != nullptr;
	const bool wide = bp.n > 64;
	auto kern = learned ? (wide ? family_kernel<true, true> : family_kernel<true, false>)
	                    : (wide ? family_kernel<false, true> : family_kernel<false, false>);
	cudaError_t e = allow_max_dynamic_smem(kern);
	if (e != cudaSuccess)
		return e;
	int occ = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kFamThreads, L.bytes);
	if (e != cudaSuccess)
		return e;
	const long long grid = std::min<long long>(max_fathers, (long long)num_sms * std::max(occ, 1));
	kern<<<unsigned(grid), kFamThreads, L.bytes, s>>>(A, bp, T.johnsonT, T.jobposT, L);
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
	A.next = ctx->d_claim;
	if (e == cudaSuccess && ctx->d_claim)
		e = cudaMemsetAsync(ctx->d_claim, 0, sizeof(unsigned long long),
		                    static_cast<cudaStream_t>(stream));
	if (e == cudaSuccess)
		e = wsbb::launch_family_lb2(ctx->bp, ctx->tables, A, count, ctx->num_sms,
		                            static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess)
		return wsbb_set_error(ctx, WSBB_ERR_CUDA,
		                      std::string("family bound launch: ") + cudaGetErrorString(e));
	return WSBB_OK;
}
