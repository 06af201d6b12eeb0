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
//
// Work split in a CTA (one father at a time): warps 0-1 compute the fronts
// and backs while warps 2-7 run the forward pass of each pair (thread per
// pair); after a barrier the same threads run the backward pass, and at
// job j, the moment X_j is known, bound both children that move j for the
// pair and store the two values in the pair's row (column j). A last
// sweep takes, per child, the maximum over the rows. With no back jobs the
// reference's pair value is t1 + tails[m2]; here the back term of m1 is 0,
// which gives the same maximum because t0 <= t1 once one job has been
// walked (t1 >= t0 + lag + b after every step) and tails >= 0. Every value
// is then a staircase-path length of some permutation, at most
// (n + m - 1) * max p, so when that fits 16 bits both children's values
// share one 32-bit slot (BoundParams::span16) and the sweep is one
// two-halves max per slot.
#include <algorithm>

#include "family_staged.cuh"
#include "wsbb_internal.h"

namespace wsbb {
namespace {

constexpr int kFamThreads = 256;
constexpr int kFrontThreads = 64; // warps 0-1: fronts and backs, while the rest walk pairs
constexpr int kWalkThreads = kFamThreads - kFrontThreads;
constexpr int32_t kNeg = -(1 << 28); // max-plus -inf, far from any sum of times

// One X slot: the forward pass leaves C of the prefix before the job there;
// the backward pass replaces it with the bounds of the job's BEGIN and END
// children for the pair.
template <bool k16>
struct Slot;
template <>
struct Slot<true> { // both bounds as uint16 halves (BEGIN low, END high)
	using T = uint32_t;
	static __device__ __forceinline__ T pre(int32_t c) { return uint32_t(c); }
	static __device__ __forceinline__ int32_t pre_of(T s) { return int32_t(s); }
	static __device__ __forceinline__ T pack(int32_t b, int32_t e)
	{
		return __byte_perm(uint32_t(b), uint32_t(e), 0x5410);
	}
	static __device__ __forceinline__ T none() { return 0u; } // every bound is >= 0
	static __device__ __forceinline__ T vmax(T a, T b) { return __vmaxu2(a, b); }
	static __device__ __forceinline__ int32_t begin(T s) { return int32_t(s & 0xffffu); }
	static __device__ __forceinline__ int32_t end(T s) { return int32_t(s >> 16); }
};
template <>
struct Slot<false> {
	using T = int2;
	static __device__ __forceinline__ T pre(int32_t c) { return make_int2(c, 0); }
	static __device__ __forceinline__ int32_t pre_of(T s) { return s.x; }
	static __device__ __forceinline__ T pack(int32_t b, int32_t e) { return make_int2(b, e); }
	static __device__ __forceinline__ T none() { return make_int2(kNeg, kNeg); }
	static __device__ __forceinline__ T vmax(T a, T b)
	{
		return make_int2(max(a.x, b.x), max(a.y, b.y));
	}
	static __device__ __forceinline__ int32_t begin(T s) { return s.x; }
	static __device__ __forceinline__ int32_t end(T s) { return s.y; }
};

struct FamLayout {
	int xs;   // X row stride in slots (odd: rows of consecutive pairs start in different banks)
	int pc;   // pairs per chunk
	int slot; // bytes per X slot (4: packed 16-bit bounds, 8: int32 bounds)
	size_t off_pairs, off_VW, off_PFR, off_X, off_PI, off_red, off_F, off_G, off_fr, off_misc,
	    bytes;
};

FamLayout fam_layout(int n, int m, int P, size_t budget, bool pack16)
{
	FamLayout L;
	L.xs = n | 1;
	L.slot = pack16 ? 4 : 8;
	auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
	// pt as uint16 (the tables cap times at 65535), rows of n + 1 like V and W
	size_t off = a16(size_t(m) * (n + 1) * 2);
	L.off_pairs = off;
	off = a16(off + size_t(P) * 4);
	L.off_VW = off;
	off = a16(off + size_t(m) * (n + 1) * 8);
	L.off_PFR = off;
	off = a16(off + size_t(P) * 16);
	const size_t fixed_after = a16(32 * 4) * 2 + a16(size_t(n + 4) * 2) + 32;
	const size_t per_pair = size_t(L.xs) * L.slot + 16;
	long long pc = budget > off + fixed_after ? (long long)((budget - off - fixed_after) / per_pair)
	                                          : 0;
	pc = std::max<long long>(pc, 32);
	// as few chunks as the budget allows, of equal length (a short last
	// chunk costs a full round of walks and barriers for a few pairs)
	const long long chunks = (P + pc - 1) / pc;
	L.pc = int((P + chunks - 1) / chunks);
	// the cross-slice reduction reuses the X rows once the chunk is consumed
	L.off_X = off;
	L.off_red = off;
	off = a16(off + std::max(size_t(L.pc) * L.xs, size_t(kFamThreads)) * L.slot);
	L.off_PI = off;
	off = a16(off + size_t(L.pc) * 16);
	L.off_F = off;
	off = a16(off + 32 * 4);
	L.off_G = off;
	off = a16(off + 32 * 4);
	L.off_fr = off;
	off = a16(off + size_t(n + 4) * 2);
	L.off_misc = off;
	off += 32;
	L.bytes = a16(off);
	return L;
}

struct FamSmem {
	uint16_t *pt;
	int32_t *pairs, *F, *G;
	// per (machine k, column j): (V, W) = the front of the BEGIN child that
	// moves job j and the back of the END child that moves it (column n:
	// the father's own front, or the heads, and back, or the tails)
	int2 *VW;
	int4 *PFR; // per pair: the father's front (m1, m2) and back (m1, m2) times
	int4 *PI;  // per chunk slot: (m1 (n+1) | m2 (n+1) << 16, A, B, pair)
	uint8_t *X, *red;
	int16_t *fr;
	uint32_t *mask; // [4] free jobs (scan walks)
	int *cnt;       // [1]
};

__device__ __forceinline__ FamSmem carve(uint8_t *smem, const FamLayout &L)
{
	FamSmem S;
	S.pt = reinterpret_cast<uint16_t *>(smem);
	S.pairs = reinterpret_cast<int32_t *>(smem + L.off_pairs);
	S.VW = reinterpret_cast<int2 *>(smem + L.off_VW);
	S.PFR = reinterpret_cast<int4 *>(smem + L.off_PFR);
	S.X = smem + L.off_X;
	S.PI = reinterpret_cast<int4 *>(smem + L.off_PI);
	S.red = smem + L.off_red;
	S.F = reinterpret_cast<int32_t *>(smem + L.off_F);
	S.G = reinterpret_cast<int32_t *>(smem + L.off_G);
	S.fr = reinterpret_cast<int16_t *>(smem + L.off_fr);
	S.mask = reinterpret_cast<uint32_t *>(smem + L.off_misc);
	S.cnt = reinterpret_cast<int *>(smem + L.off_misc + 16);
	return S;
}

// Warp 0: the father's raw front F (a wavefront, lane = machine: lane k
// takes job s - k at step s), the children's inherited front (column n of
// V: F or the static heads), every BEGIN child's front (column j: F
// followed by job j) and the per-pair front (F[m1], F[m2]). Warp 1: the
// same for the reversed back G, W and the per-pair back (back[m1], or 0
// without back jobs, and back[m2]). With `leaves_only`, F and G only.
__device__ __forceinline__ void fronts_and_backs(const FamSmem &S, int warp, int lane, int n,
                                                 int m, int P, int l1, int l2, int u,
                                                 const int32_t *heads, const int32_t *tails,
                                                 bool leaves_only)
{
	const int ld = n + 1;
	int2 *pfr = reinterpret_cast<int2 *>(S.PFR);
	// warp 0 writes the V halves, warp 1 the W halves
	int32_t *V = reinterpret_cast<int32_t *>(S.VW), *W = V + 1;
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
			V[2 * (lane * ld + n)] = l1 >= 0 ? Fk : heads[lane];
		}
		if (leaves_only)
			return;
		__syncwarp();
		for (int i = lane; i < u; i += 32) {
			const int j = S.fr[l1 + 1 + i];
			int32_t v = 0;
			for (int k = 0; k < m; ++k) {
				v = max(v, S.F[k]) + S.pt[k * ld + j];
				V[2 * (k * ld + j)] = v;
			}
		}
		for (int p = lane; p < P; p += 32) {
			const int pr = S.pairs[p];
			pfr[2 * p] = make_int2(V[2 * ((pr & 0xff) * ld + n)], V[2 * ((pr >> 8) * ld + n)]);
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
			W[2 * (lane * ld + n)] = l2 < n ? S.G[m - 1 - lane] : tails[lane];
		for (int i = lane; i < u; i += 32) {
			const int j = S.fr[l1 + 1 + i];
			int32_t g = 0;
			for (int q = 0; q < m; ++q) {
				g = max(g, S.G[q]) + S.pt[(m - 1 - q) * ld + j];
				W[2 * ((m - 1 - q) * ld + j)] = g;
			}
		}
		__syncwarp();
		for (int p = lane; p < P; p += 32) {
			const int pr = S.pairs[p];
			const int32_t r1 = W[2 * ((pr & 0xff) * ld + n)];
			pfr[2 * p + 1] = make_int2(l2 < n ? r1 : 0, W[2 * ((pr >> 8) * ld + n)]);
		}
	}
}

constexpr int kWalkBatch = 4;
constexpr int kScanBatch = 8;

// The next free position of a pair's Johnson order (ascending or
// descending) from its free-position mask (w0: positions 0-63, w1: 64-127);
// -1 when none is left. For n <= 64 the mask is taken as two 32-bit words.
template <bool kWide>
__device__ __forceinline__ int next_up(uint64_t &w0, uint64_t &w1)
{
	if (!kWide) {
		uint32_t lo = uint32_t(w0), hi = uint32_t(w0 >> 32);
		int q = -1;
		if (lo) {
			q = __ffs(lo) - 1;
			lo &= lo - 1;
		} else if (hi) {
			q = 31 + __ffs(hi);
			hi &= hi - 1;
		}
		w0 = (uint64_t(hi) << 32) | lo;
		return q;
	}
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
	if (!kWide) {
		uint32_t lo = uint32_t(w0), hi = uint32_t(w0 >> 32);
		int q = -1;
		if (hi) {
			const int b = 31 - __clz(hi);
			hi ^= 1u << b;
			q = 32 + b;
		} else if (lo) {
			q = 31 - __clz(lo);
			lo ^= 1u << q;
		}
		w0 = (uint64_t(hi) << 32) | lo;
		return q;
	}
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
__device__ __forceinline__ bool free_bit(const uint32_t *w, int job)
{
	return ((w[(kWide ? job & 127 : job & 63) >> 5] >> (job & 31)) & 1u) != 0;
}

// Positions of the father's free jobs in pair p's Johnson order, as a mask
// (u lookups in the job-position table).
template <bool kWide>
__device__ __forceinline__ void walk_mask(const uint8_t *__restrict__ jobposT, const int16_t *fj,
                                          int u, int p, int P, uint64_t &m0, uint64_t &m1)
{
	m0 = 0;
	m1 = 0;
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
}

// body(entry) for each of the father's free jobs in a pair's Johnson order
// (entries e[q * P], q = position), ascending (kUp) or descending. Walk
// form: the set bits of the position mask (m0, m1), u of them. Scan form:
// all n positions, keeping the entries whose job is in the free-job mask w
// (cheaper when almost every job is free).
template <bool kUp, bool kScan, bool kWide, typename Body>
__device__ __forceinline__ void each_free(const uint2 *__restrict__ e, int n, int P, int u,
                                          uint64_t m0, uint64_t m1, const uint32_t *w,
                                          Body &&body)
{
	if (kScan) {
		for (int k0 = 0; k0 < n; k0 += kScanBatch) {
			uint2 v[kScanBatch];
#pragma unroll
			for (int k = 0; k < kScanBatch; ++k) {
				const int q = kUp ? k0 + k : n - 1 - k0 - k;
				v[k] = k0 + k < n ? __ldg(e + (size_t)q * P) : make_uint2(0u, 0u);
			}
#pragma unroll
			for (int k = 0; k < kScanBatch; ++k)
				if (k0 + k < n && free_bit<kWide>(w, int(v[k].x & 0xffu)))
					body(v[k]);
		}
	} else {
		for (int left = u; left > 0; left -= kWalkBatch) {
			int q[kWalkBatch];
			uint2 v[kWalkBatch];
#pragma unroll
			for (int k = 0; k < kWalkBatch; ++k)
				q[k] = kUp ? next_up<kWide>(m0, m1) : next_down<kWide>(m0, m1);
#pragma unroll
			for (int k = 0; k < kWalkBatch; ++k)
				v[k] = q[k] >= 0 ? __ldg(e + (size_t)q[k] * P) : make_uint2(0u, 0u);
#pragma unroll
			for (int k = 0; k < kWalkBatch; ++k)
				if (q[k] >= 0)
					body(v[k]);
		}
	}
}

// Entry fields: x = job | a << 16, y = b | c << 16 (a = p[m1][job],
// b = p[m2][job], c = a + lag + b).
#define WSBB_ENTRY(v)                                                         \
	const int job = int((v).x & 0xffu);                                       \
	const int32_t a = int32_t((v).x >> 16), b = int32_t((v).y & 0xffffu);    \
	const int32_t cj = int32_t((v).y >> 16)

// Forward pass of pair p (chunk slot t): X[t][j] = C of the free jobs
// before j; PI[t] = (row offsets of m1, m2, A, B, p).
template <bool kScan, bool kWide, bool k16>
__device__ __forceinline__ void pair_forward(const FamSmem &S, const uint2 *__restrict__ tjT,
                                             int p, int t, int n, int P, int xs, int u,
                                             uint64_t m0, uint64_t m1, const uint32_t *w)
{
	using Sl = Slot<k16>;
	typename Sl::T *xrow = reinterpret_cast<typename Sl::T *>(S.X) + t * xs;
	int32_t a_sum = 0, b_sum = 0, c = kNeg;
	each_free<true, kScan, kWide>(tjT + p, n, P, u, m0, m1, w, [&](uint2 v) {
		WSBB_ENTRY(v);
		xrow[job] = Sl::pre(c);
		c = max(c + b, a_sum + cj);
		a_sum += a;
		b_sum += b;
	});
	const int pr = S.pairs[p], ld = n + 1;
	S.PI[t] = make_int4((pr & 0xff) * ld | ((pr >> 8) * ld) << 16, a_sum, b_sum, p);
}

// Backward pass of chunk slot t: at each free job j, X_j = C of (the free
// jobs after j) x (those before j), then both children that move j:
//   BEGIN (front V[.][j], the father's back r):
//     max(v2 + B - b + r2, v1 + X_j + r2, v1 + A - a + r1)
//   END (the father's front f, back W[.][j]):
//     max(w2 + B - b + f2, w2 + X_j + f1, w1 + A - a + f1)
// (t0 = v1 + A - a, t1 = max(v2 + B - b, v1 + X_j), bound max(t1 + r2,
// t0 + r1), expanded), stored in X[t][j].
template <bool kScan, bool kWide, bool k16>
__device__ __forceinline__ void pair_backward(const FamSmem &S, const uint2 *__restrict__ tjT,
                                              int t, int n, int P, int xs, int u, uint64_t m0,
                                              uint64_t m1, const uint32_t *w)
{
	using Sl = Slot<k16>;
	typename Sl::T *xrow = reinterpret_cast<typename Sl::T *>(S.X) + t * xs;
	const int4 pi = S.PI[t];
	const int4 fr = S.PFR[pi.w]; // (f1, f2, r1, r2)
	const int row1 = pi.x & 0xffff, row2 = int(unsigned(pi.x) >> 16);
	const int32_t A = pi.y, B = pi.z;
	const int32_t kb1 = B + fr.w, kb2 = A + fr.z, ke1 = B + fr.y, ke2 = A + fr.x;
	int32_t as = 0, bs = 0, cs = kNeg;
	each_free<false, kScan, kWide>(tjT + pi.w, n, P, u, m0, m1, w, [&](uint2 v) {
		WSBB_ENTRY(v);
		const int32_t x = max(Sl::pre_of(xrow[job]) + bs, (A - as - a) + cs);
		cs = max(cs + a, bs + cj);
		as += a;
		bs += b;
		const int2 e1 = S.VW[row1 + job], e2 = S.VW[row2 + job];
		const int32_t v1 = e1.x, v2 = e2.x, w1 = e1.y, w2 = e2.y;
		const int32_t tb = max(max(v2 - b + kb1, v1 + x + fr.w), v1 - a + kb2);
		const int32_t te = max(max(w2 - b + ke1, w2 + x + fr.x), w1 - a + ke2);
		xrow[job] = Sl::pack(tb, te);
	});
}
#undef WSBB_ENTRY

// Bounds of the father's children over one chunk of pairs (slot t holds
// pair fp[t] when fp is set, else p_lo + t), folded into `acc` for the
// calling thread's job column rj over the slots t = rs (mod NS). The front
// threads compute the fronts and backs first when `fronts` is set. Called
// by every thread; X must be free on entry.
template <bool kWide, bool k16>
__device__ __forceinline__ void chunk_bounds(const FamSmem &S, const uint2 *__restrict__ tjT,
                                             const uint8_t *__restrict__ jobposT,
                                             const BoundParams &bp, const int16_t *fp, int p_lo,
                                             int len, bool fronts, bool scan, int xs, int l1,
                                             int l2, int u, bool ract, int rj, int rs, int NS,
                                             typename Slot<k16>::T &acc)
{
	using Sl = Slot<k16>;
	const int tid = threadIdx.x, n = bp.n, m = bp.m, P = bp.P;
	const uint32_t *w = S.mask;
	const int16_t *fj = S.fr + l1 + 1; // the father's free jobs
	uint64_t km0 = 0, km1 = 0;          // the walk mask of a walker's single pair
	if (tid < kFrontThreads) {
		if (fronts)
			fronts_and_backs(S, tid >> 5, tid & 31, n, m, P, l1, l2, u,
			                 reinterpret_cast<const int32_t *>(bp.t8.blob + bp.t8.off_heads),
			                 reinterpret_cast<const int32_t *>(bp.t8.blob + bp.t8.off_tails),
			                 false);
	} else {
		for (int t = tid - kFrontThreads; t < len; t += kWalkThreads) {
			const int p = fp ? min(max(int(fp[t]), 0), P - 1) : p_lo + t;
			if (scan) {
				pair_forward<true, kWide, k16>(S, tjT, p, t, n, P, xs, u, 0, 0, w);
			} else {
				walk_mask<kWide>(jobposT, fj, u, p, P, km0, km1);
				pair_forward<false, kWide, k16>(S, tjT, p, t, n, P, xs, u, km0, km1, w);
			}
		}
	}
	__syncthreads(); // fronts, backs and every forward pass done
	if (tid >= kFrontThreads) {
		for (int t = tid - kFrontThreads; t < len; t += kWalkThreads) {
			if (scan) {
				pair_backward<true, kWide, k16>(S, tjT, t, n, P, xs, u, 0, 0, w);
			} else {
				// a walker with several pairs rebuilds each one's mask
				if (len > kWalkThreads)
					walk_mask<kWide>(jobposT, fj, u, S.PI[t].w, P, km0, km1);
				pair_backward<false, kWide, k16>(S, tjT, t, n, P, xs, u, km0, km1, w);
			}
		}
	}
	__syncthreads();
	if (ract) {
		const typename Sl::T *col = reinterpret_cast<const typename Sl::T *>(S.X) + rj;
		for (int t = rs; t < len; t += NS)
			acc = Sl::vmax(acc, col[t * xs]);
	}
}

// kLearned: the father's K ranked pairs first; a child whose bound over
// them reaches max(best, incumbent) is settled with that value (the search
// only compares such bounds with the thresholds, never ranks or sums
// them); fathers with children left take every pair for those children.
template <bool kLearned, bool kWide, bool k16>
__global__ void __launch_bounds__(kFamThreads, 4) family_kernel(FamilyArgs A, BoundParams bp,
                                                             const uint2 *__restrict__ tjT,
                                                             const uint8_t *__restrict__ jobposT,
                                                             FamLayout L)
{
	using Sl = Slot<k16>;
	using T = typename Sl::T;
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
	// the K ranked pairs form one chunk
	const int K = kLearned ? min(min(A.K, P), L.pc) : 0;
	T *red = reinterpret_cast<T *>(S.red);

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
			// walks: scan all n positions when most jobs are free (more than
			// 3/4, or half for n > 64 where the position masks take two
			// words), else follow the position table over the free ones only
			const bool scan = kWide ? 2 * u > n : 4 * u > 3 * n;
			if (scan) {
				if (tid < 4)
					S.mask[tid] = 0;
				__syncthreads();
				if (tid < u)
					atomicOr(&S.mask[S.fr[l1 + 1 + tid] >> 5], 1u << (S.fr[l1 + 1 + tid] & 31));
				__syncthreads();
			}
			// the final sweep: thread (free job tid - rs u, slice rs) of NS
			// slices. tid / u without an integer division: (tid + 1/2) / u
			// lies at least 1/(2u) >= 1/256 from an integer, far beyond the
			// float error of a quotient below 256
			const int rs = int((float(tid) + 0.5f) * __frcp_rn(float(u)));
			const int NS = min(int((float(kFamThreads) + 0.5f) * __frcp_rn(float(u))), 32);
			const bool ract = rs < NS;
			const int rj = ract ? S.fr[l1 + 1 + (tid - rs * u)] : 0;
			T acc = Sl::none();
			int32_t lbB = 0, lbE = 0;
			bool needB = true, needE = true;
			if (kLearned) {
				chunk_bounds<kWide, k16>(S, tjT, jobposT, bp, A.fpairs + f * A.K, 0, K, true, scan,
				                         xs, l1, l2, u, ract, rj, rs, NS, acc);
				__syncthreads(); // red overwrites the X rows
				red[tid] = acc;
				__syncthreads();
				int nu = 0;
				if (tid < u) {
					T s = red[tid];
					for (int k = 1; k < NS; ++k)
						s = Sl::vmax(s, red[k * u + tid]);
					lbB = Sl::begin(s);
					lbE = Sl::end(s);
					// settled children keep the bound over the K pairs
					needB = lbB < thr;
					needE = lbE < thr;
					if (!needB)
						A.child_lb[c0 + tid] = lbB;
					if (!needE)
						A.child_lb[c0 + u + tid] = lbE;
					nu = int(needB) + int(needE);
					if (nu)
						atomicAdd(S.cnt, nu);
				}
				__syncthreads();
				const int left = *S.cnt;
				if (tid == 0 && 2 * u - left > 0)
					atomicAdd(A.early, (unsigned long long)(2 * u - left));
				if (tid == 0 && left == 0 && A.settled_fathers)
					atomicAdd(A.settled_fathers, 1ull);
				if (left == 0) {
					if (tid < u) {
						const int16_t job = S.fr[l1 + 1 + tid];
						A.child_job[c0 + tid] = job;
						A.child_job[c0 + u + tid] = job;
					}
					__syncthreads();
					continue;
				}
				acc = Sl::none();
			}
			// every pair, in chunks
			for (int p_lo = 0; p_lo < P; p_lo += L.pc) {
				if (p_lo > 0 || kLearned)
					__syncthreads(); // the previous chunk (or red) consumed
				chunk_bounds<kWide, k16>(S, tjT, jobposT, bp, nullptr, p_lo, min(L.pc, P - p_lo),
				                         !kLearned && p_lo == 0, scan, xs, l1, l2, u, ract, rj, rs,
				                         NS, acc);
			}
			__syncthreads(); // red overwrites the X rows
			red[tid] = acc;
			__syncthreads();
			if (tid < u) {
				T s = red[tid];
				for (int k = 1; k < NS; ++k)
					s = Sl::vmax(s, red[k * u + tid]);
				const int16_t job = S.fr[l1 + 1 + tid];
				A.child_job[c0 + tid] = job;
				A.child_job[c0 + u + tid] = job;
				if (needB)
					A.child_lb[c0 + tid] = Sl::begin(s);
				if (needE)
					A.child_lb[c0 + u + tid] = Sl::end(s);
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

// The staged form (family_staged.cuh), launched on its own: CTAs of
// L.groups groups of NT threads over one copy of the tables; group g of CTA
// b starts with father g * gridDim.x + b (a batch smaller than the grid
// spreads over the SMs) and takes the next ones from the device counter.
template <bool kWide, int NT>
__global__ void __launch_bounds__(staged::kMaxCtaThreads, 1)
    family_staged_kernel(FamilyArgs A, BoundParams bp, const uint32_t *__restrict__ tpack,
                         const uint8_t *__restrict__ jobposT, staged::StagedLayout L)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const long long nf = A.count_dev ? *A.count_dev : A.count;
	const long long groups = L.groups;
	if ((long long)blockIdx.x >= nf)
		return;
	staged::staged_load_tables(bp, tpack, jobposT, L, smem);
	__syncthreads();
	const int group = int(threadIdx.x) / NT;
	const long long base = (long long)gridDim.x * groups;
	staged::staged_fathers<kWide, NT>(A, bp, L, smem, group, nf,
	                                  (long long)group * gridDim.x + blockIdx.x,
	                                  [&](long long after) -> long long {
		                                  // one warp calls it: lane 0 claims for all
		                                  long long c = after + base;
		                                  if (A.next && (threadIdx.x & 31) == 0)
			                                  c = base + (long long)atomicAdd(A.next, 1ull);
		                                  return __shfl_sync(0xffffffffu, c, 0);
	                                  });
}

}  // namespace

size_t family_smem(const BoundParams &bp, int smem_kb)
{
	return fam_layout(bp.n, bp.m, bp.P, size_t(smem_kb > 0 ? smem_kb : 56) * 1024, bp.span16 != 0)
	    .bytes;
}

cudaError_t launch_family_lb2(const BoundParams &bp, const DeviceTables &T, const FamilyArgs &A,
                              long long max_fathers, int num_sms, cudaStream_t s, int smem_kb)
{
	if (max_fathers <= 0)
		return cudaSuccess;
	const size_t budget = size_t(std::min(std::max(smem_kb > 0 ? smem_kb : 56, 16), 220)) * 1024;
	const bool p16 = bp.span16 != 0;
	const FamLayout L = fam_layout(bp.n, bp.m, bp.P, budget, p16);
	const bool learned = A.fpairs != nullptr;
	const bool wide = bp.n > 64;
	if (!learned && T.tpack && p16 && bp.P <= kWalkThreads && smem_kb <= 0) {
		int dev = 0, max_optin = 0;
		cudaError_t e = cudaGetDevice(&dev);
		if (e == cudaSuccess)
			e = cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
		if (e != cudaSuccess)
			return e;
		// up to 64 pairs: groups of 128 threads; as many groups per CTA as
		// its shared memory and kMaxCtaThreads allow
		const bool small = bp.P <= staged::kFamThreadsSmall - staged::kFrontThreads;
		const int nt = small ? staged::kFamThreadsSmall : staged::kFamThreads;
		int groups = staged::kMaxCtaThreads / nt;
		staged::StagedLayout SL = staged::staged_layout(bp.n, bp.m, bp.P, T.Pp, groups);
		while (groups > 1 && SL.bytes + 1024 > size_t(max_optin))
			SL = staged::staged_layout(bp.n, bp.m, bp.P, T.Pp, --groups);
		if (SL.bytes + 1024 <= size_t(max_optin)) {
			using SKern = void (*)(FamilyArgs, BoundParams, const uint32_t *, const uint8_t *,
			                       staged::StagedLayout);
			const SKern sk = small ? (wide ? family_staged_kernel<true, staged::kFamThreadsSmall>
			                               : family_staged_kernel<false, staged::kFamThreadsSmall>)
			                       : (wide ? family_staged_kernel<true, staged::kFamThreads>
			                               : family_staged_kernel<false, staged::kFamThreads>);
			e = allow_max_dynamic_smem(sk);
			int occ = 0;
			if (e == cudaSuccess)
				e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sk, nt * groups, SL.bytes);
			if (e != cudaSuccess)
				return e;
			const long long grid = std::min<long long>((max_fathers + groups - 1) / groups,
			                                           (long long)num_sms * std::max(occ, 1));
			sk<<<unsigned(grid), nt * groups, SL.bytes, s>>>(A, bp, T.tpack, T.jobposT, SL);
			return cudaGetLastError();
		}
	}
	using Kern = void (*)(FamilyArgs, BoundParams, const uint2 *, const uint8_t *, FamLayout);
	static const Kern kernels[8] = {
	    family_kernel<false, false, false>, family_kernel<false, false, true>,
	    family_kernel<false, true, false>,  family_kernel<false, true, true>,
	    family_kernel<true, false, false>,  family_kernel<true, false, true>,
	    family_kernel<true, true, false>,   family_kernel<true, true, true>};
	const Kern kern = kernels[(learned ? 4 : 0) + (wide ? 2 : 0) + (p16 ? 1 : 0)];
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
