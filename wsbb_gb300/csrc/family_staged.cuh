// Family bounds, staged form (see family.cu for the method): the device
// code shared by the standalone kernel (family.cu, wsbb_decompose_lb2 and the
// graph-launched search) and the resident search (resident.cu), which bounds
// the fathers of many instances from CTAs that stay resident.
#pragma once

#include <algorithm>

#include "wsbb_internal.h"

namespace wsbb {
namespace staged {

// Groups of kFamThreads threads (P > 64 pairs) or kFamThreadsSmall (P <=
// 64): each group bounds its own fathers, two of its warps computing fronts
// and backs while the rest walk pairs. A CTA holds up to kMaxCtaThreads
// threads of groups that share one copy of the instance's tables, so that
// the table is staged once per SM rather than once per father in flight.
constexpr int kFamThreads = 256;
constexpr int kFamThreadsSmall = 128;
constexpr int kFrontThreads = 64;
constexpr int kWalkThreads = kFamThreads - kFrontThreads;
constexpr int kMaxCtaThreads = 768;
constexpr int32_t kNeg = -(1 << 28); // max-plus -inf, far from any sum of times

// The same bounds, organised around shared memory (plain bounds of fathers
// whose pairs fit the walkers, P <= 192, with times that pack into the
// 32-bit Johnson entries of DeviceTables::tpack and 16-bit staircase paths):
//
//  * the packed Johnson table is staged once per CTA (for all its
//    groups), position-major with rows of Pp (a multiple of 64) words, so a
//    warp of walkers (consecutive pairs) reading entries at any positions
//    hits 32 distinct banks;
//  * the forward pass leaves, per walk rank k, the prefix C (16 bits) and
//    the position q in rows [k][Pp] (lanes walk in step, so these accesses
//    are conflict-free too) and the backward pass reads them back instead
//    of walking the position masks a second time;
//  * the backward pass leaves X_j per pair and job, and the children's
//    bounds are formed afterwards by every thread of the group, lanes on
//    consecutive columns (free positions) of one pair: the fronts and backs
//    they read (per machine and column) are consecutive words, the X_j one
//    pair's row (at n <= 64 at most 32 consecutive words: distinct banks),
//    and both children's three terms are computed as 16-bit halves of one
//    word (add, then one three-way and one two-way unsigned 16-bit
//    maximum).
// The CTA's tables first (T, heads and tails, processing times, pairs, the
// job positions per pair), then one region per group, `grp_bytes` apart from
// `off_grp`; the offsets Xr ... misc lie within a group's region.
struct StagedLayout {
	int Pp, xcs, xvs, frs, groups;
	size_t off_T, off_HT, off_pt, off_pairs, off_JP, off_grp, grp_bytes;
	size_t off_Xr, off_Xq, off_Xc, off_VW, off_PK, off_F, off_G, off_fr, off_misc;
	size_t bytes;
};

inline StagedLayout staged_layout(int n, int m, int P, int Pp, int groups = 1)
{
	StagedLayout L;
	L.Pp = Pp;
	L.xcs = n | 1;
	L.xvs = n;
	L.groups = groups;
	auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
	size_t off = 0;
	L.off_T = off;
	off = a16(off + size_t(n) * Pp * 4);
	L.off_HT = off;
	off = a16(off + 64 * 4);
	L.off_pt = off;
	off = a16(off + size_t(m) * (n + 1) * 2);
	L.off_pairs = off;
	off = a16(off + size_t(P) * 4);
	L.off_JP = off; // jobposT: the position of job j in pair p's order at [j][P]
	off = a16(off + size_t(n) * P);
	L.off_grp = off;
	off = 0; // a group's region
	L.off_Xr = off; // the cross-slice reduction reuses it after the backward pass
	off = a16(off + std::max(size_t(n) * Pp * 2, size_t(kFamThreads) * 4));
	L.off_Xq = off;
	off = a16(off + size_t(n) * Pp);
	L.off_Xc = off;
	off = a16(off + size_t(P) * L.xcs * 2);
	L.off_VW = off;
	off = a16(off + size_t(m) * L.xvs * 8);
	L.off_PK = off;
	off = a16(off + size_t(P) * 16);
	L.off_F = off;
	off = a16(off + 32 * 4);
	L.off_G = off;
	off = a16(off + 32 * 4);
	L.frs = (n + 4 + 7) & ~7; // two record buffers
	L.off_fr = off;
	off = a16(off + size_t(2 * L.frs) * 2);
	// two 4-word job masks, two claimed fathers, two child ranges
	L.off_misc = off;
	off += 32 + 16 + 32;
	L.grp_bytes = a16(off);
	L.bytes = L.off_grp + size_t(groups) * L.grp_bytes;
	return L;
}

// Barrier of one group's NT threads (named barrier 1 + group; barrier 0
// stays the CTA's).
template <int NT>
__device__ __forceinline__ void group_sync(int group)
{
	asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "n"(NT) : "memory");
}

// Free positions of a walk mask in ascending order (words w[0..NW-1]).
template <int NW>
__device__ __forceinline__ int pop_lowest(uint32_t (&w)[NW]);
template <>
__device__ __forceinline__ int pop_lowest<2>(uint32_t (&w)[2])
{
	uint64_t v = uint64_t(w[1]) << 32 | w[0];
	const int q = __ffsll((long long)v) - 1;
	v &= v - 1;
	w[0] = uint32_t(v);
	w[1] = uint32_t(v >> 32);
	return q;
}
template <int NW>
__device__ __forceinline__ int pop_lowest(uint32_t (&w)[NW])
{
	int wi = NW - 1;
#pragma unroll
	for (int i = NW - 2; i >= 0; --i)
		wi = w[i] ? i : wi;
	uint32_t v = w[0];
#pragma unroll
	for (int i = 1; i < NW; ++i)
		v = wi == i ? w[i] : v;
	const int b = __ffs(v) - 1;
#pragma unroll
	for (int i = 0; i < NW; ++i)
		if (wi == i)
			w[i] = v & (v - 1);
	return 32 * wi + b;
}

template <int NW>
__device__ __forceinline__ bool mask_has(const uint32_t (&w)[NW], int job)
{
	uint32_t v = w[0];
#pragma unroll
	for (int i = 1; i < NW; ++i)
		v = (job >> 5) == i ? w[i] : v;
	return ((v >> (job & 31)) & 1u) != 0;
}

// Fronts and backs of the children by column (free position i): per
// machine k four 16-bit values, vm = the time job j starts on k in the
// BEGIN child's front, v = when it ends there, wm / w the same for the END
// child's back. Warp 0 the father's front F and the fronts, warp 1 its
// reversed back G and the backs (each a wavefront, lane = machine, then one
// lane per free job); with leaves_only, F and G alone.
//
// The wavefront's step s has lane k add job s - k's time on its machine to
// max(its own time, lane k-1's); the times of kWaveBatch steps are loaded
// before their steps run, so that only the steps' own chain (a shuffle, a
// maximum and an add) is serial.
constexpr int kWaveBatch = 4;
template <typename TimeOf>
__device__ __forceinline__ int32_t staged_wave(int lane, int m, int nj, TimeOf time_of)
{
	int32_t Fk = 0;
	for (int s0 = 0; s0 < nj + m - 1; s0 += kWaveBatch) {
		int32_t tv[kWaveBatch];
#pragma unroll
		for (int d = 0; d < kWaveBatch; ++d) {
			const int i = s0 + d - lane;
			tv[d] = (lane < m && i >= 0 && i < nj) ? int32_t(time_of(i)) : -1; // -1: no step
		}
#pragma unroll
		for (int d = 0; d < kWaveBatch; ++d) {
			const int32_t left = __shfl_up_sync(0xffffffffu, Fk, 1);
			if (tv[d] >= 0)
				Fk = max(Fk, lane > 0 ? left : 0) + tv[d];
		}
	}
	return Fk;
}

__device__ __forceinline__ void staged_fronts(int warp, int lane, int n, int m, int l1, int l2,
                                              int u, int xvs, const uint16_t *pt,
                                              const int16_t *fr, int32_t *F, int32_t *G,
                                              uint16_t *VW16, bool leaves_only = false)
{
	const int ld = n + 1;
	if (warp == 0) {
		const int32_t Fk =
		    staged_wave(lane, m, l1 + 1, [&](int i) { return pt[lane * ld + fr[i]]; });
		if (lane < m)
			F[lane] = Fk;
		if (leaves_only)
			return;
		__syncwarp();
		for (int i = lane; i < u; i += 32) {
			const int j = fr[l1 + 1 + i];
			int32_t v = 0;
#pragma unroll 4
			for (int k = 0; k < m; ++k) {
				const int32_t vm = max(v, F[k]);
				v = vm + pt[k * ld + j];
				VW16[(k * xvs + i) * 4 + 0] = uint16_t(vm);
				VW16[(k * xvs + i) * 4 + 2] = uint16_t(v);
			}
		}
	} else if (warp == 1) {
		const int32_t Gq = staged_wave(lane, m, n - l2, [&](int i) {
			return pt[(m - 1 - lane) * ld + fr[n - 1 - i]];
		});
		if (lane < m)
			G[lane] = Gq;
		if (leaves_only)
			return;
		__syncwarp();
		for (int i = lane; i < u; i += 32) {
			const int j = fr[l1 + 1 + i];
			int32_t g = 0;
#pragma unroll 4
			for (int q = 0; q < m; ++q) {
				const int k = m - 1 - q;
				const int32_t wm = max(g, G[q]);
				g = wm + pt[k * ld + j];
				VW16[(k * xvs + i) * 4 + 1] = uint16_t(wm);
				VW16[(k * xvs + i) * 4 + 3] = uint16_t(g);
			}
		}
	}
}

// Staged walks and sweep: entries loaded ahead per batch. One: with three
// groups per SM the other warps hide a load's latency, and batches of 2 or
// 4 only added registers and predicated slots past the last entry (the
// search 11 % slower with 4, 5 % with 2).
constexpr int kSB = 1;


// Stages one instance's tables for staged_fathers: the packed Johnson
// table, processing times, pairs, heads and tails, job positions. Every
// thread of the CTA calls it; a barrier of the whole CTA must follow before
// staged_fathers reads them.
__device__ __forceinline__ void staged_load_tables(const BoundParams &bp,
                                                   const uint32_t *__restrict__ tpack,
                                                   const uint8_t *__restrict__ jobposT,
                                                   const StagedLayout &L, uint8_t *smem)
{
	const int n = bp.n, m = bp.m, P = bp.P, tid = threadIdx.x;
	const uint4 *src = reinterpret_cast<const uint4 *>(tpack);
	uint4 *dst = reinterpret_cast<uint4 *>(smem + L.off_T);
	const int words = n * L.Pp / 4;
	for (int i = tid; i < words; i += int(blockDim.x))
		dst[i] = __ldg(src + i);
	const uint8_t *tb = bp.t8.blob;
	const int32_t *g_pt = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pt);
	const int32_t *g_pairs = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pairs);
	const int32_t *g_heads = reinterpret_cast<const int32_t *>(tb + bp.t8.off_heads);
	const int32_t *g_tails = reinterpret_cast<const int32_t *>(tb + bp.t8.off_tails);
	uint16_t *sPt = reinterpret_cast<uint16_t *>(smem + L.off_pt);
	int32_t *sPairs = reinterpret_cast<int32_t *>(smem + L.off_pairs);
	int32_t *sHT = reinterpret_cast<int32_t *>(smem + L.off_HT);
	for (int i = tid; i < m * n; i += int(blockDim.x))
		sPt[(i / n) * (n + 1) + i % n] = uint16_t(g_pt[i]);
	for (int i = tid; i < P; i += int(blockDim.x))
		sPairs[i] = g_pairs[i];
	for (int i = tid; i < n * P; i += int(blockDim.x))
		smem[L.off_JP + i] = __ldg(jobposT + i);
	if (tid < m) {
		sHT[tid] = g_heads[tid];
		sHT[32 + tid] = g_tails[tid];
	}
}

// A group bounds one father at a time; while its walkers run the backward
// passes, its warps 0-1 (idle then) claim the group's father after next and
// load the next father's record and job mask into the other buffers, so
// neither the claim's round trip nor the record load sits between two
// fathers. Four barriers per father: record and mask ready, forward passes
// and fronts, backward passes, children's bounds.
//
// staged_fathers bounds the fathers first, claim(first), claim(that), ...
// until a claim returns nf or more, with the tables already staged
// (staged_load_tables, then a barrier of the CTA); every thread of group
// `group` (NT threads from threadIdx.x = group * NT, P <= NT - 64) calls it
// with the same arguments. Every lane of one warp calls claim(after) with
// the same argument, and it returns the same index on every lane. Returns
// the number of fathers it bounded.
//
// The group's warps take their roles rotated by two warps per group (role
// warp w is warp (w - 2 * group) mod NT/32 of the group), so that the
// groups' front and back warps, which issue little, sit on different SM
// sub-partitions (warp slot mod 4) and the walkers spread evenly over them.
template <bool kWide, int NT, typename Claim>
__device__ long long staged_fathers(const FamilyArgs &A, const BoundParams &bp,
                                    const StagedLayout &L,
                                    uint8_t *smem, int group, long long nf, long long first,
                                    Claim claim)
{
	constexpr int NW = kWide ? 4 : 2; // 32-bit words of a job or position mask
	constexpr int kWarps = NT / 32;
	const int n = bp.n, m = bp.m, P = bp.P, Pp = L.Pp, xcs = L.xcs, xvs = L.xvs;
	const int lane = int(threadIdx.x) & 31;
	const int warp = ((int(threadIdx.x) >> 5) - group * kWarps + 2 * group) % kWarps; // role
	const int tid = warp * 32 + lane;
	uint8_t *gsm = smem + L.off_grp + size_t(group) * L.grp_bytes;
	uint32_t *sT = reinterpret_cast<uint32_t *>(smem + L.off_T);
	uint16_t *sXr = reinterpret_cast<uint16_t *>(gsm + L.off_Xr);
	uint32_t *sRed = reinterpret_cast<uint32_t *>(gsm + L.off_Xr);
	uint8_t *sXq = gsm + L.off_Xq;
	uint16_t *sXc = reinterpret_cast<uint16_t *>(gsm + L.off_Xc);
	uint16_t *sVW16 = reinterpret_cast<uint16_t *>(gsm + L.off_VW);
	const uint2 *sVW = reinterpret_cast<const uint2 *>(gsm + L.off_VW);
	uint4 *sPK = reinterpret_cast<uint4 *>(gsm + L.off_PK);
	int32_t *sHT = reinterpret_cast<int32_t *>(smem + L.off_HT); // heads[32], tails[32]
	uint16_t *sPt = reinterpret_cast<uint16_t *>(smem + L.off_pt);
	int32_t *sPairs = reinterpret_cast<int32_t *>(smem + L.off_pairs);
	int32_t *sF = reinterpret_cast<int32_t *>(gsm + L.off_F);
	int32_t *sG = reinterpret_cast<int32_t *>(gsm + L.off_G);
	int16_t *sFrBuf = reinterpret_cast<int16_t *>(gsm + L.off_fr); // [2][L.frs]
	uint32_t *sMaskBuf = reinterpret_cast<uint32_t *>(gsm + L.off_misc); // [2][4]
	long long *sNext = reinterpret_cast<long long *>(gsm + L.off_misc + 32); // [2]
	long long *sKids = reinterpret_cast<long long *>(gsm + L.off_misc + 48); // [2][2]
	const uint8_t *sJP = smem + L.off_JP;
	auto sync = [group]() { group_sync<NT>(group); };

	// record of father g into buffer b, its free jobs into job mask b
	// (zeroed before) and its child range into sKids[b]; job ids clamped to
	// [0, n): a malformed record gives wrong bounds, never an access outside
	// the tables. Threads t0 .. t0 + nt - 1.
	auto load_record = [&](long long g, int b, int t0, int nt) {
		if (g >= nf)
			return;
		if (tid - t0 < 2)
			sKids[2 * b + tid - t0] = A.child_off[g + tid - t0];
		const long long ri = A.ridx ? A.ridx[g] : g;
		const int16_t *g_fr = reinterpret_cast<const int16_t *>(A.fathers + ri * A.stride);
		int16_t *dst = sFrBuf + b * L.frs;
		const int gl1 = g_fr[n], gl2 = g_fr[n + 1];
		for (int i = tid - t0; i < n + 2; i += nt) {
			const int v = i < n ? min(max(int(g_fr[i]), 0), n - 1) : int(g_fr[i]);
			dst[i] = int16_t(v);
			if (i > gl1 && i < gl2 && i < n)
				atomicOr(&sMaskBuf[4 * b + (v >> 5)], 1u << (v & 31));
		}
	};
	if (tid < 8)
		sMaskBuf[tid] = 0;
	if (warp == 0) {
		const long long c = first < nf ? claim(first) : nf;
		if (lane == 0)
			sNext[0] = c;
	}
	sync(); // the masks are clear
	load_record(first, 0, 0, NT);
	long long done = 0;
	const int t = tid - kFrontThreads; // walker: pair t
	const bool walker = t >= 0 && t < P;
	int cur = 0;
	for (long long f = first; f < nf;) {
		sync(); // record f and its job mask in buffer cur, its successor in sNext[cur]
		const long long fn = sNext[cur];
		const int16_t *sFr = sFrBuf + cur * L.frs;
		uint32_t *sMask = sMaskBuf + 4 * cur;
		const int l1 = sFr[n], l2 = sFr[n + 1];
		const int u = l2 - l1 - 1;
		const long long c0 = sKids[2 * cur];
		// the other mask buffer (its father is done) is cleared for the
		// next record, which prefetch() loads after a barrier at least
		if (tid < 4)
			sMaskBuf[4 * (cur ^ 1) + tid] = 0;
		// the next record and the claim after it, by warps 0-1 while they
		// have nothing else to do
		auto prefetch = [&]() {
			if (tid < kFrontThreads) {
				if (warp == 0) {
					const long long c = fn < nf ? claim(fn) : nf;
					if (lane == 0)
						sNext[cur ^ 1] = c;
				}
				load_record(fn, cur ^ 1, 0, kFrontThreads);
			}
		};
		// cursors outside -1 <= l1, l2 <= n with two free jobs or more, or a
		// child range of another size: the father is skipped
		if (l1 < -1 || l2 > n || u < 2 || sKids[2 * cur + 1] - c0 != (u == 2 ? 2 : 2 * u)) {
			sync(); // the other mask is clear
			prefetch();
			++done;
			f = fn;
			cur ^= 1;
			continue;
		}
		if (u == 2) {
			// two leaves: makespans of front + (x, y) + back, both orders
			staged_fronts(warp, lane, n, m, l1, l2, u, xvs, sPt, sFr, sF, sG, sVW16, true);
			sync();
			if (tid < 2) {
				const int x = sFr[l1 + 1 + tid], y = sFr[l1 + 2 - tid];
				int32_t v1 = 0, v2 = 0, mk = 0;
				for (int k = 0; k < m; ++k) {
					v1 = max(v1, sF[k]) + sPt[k * (n + 1) + x];
					v2 = max(v2, v1) + sPt[k * (n + 1) + y];
					mk = max(mk, v2 + sG[m - 1 - k]);
				}
				A.child_lb[c0 + tid] = mk;
				A.child_job[c0 + tid] = int16_t(x);
			}
			prefetch();
			++done;
			f = fn;
			cur ^= 1;
			continue;
		}
		// a record whose free jobs repeat one another is skipped (its walks
		// would find fewer than u positions)
		if (__popc(sMask[0]) + __popc(sMask[1]) + __popc(sMask[2]) + __popc(sMask[3]) != u) {
			sync(); // the other mask is clear
			prefetch();
			++done;
			f = fn;
			cur ^= 1;
			continue;
		}
		// walks: the pair's free positions by a scan of all n positions when
		// most jobs are free (more than 3/4), which then runs the recurrence
		// over the ranks it found, else by the position table's u entries
		// sorted through a bit mask, the recurrence following each batch
		const bool scan = 4 * u > 3 * n;
		int32_t Asum = 0, Bsum = 0;
		if (walker) {
			int32_t c = kNeg, as = 0, bs = 0;
			auto step = [&](uint32_t e, int k) {
				sXr[k * Pp + t] = uint16_t(c);
				const int32_t a = int32_t((e >> 7) & 127u), b = int32_t((e >> 14) & 127u);
				c = max(c + b, as + int32_t(e >> 21));
				as += a;
				bs += b;
			};
			if (scan) {
				uint32_t w[NW];
#pragma unroll
				for (int i = 0; i < NW; ++i)
					w[i] = sMask[i];
				int k = 0;
				for (int q0 = 0; q0 < n; q0 += kSB) {
					uint32_t e[kSB];
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						e[j] = q0 + j < n ? sT[(q0 + j) * Pp + t] : 0u;
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						if (q0 + j < n && mask_has<NW>(w, int(e[j] & 127u))) {
							sXq[k * Pp + t] = uint8_t(q0 + j);
							step(e[j], k++);
						}
				}
			} else {
				uint32_t w[NW];
#pragma unroll
				for (int i = 0; i < NW; ++i)
					w[i] = 0;
				const int16_t *fj = sFr + l1 + 1;
				if (NW == 2) { // n <= 64: one 64-bit word
					uint64_t m64 = 0;
#pragma unroll 4
					for (int i = 0; i < u; ++i)
						m64 |= 1ull << sJP[fj[i] * P + t];
					w[0] = uint32_t(m64);
					w[NW - 1] = uint32_t(m64 >> 32);
				} else {
#pragma unroll 4
					for (int i = 0; i < u; ++i) {
						const int q = sJP[fj[i] * P + t];
#pragma unroll
						for (int wi = 0; wi < NW; ++wi)
							w[wi] |= (q >> 5) == wi ? 1u << (q & 31) : 0u;
					}
				}
				// batches of kSB: positions first, then their entries, then
				// the recurrence
				for (int k0 = 0; k0 < u; k0 += kSB) {
					int q[kSB];
					uint32_t e[kSB];
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						q[j] = k0 + j < u ? pop_lowest<NW>(w) : 0;
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						e[j] = sT[q[j] * Pp + t];
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						if (k0 + j < u) {
							sXq[(k0 + j) * Pp + t] = uint8_t(q[j]);
							step(e[j], k0 + j);
						}
				}
			}
			Asum = as;
			Bsum = bs;
		} else if (tid < kFrontThreads) {
			staged_fronts(warp, lane, n, m, l1, l2, u, xvs, sPt, sFr, sF, sG, sVW16);
		}
		sync(); // fronts, backs and every forward pass done
		if (walker) {
			// the pair's constants for the children's bounds: the father's
			// front on m1, m2 (the static heads without one) and back (0 on m1
			// and the static tail on m2 without one)
			const int pr = sPairs[t], ma = pr & 0xff, mb = pr >> 8;
			const int32_t f1 = l1 >= 0 ? sF[ma] : sHT[ma], f2 = l1 >= 0 ? sF[mb] : sHT[mb];
			const int32_t r1 = l2 < n ? sG[m - 1 - ma] : 0;
			const int32_t r2 = l2 < n ? sG[m - 1 - mb] : sHT[32 + mb];
			sPK[t] = make_uint4(uint32_t(Bsum + r2) | uint32_t(Bsum + f2) << 16,
			                    uint32_t(r2) | uint32_t(f1) << 16,
			                    uint32_t(Asum + r1) | uint32_t(Asum + f1) << 16,
			                    uint32_t(ma * xvs * 8) | uint32_t(mb * xvs * 8) << 16);
			// backward: X_j = max(Csuf + Apre, Bsuf + Cpre) at each free job
			int32_t cs = kNeg, bs = 0, R = Asum; // R = A minus the suffix's a
			auto step = [&](uint32_t e, int32_t pre, int col) {
				const int32_t a = int32_t((e >> 7) & 127u), b = int32_t((e >> 14) & 127u);
				const int32_t x = max(pre + bs, R - a + cs);
				cs = max(cs + a, bs + int32_t(e >> 21));
				R -= a;
				bs += b;
				sXc[t * xcs + col] = uint16_t(x);
			};
			{
				for (int k0 = u - 1; k0 >= 0; k0 -= kSB) {
					int q[kSB], col[kSB];
					int32_t pre[kSB];
					uint32_t e[kSB];
#pragma unroll
					for (int j = 0; j < kSB; ++j) {
						const int k = max(k0 - j, 0);
						q[j] = sXq[k * Pp + t];
						pre[j] = int32_t(sXr[k * Pp + t]);
					}
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						e[j] = sT[q[j] * Pp + t];
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						col[j] = int(e[j] & 127u);
#pragma unroll
					for (int j = 0; j < kSB; ++j)
						if (k0 - j >= 0)
							step(e[j], pre[j], col[j]);
				}
			}
		} else {
			// warps 0-1: claim and load ahead
			prefetch();
		}
		sync(); // every X_j and pair constant in place
		// the children's bounds: thread (column i, slice rs) of NS slices
		// takes the pairs rs, rs + NS, ...; tid / u without an integer
		// division ((tid + 1/2) / u lies at least 1/(2u) >= 1/256 from an
		// integer, far beyond the float error of a quotient below 256)
		const int rs = int((float(tid) + 0.5f) * __frcp_rn(float(u)));
		const int NS = min(int((float(NT) + 0.5f) * __frcp_rn(float(u))), 32);
		uint32_t acc = 0; // (BEGIN bound | END bound << 16)
		if (rs < NS) {
			const int i = tid - rs * u;
			const int ji = sFr[l1 + 1 + i]; // the column's job: its X_j entry
			const uint8_t *vwi = reinterpret_cast<const uint8_t *>(sVW + i);
			for (int p0 = rs; p0 < P; p0 += kSB * NS) {
				uint4 pk[kSB];
				uint32_t x[kSB];
				uint2 e1[kSB], e2[kSB];
#pragma unroll
				for (int j = 0; j < kSB; ++j) {
					const int p = min(p0 + j * NS, P - 1);
					pk[j] = sPK[p];
					x[j] = sXc[p * xcs + ji];
				}
#pragma unroll
				for (int j = 0; j < kSB; ++j) {
					e1[j] = *reinterpret_cast<const uint2 *>(vwi + (pk[j].w & 0xffffu));
					e2[j] = *reinterpret_cast<const uint2 *>(vwi + (pk[j].w >> 16));
				}
				// a repeated last pair (past P) only repeats a maximum
#pragma unroll
				for (int j = 0; j < kSB; ++j) {
					const uint32_t T1 = e2[j].x + pk[j].x;
					const uint32_t T3 = e1[j].x + pk[j].z;
					const uint32_t T2 =
					    __byte_perm(e1[j].y, e2[j].y, 0x7610) + x[j] * 0x10001u + pk[j].y;
					acc = __vmaxu2(acc, __vimax3_u16x2(T1, T2, T3));
				}
			}
		}
		sRed[tid] = acc; // Xr is consumed
		sync();
		if (tid < u) {
			uint32_t r = sRed[tid];
			for (int k = 1; k < NS; ++k)
				r = __vmaxu2(r, sRed[k * u + tid]);
			const int16_t job = sFr[l1 + 1 + tid];
			A.child_job[c0 + tid] = job;
			A.child_job[c0 + u + tid] = job;
			A.child_lb[c0 + tid] = int32_t(r & 0xffffu);
			A.child_lb[c0 + u + tid] = int32_t(r >> 16);
		}
		++done;
		f = fn;
		cur ^= 1;
	}
	return done;
}


}  // namespace staged
}  // namespace wsbb
