// Host-side instance work: seeded instances and pools, the NEH heuristic,
// and the LB2 precompute (pairs, lags, Johnson orders, static heads and
// tails) that the reference does once per instance in
// bound_flowshop::initialiserVar (src/bound_flowshop.cpp:556-576).
#include <algorithm>
#include <climits>
#include <cstring>

#include "wsbb_internal.h"

namespace wsbb {
namespace {

struct SplitMix64 {
	uint64_t s;
	uint64_t next()
	{
		uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
		return z ^ (z >> 31);
	}
	// uniform in [0, k) by rejection
	uint64_t below(uint64_t k)
	{
		const uint64_t limit = (UINT64_MAX / k) * k;
		uint64_t x;
		do {
			x = next();
		} while (x >= limit);
		return x % k;
	}
	double unit() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Johnson-with-lags order of one machine pair, sorted exactly as the
// reference does it: the Hoare partition with the first element as pivot
// and its recursion (src/bound_flowshop.cpp:597-625) over the keys of
// src/bound_flowshop.cpp:627-643 — class 1 (p[m1] < p[m2]) ascending by
// p[m1] + lag, then class 2 descending by p[m2] + lag. Equal keys keep the
// order this scheme leaves them in, which the bound's result depends on.
class JohnsonSorter {
public:
	JohnsonSorter(const std::vector<int> &cls, const std::vector<int32_t> &key)
	    : cls_(cls), key_(key) {}

	void sort(int32_t *order, int lo, int hi) const
	{
		while (hi - lo > 0) {
			int cut = partition(order, lo, hi);
			sort(order, lo, cut);
			lo = cut + 1;
		}
	}

private:
	bool before(int a, int b) const
	{
		if (cls_[a] != cls_[b])
			return cls_[a] < cls_[b];
		return cls_[a] == 1 ? key_[a] < key_[b] : key_[a] > key_[b];
	}
	bool after(int a, int b) const
	{
		if (cls_[a] != cls_[b])
			return cls_[a] > cls_[b];
		return cls_[a] == 1 ? key_[a] > key_[b] : key_[a] < key_[b];
	}
	int partition(int32_t *order, int lo, int hi) const
	{
		const int32_t pivot = order[lo];
		int left = lo - 1, right = hi + 1;
		for (;;) {
			do
				--right;
			while (after(order[right], pivot));
			do
				++left;
			while (before(order[left], pivot));
			if (left >= right)
				return right;
			std::swap(order[left], order[right]);
		}
	}
	const std::vector<int> &cls_;
	const std::vector<int32_t> &key_;
};

int32_t sequence_makespan(const int32_t *p, int n, int m, const int32_t *seq,
                          int len)
{
	int32_t c[WSBB_MAX_MACHINES] = {0};
	for (int q = 0; q < len; ++q) {
		const int job = seq[q];
		c[0] += p[job];
		for (int k = 1; k < m; ++k)
			c[k] = std::max(c[k], c[k - 1]) + p[k * n + job];
	}
	return c[m - 1];
}

}  // namespace

std::string build_instance(const int32_t *p, int n, int m, Instance &I)
{
	if (n < 2 || n > WSBB_MAX_JOBS)
		return "n must be in [2, 128]";
	if (m < 2 || m > WSBB_MAX_MACHINES)
		return "m must be in [2, 32]";
	I.n = n;
	I.m = m;
	I.P = m * (m - 1) / 2;
	I.p.assign(p, p + size_t(m) * n);
	for (int32_t v : I.p)
		if (v < 0 || v > 65535)
			return "processing times must be in [0, 65535]";

	// static heads / tails over all jobs (remplirTempsArriverDepart)
	I.heads.assign(m, 0);
	I.tails.assign(m, 0);
	for (int k = 1; k < m; ++k) {
		int32_t h = INT32_MAX, t = INT32_MAX;
		for (int j = 0; j < n; ++j) {
			int32_t before = 0, after = 0;
			for (int q = 0; q < k; ++q)
				before += p[q * n + j];
			for (int q = m - k; q < m; ++q)
				after += p[q * n + j];
			h = std::min(h, before);
			t = std::min(t, after);
		}
		I.heads[k] = h;
		I.tails[m - 1 - k] = t;
	}

	// machine pairs, lexicographic (remplirMachine), and lags (remplirLag)
	I.mach0.clear();
	I.mach1.clear();
	for (int a = 0; a < m - 1; ++a)
		for (int b = a + 1; b < m; ++b) {
			I.mach0.push_back(a);
			I.mach1.push_back(b);
		}
	I.lag.assign(size_t(I.P) * n, 0);
	I.johnson.assign(size_t(I.P) * n, 0);
	std::vector<int> cls(n);
	std::vector<int32_t> key(n);
	for (int i = 0; i < I.P; ++i) {
		const int a = I.mach0[i], b = I.mach1[i];
		int32_t *lag = &I.lag[size_t(i) * n];
		for (int j = 0; j < n; ++j) {
			int32_t s = 0;
			for (int k = a + 1; k < b; ++k)
				s += p[k * n + j];
			lag[j] = s;
			if (s + p[a * n + j] + p[b * n + j] > 65535)
				return "machine-pair sums p1 + lag + p2 must be <= 65535";
			const bool first = p[a * n + j] < p[b * n + j];
			cls[j] = first ? 1 : 2;
			key[j] = (first ? p[a * n + j] : p[b * n + j]) + s;
		}
		int32_t *order = &I.johnson[size_t(i) * n];
		for (int j = 0; j < n; ++j)
			order[j] = j;
		JohnsonSorter(cls, key).sort(order, 0, n - 1);
	}
	return std::string();
}

namespace {

// One table image: the Johnson table (entry_bytes per entry) then the
// shared trailing arrays.
std::vector<uint8_t> pack_image(const Instance &I, int entry_bytes, TableView &L)
{
	const int n = I.n, m = I.m, P = I.P;
	auto align16 = [](size_t x) { return (x + 15) & ~size_t(15); };
	size_t off = align16(size_t(P) * n * entry_bytes);
	L.off_pt = uint32_t(off);
	off = align16(off + size_t(m) * n * 4);
	L.off_pairs = uint32_t(off);
	off = align16(off + size_t(P) * 4);
	L.off_heads = uint32_t(off);
	off = align16(off + size_t(m) * 4);
	L.off_tails = uint32_t(off);
	off = align16(off + size_t(m) * 4);
	L.bytes = uint32_t(off);

	std::vector<uint8_t> img(off, 0);
	uint32_t *w = reinterpret_cast<uint32_t *>(img.data());
	for (int i = 0; i < P; ++i) {
		const int a = I.mach0[i], b = I.mach1[i];
		for (int q = 0; q < n; ++q) {
			const int j = I.johnson[size_t(i) * n + q];
			const uint32_t p1 = uint32_t(I.p[a * n + j]);
			const uint32_t p2 = uint32_t(I.p[b * n + j]);
			const uint32_t lag = uint32_t(I.lag[size_t(i) * n + j]);
			const size_t e = size_t(i) * n + q;
			if (entry_bytes == 8) {
				w[2 * e] = uint32_t(j) | (p1 << 16);
				w[2 * e + 1] = p2 | (lag << 16);
			} else {
				w[4 * e] = 1u << j;
				w[4 * e + 1] = p1;
				w[4 * e + 2] = p2;
				w[4 * e + 3] = lag + p2;
			}
		}
	}
	std::memcpy(img.data() + L.off_pt, I.p.data(), size_t(m) * n * 4);
	int32_t *pairs = reinterpret_cast<int32_t *>(img.data() + L.off_pairs);
	for (int i = 0; i < P; ++i)
		pairs[i] = I.mach0[i] | (I.mach1[i] << 8);
	std::memcpy(img.data() + L.off_heads, I.heads.data(), size_t(m) * 4);
	std::memcpy(img.data() + L.off_tails, I.tails.data(), size_t(m) * 4);
	return img;
}

}  // namespace

HostTables pack_tables(const Instance &I, std::string &err)
{
	HostTables H;
	H.img8 = pack_image(I, 8, H.t8);
	if (I.n <= 32)
		H.img16 = pack_image(I, 16, H.t16);
	// position-major Johnson entries for the family bounds:
	// x = job | p1 << 16, y = p2 | (p1 + lag + p2) << 16
	const int n = I.n;
	H.imgT.resize(size_t(I.P) * n * 8);
	uint32_t *dst = reinterpret_cast<uint32_t *>(H.imgT.data());
	for (int i = 0; i < I.P; ++i) {
		const int a = I.mach0[i], b = I.mach1[i];
		for (int q = 0; q < n; ++q) {
			const int j = I.johnson[size_t(i) * n + q];
			const uint32_t p1 = uint32_t(I.p[a * n + j]), p2 = uint32_t(I.p[b * n + j]);
			const uint32_t c = p1 + uint32_t(I.lag[size_t(i) * n + j]) + p2;
			const size_t e = size_t(q) * I.P + i;
			dst[2 * e] = uint32_t(j) | (p1 << 16);
			dst[2 * e + 1] = p2 | (c << 16);
		}
	}
	// job positions in each pair's Johnson order, job-major: pos[j * P + i]
	H.imgPos.resize(size_t(I.P) * n);
	for (int i = 0; i < I.P; ++i)
		for (int q = 0; q < n; ++q)
			H.imgPos[size_t(I.johnson[size_t(i) * n + q]) * I.P + i] = uint8_t(q);
	// packed 32-bit entries, position-major, rows of Pp words (P rounded up
	// to 64): job | p1 << 7 | p2 << 14 | (p1 + lag + p2) << 21, when every
	// field fits
	{
		bool fits = n <= 128;
		for (int i = 0; fits && i < I.P; ++i)
			for (int j = 0; fits && j < n; ++j) {
				const int p1 = I.p[I.mach0[i] * n + j], p2 = I.p[I.mach1[i] * n + j];
				fits = p1 <= 127 && p2 <= 127 && p1 + I.lag[size_t(i) * n + j] + p2 <= 2047;
			}
		if (fits) {
			H.Pp = (I.P + 63) / 64 * 64;
			H.imgPack.assign(size_t(n) * H.Pp * 4, 0);
			uint32_t *pk = reinterpret_cast<uint32_t *>(H.imgPack.data());
			for (int i = 0; i < I.P; ++i)
				for (int q = 0; q < n; ++q) {
					const int j = I.johnson[size_t(i) * n + q];
					const uint32_t p1 = uint32_t(I.p[I.mach0[i] * n + j]);
					const uint32_t p2 = uint32_t(I.p[I.mach1[i] * n + j]);
					const uint32_t c = p1 + uint32_t(I.lag[size_t(i) * n + j]) + p2;
					pk[size_t(q) * H.Pp + i] = uint32_t(j) | p1 << 7 | p2 << 14 | c << 21;
				}
		}
	}
	if (H.t8.bytes > 200 * 1024)
		err = "bound tables exceed the shared-memory budget (n * m too large)";
	return H;
}

}  // namespace wsbb

extern "C" void wsbb_gen_instance(uint64_t seed, int n, int m, int32_t *p)
{
	wsbb::SplitMix64 g{seed};
	for (int k = 0; k < m; ++k)
		for (int j = 0; j < n; ++j)
			p[k * n + j] = int32_t(1 + g.below(99));
}

// Taillard's generator (E. Taillard, "Benchmarks for basic scheduling
// problems", EJOR 64, 1993): the Lehmer sequence seed' = 16807 seed mod
// (2^31 - 1), computed with Schrage's decomposition (127773 = m div 16807,
// 2836 = m mod 16807) so that no intermediate leaves 32 bits, and a time
// low + floor(seed / m * (high - low + 1)). The reference
// (src/instance_flowshop.cpp:74-82) forms the quotient seed / m in single
// precision, which this follows so that the streams agree time for time.
// Times are drawn machine-major (src/instance_flowshop.cpp:84-89).
extern "C" int wsbb_taillard_instance(int64_t seed, int n, int m, int32_t *p)
{
	if (!p || n <= 0 || m <= 0)
		return WSBB_ERR_ARG;
	const int64_t mod = 2147483647, mult = 16807, q = 127773, r = 2836;
	int64_t s = seed;
	for (int k = 0; k < m; ++k)
		for (int j = 0; j < n; ++j) {
			s = mult * (s % q) - (s / q) * r;
			if (s < 0)
				s += mod;
			const double u01 = double(float(s) / float(mod));
			p[k * n + j] = int32_t(1 + int64_t(u01 * 99.0));
		}
	return WSBB_OK;
}

extern "C" size_t wsbb_node_stride(int n)
{
	return (size_t(2 * n + 8) + 15) & ~size_t(15);
}

extern "C" int wsbb_gen_pool(uint64_t seed, int n, int64_t count,
                             double leaf_share, void *recs_out)
{
	if (n < 3 || n > WSBB_MAX_JOBS || count < 0 || !recs_out)
		return WSBB_ERR_ARG;
	const size_t stride = wsbb_node_stride(n);
	wsbb::SplitMix64 g{seed};
	uint8_t *base = static_cast<uint8_t *>(recs_out);
	int perm[WSBB_MAX_JOBS];
	for (int64_t r = 0; r < count; ++r) {
		for (int j = 0; j < n; ++j)
			perm[j] = j;
		for (int j = n - 1; j > 0; --j)
			std::swap(perm[j], perm[g.below(uint64_t(j) + 1)]);
		int l1, l2;
		if (g.unit() < leaf_share) {
			const int b = int(g.below(uint64_t(n) - 1));
			l2 = n - b;
			l1 = l2 - 1;
		} else {
			const int f = int(g.below(uint64_t(n) - 2));
			const int b = int(g.below(uint64_t(n - 2 - f)));
			l1 = f - 1;
			l2 = n - b;
		}
		int16_t *rec = reinterpret_cast<int16_t *>(base + r * stride);
		std::memset(rec, 0, stride);
		for (int j = 0; j < n; ++j)
			rec[j] = int16_t(perm[j]);
		rec[n] = int16_t(l1);
		rec[n + 1] = int16_t(l2);
		rec[n + 2] = int16_t((l1 + 1) + (n - l2));
	}
	return WSBB_OK;
}

// NEH: jobs by non-increasing total work (stable: lower index first on
// ties), each inserted at the first position with the smallest partial
// makespan. Not part of the reference; it supplies the initial incumbent.
extern "C" int32_t wsbb_neh(const int32_t *p, int n, int m, int32_t *perm_out)
{
	if (n < 1 || n > WSBB_MAX_JOBS || m < 1 || m > WSBB_MAX_MACHINES)
		return -1;
	std::vector<int32_t> order(n), total(n, 0);
	for (int j = 0; j < n; ++j) {
		order[j] = j;
		for (int k = 0; k < m; ++k)
			total[j] += p[k * n + j];
	}
	std::stable_sort(order.begin(), order.end(),
	                 [&](int32_t a, int32_t b) { return total[a] > total[b]; });
	std::vector<int32_t> seq, trial;
	seq.reserve(n);
	for (int32_t job : order) {
		int32_t best = INT32_MAX;
		size_t best_pos = 0;
		for (size_t pos = 0; pos <= seq.size(); ++pos) {
			trial = seq;
			trial.insert(trial.begin() + pos, job);
			const int32_t c = wsbb::sequence_makespan(p, n, m, trial.data(),
			                                          int(trial.size()));
			if (c < best) {
				best = c;
				best_pos = pos;
			}
		}
		seq.insert(seq.begin() + best_pos, job);
	}
	std::copy(seq.begin(), seq.end(), perm_out);
	return wsbb::sequence_makespan(p, n, m, seq.data(), n);
}
