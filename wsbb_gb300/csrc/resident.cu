// The resident search (wsbb_explore_resident): the exact search of one or
// many instances in one cooperative launch of CTAs that stay resident. Its
// CTAs hand each other global data within the launch, so this translation
// unit is compiled with global loads cached in L2 only (-dlcm=cg,
// wsbb_gb300/build.py): no SM can read a stale copy from its own L1. The
// instance tables, constant for the launch, go through the read-only path.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

// The search phases' bodies run on the first 256 threads of a CTA and
// synchronise those alone, on barrier 4 (barrier 0 is the whole CTA's, 1
// and 2 the family groups').
#define WSBB_BODY_SYNC() asm volatile("bar.sync 4, 256;" ::: "memory")
#define WSBB_BODY_SYNC_OR(p) wsbb_body_sync_or(p)
__device__ __forceinline__ int wsbb_body_sync_or(int p)
{
	int r;
	asm volatile("{\n\t.reg .pred a, b;\n\tsetp.ne.s32 a, %1, 0;\n\t"
	             "bar.red.or.pred b, 4, 256, a;\n\tselp.s32 %0, 1, 0, b;\n\t}"
	             : "=r"(r)
	             : "r"(p)
	             : "memory");
	return r;
}

#include "family_staged.cuh"
#include "search_host.h"

namespace wsbb {
namespace {

// ---- resident search ---------------------------------------------------
//
// The same iteration as enqueue_iteration, run by CTAs that stay resident
// for the whole search (one cooperative launch): one group of CTAs per
// instance, so one launch searches many instances. A group's CTAs meet at
// group barriers between the phases; the phases that take one CTA (commit
// and doom, plan, kept scan, finish) run on the group's first CTA. In the
// family phase the iteration's fathers are split into pools; each CTA
// starts at a pool of its own and moves on to the others when it is empty;
// CTAs outside every group, and those whose instance has finished, steal
// fathers from the family phases of the instances still running, so a
// launch keeps every SM busy until the last instance ends. Every wait
// between CTAs is bounded by a %globaltimer limit; one that runs out
// records WSBB_ERR_WATCHDOG for its instance and aborts the launch, every
// CTA leaving at its next wait.

// Father pools: a phase's fathers are split into pools of about
// kFathersPerPool (at most kMaxPools, one per lane of a warp), each with a
// claim counter = phase tag << kTagShift | next index. A claim is valid
// only for the tag it was made under and below its pool's end, so a late
// claim can never take a father of another iteration. The open phase's
// word holds tag << kTagShift | pools << kPoolShift | fathers, so every
// claimer splits the fathers into the same pools. A claim is made by one
// warp, which reads every pool's counter at once and takes the first
// non-empty pool from its own on.
constexpr int kTagShift = 40;
constexpr unsigned long long kIdxMask = (1ull << kTagShift) - 1;
constexpr int kPoolShift = 32;
constexpr unsigned long long kNfMask = (1ull << kPoolShift) - 1;
constexpr int kMaxPools = 32;
constexpr int kFathersPerPool = 16;

struct ResSync {
	unsigned arrive, gen;        // group barrier
	unsigned long long phase;    // open family phase (see kPoolShift; 0: closed)
	unsigned long long fam_done; // fathers bounded in the open phase
	int stopped;                 // the search reached its iteration or node limit
	int hold;                    // watchdog self-test: a flag nothing sets
	int watchdog;                // a wait of this instance ran out
};

struct ResInst {
	ExParams P;
	BoundParams bp;
	FamilyArgs FA;
	const uint32_t *tpack;
	const uint8_t *jobposT;
	staged::StagedLayout L;
	unsigned scratch_off;        // single-CTA phases' shared memory
	ResSync *sync;
	unsigned long long *heads;   // [kMaxPools] pool claim counters
	long long max_iters, max_bounded;
	int first_cta, num_ctas, wide;
};

struct ResGlobal {
	int abort;
	int self_test;
	unsigned finished;           // instances whose search ended
	unsigned long long wait_ns;  // limit of every wait
};

// CTAs of kResThreads: the phases' bodies on the first kResBodyThreads,
// the family phase on kResGroups groups of staged::kFamThreads (as many as
// the instance's shared memory allows), the element-wise phases on all.
constexpr int kResBodyThreads = 256;
constexpr int kResGroups = 2;
constexpr int kResThreads = staged::kFamThreads * kResGroups;
constexpr int kResCommitItems = 16;
static_assert(kResBodyThreads == staged::kFamThreads && kResThreads == 2 * kResBodyThreads,
              "the bodies' barrier (WSBB_BODY_SYNC) counts 256 threads");

__device__ __forceinline__ unsigned long long gtimer()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}
template <typename T>
__device__ __forceinline__ T vload(const T *p)
{
	return *reinterpret_cast<const volatile T *>(p);
}

// Scratch of the single-CTA phases inside the shared-memory window.
struct ResScratch {
	CommitShared commit;
	long long s_ll[32];
	int tile[kScanItems * kResBodyThreads + kScanItems * kResBodyThreads / 32];
	uint8_t inv[kResBodyThreads / 32][WSBB_MAX_JOBS];
};

// Group barrier; the last CTA to arrive runs act() (on its thread 0) before
// releasing the others. False when the launch aborts (a wait ran out).
template <typename Act>
__device__ bool group_barrier(const ResInst &I, ResGlobal *G, Act act)
{
	__shared__ int s_ok;
	__threadfence(); // this thread's global writes, before the group goes on
	__syncthreads();
	if (threadIdx.x == 0) {
		ResSync *S = I.sync;
		int ok = 1;
		const unsigned g0 = vload(&S->gen);
		__threadfence();
		if (atomicAdd(&S->arrive, 1u) == unsigned(I.num_ctas) - 1) {
			atomicExch(&S->arrive, 0u);
			ok = act();
			__threadfence();
			atomicAdd(&S->gen, 1u);
		} else {
			// twice the limit: the releasing CTA may itself wait up to the
			// limit in act()
			const unsigned long long t0 = gtimer();
			while (vload(&S->gen) == g0) {
				if (vload(&G->abort)) {
					ok = 0;
					break;
				}
				if (gtimer() - t0 > 2 * G->wait_ns) {
					atomicExch(&S->watchdog, 1);
					atomicExch(&G->abort, 1);
					ok = 0;
					break;
				}
				__nanosleep(64);
			}
		}
		__threadfence();
		s_ok = ok && !vload(&G->abort);
	}
	__syncthreads();
	return s_ok != 0;
}
__device__ __forceinline__ bool group_barrier(const ResInst &I, ResGlobal *G)
{
	return group_barrier(I, G, [] { return 1; });
}

// Bounded wait (thread 0) until `cond` holds; false (watchdog set) if the
// limit runs out or the launch aborts.
template <typename Cond>
__device__ int bounded_wait(const ResInst &I, ResGlobal *G, Cond cond)
{
	const unsigned long long t0 = gtimer();
	while (!cond()) {
		if (vload(&G->abort))
			return 0;
		if (gtimer() - t0 > G->wait_ns) {
			atomicExch(&I.sync->watchdog, 1);
			atomicExch(&G->abort, 1);
			return 0;
		}
		__nanosleep(64);
	}
	return 1;
}

__device__ __forceinline__ long long pool_start(long long nf, int v, int nc)
{
	return nf * v / nc;
}

// A claim in instance I's open phase `ph` by every lane of one warp: lane
// k looks at pool (own + k) mod pools, and the first lane whose pool still
// holds fathers of that phase takes one by compare-and-swap (so only an
// index of that phase is ever taken); nf on every lane when every pool is
// empty. A failed swap means another claim succeeded, so the loop ends.
__device__ long long claim_father(const ResInst &I, unsigned long long ph, int own)
{
	const int lane = int(threadIdx.x) & 31;
	const long long nf = (long long)(ph & kNfMask);
	const int np = int((ph & kIdxMask) >> kPoolShift);
	const unsigned long long tag = ph >> kTagShift;
	const int v = (own + lane) % max(np, 1);
	const long long end = pool_start(nf, v + 1, max(np, 1));
	for (;;) {
		unsigned long long h = 0;
		bool live = false;
		if (lane < np) {
			h = vload(&I.heads[v]);
			live = (h >> kTagShift) == tag && (long long)(h & kIdxMask) < end;
		}
		const unsigned ball = __ballot_sync(0xffffffffu, live);
		if (ball == 0)
			return nf;
		const int src = __ffs(ball) - 1;
		long long got = -1;
		if (lane == src && atomicCAS(&I.heads[v], h, h + 1) == h)
			got = (long long)(h & kIdxMask);
		got = __shfl_sync(0xffffffffu, got, src);
		if (got >= 0)
			return got;
	}
}

// Bounds fathers of instance I's open phase `ph` in this CTA (tables of I
// staged), each of the instance's I.L.groups groups on its own fathers,
// claiming from pool `own` first; adds them to the phase's count. Every
// thread of the CTA calls it.
__device__ void bound_phase(const ResInst &I, unsigned long long ph, int own, uint8_t *smem)
{
	constexpr int NT = staged::kFamThreads;
	__shared__ long long s_first[kResGroups];
	const long long nf = (long long)(ph & kNfMask);
	const int group = int(threadIdx.x) / NT;
	if (threadIdx.x % NT < 32) { // the group's first warp
		const long long c = group < I.L.groups ? claim_father(I, ph, own) : nf;
		if (threadIdx.x % NT == 0)
			s_first[group] = c;
	}
	__syncthreads();
	const long long first = s_first[group];
	long long done = 0;
	if (first < nf) { // uniform in the group
		auto claim = [&](long long) { return claim_father(I, ph, own); };
		done = I.wide ? staged::staged_fathers<true, NT>(I.FA, I.bp, I.L, smem, group,
		                                                 nf, first, claim)
		              : staged::staged_fathers<false, NT>(I.FA, I.bp, I.L, smem, group,
		                                                  nf, first, claim);
	}
	__threadfence(); // the group's child bounds, before they are counted
	__syncthreads();
	if (threadIdx.x % NT == 0 && done > 0)
		atomicAdd(&I.sync->fam_done, (unsigned long long)done);
}

// One instance's search on its group of CTAs (rank = the CTA's place in
// the group). Returns when the search ends or the launch aborts.
__device__ void run_instance(const ResInst &I, int rank, ResGlobal *G, uint8_t *smem)
{
	ResScratch &X = *reinterpret_cast<ResScratch *>(smem + I.scratch_off);
	ExDev *D = I.P.dev;
	const bool leader = rank == 0;
	const int nc = I.num_ctas, tid = threadIdx.x;
	const bool body = tid < kResBodyThreads; // the threads that run the bodies
	ResSync *S = I.sync;
	staged::staged_load_tables(I.bp, I.tpack, I.jobposT, I.L, smem);
	// the watchdog self-test: the first barrier also waits for a flag that
	// nothing sets
	if (!group_barrier(I, G, [&] {
		    return G->self_test ? bounded_wait(I, G, [&] { return vload(&S->hold) != 0; }) : 1;
	    }))
		return;
	for (long long it = 0;; ++it) {
		if (leader) {
			// limits are checked where an iteration would begin (as the
			// graph-launched search checks them between launches)
			if (tid == 0 && ((I.max_iters > 0 && it >= I.max_iters) ||
			                 (I.max_bounded > 0 && (long long)D->bounded >= I.max_bounded)))
				S->stopped = 1;
			__syncthreads();
			if (!vload(&S->stopped)) {
				if (body)
					commit_body<kResBodyThreads, kResCommitItems>(I.P, X.commit, false);
				__syncthreads();
				if (tid < 32)
					doom_body(I.P);
			}
		}
		if (!group_barrier(I, G))
			return;
		if (vload(&D->done) || vload(&D->error) || vload(&S->stopped))
			return;
		if (body)
			select_count_body(I.P, rank, nc, X.s_ll);
		if (!group_barrier(I, G))
			return;
		if (leader && body)
			select_plan_body<kResBodyThreads>(I.P, X.s_ll);
		if (!group_barrier(I, G))
			return;
		if (body)
			select_write_body(I.P, rank, nc, X.s_ll);
		if (!group_barrier(I, G))
			return;
		make_children_body(I.P, 0, (long long)rank * kResThreads + tid,
		                   (long long)nc * kResThreads);
		// open the family phase: pools of this iteration's fathers under a
		// new tag
		if (!group_barrier(I, G, [&] {
			    const long long nf = vload(&D->n_fathers);
			    const int np = int(max(1ll, min((long long)kMaxPools, nf / kFathersPerPool)));
			    // tags 1 .. 2^24 - 1 (a closed pool counter reads tag 0)
			    const unsigned long long tag = (unsigned long long)(it % 0xffffff) + 1;
			    S->fam_done = 0;
			    for (int v = 0; v < np; ++v)
				    atomicExch(&I.heads[v], tag << kTagShift | (unsigned long long)pool_start(nf, v, np));
			    __threadfence();
			    atomicExch(&S->phase, nf > 0 ? (tag << kTagShift |
			                                    (unsigned long long)np << kPoolShift |
			                                    (unsigned long long)nf)
			                                 : 0ull);
			    return 1;
		    }))
			return;
		{
			const unsigned long long ph = vload(&S->phase);
			if (ph)
				bound_phase(I, ph, rank, smem);
		}
		// close it once every father is bounded, thieves' included
		if (!group_barrier(I, G, [&] {
			    const unsigned long long ph = vload(&S->phase);
			    const unsigned long long nf = ph & kNfMask;
			    const int np = int((ph & kIdxMask) >> kPoolShift);
			    const int ok = ph == 0 ||
			                   bounded_wait(I, G, [&] { return vload(&S->fam_done) >= nf; });
			    atomicExch(&S->phase, 0ull);
			    for (int v = 0; v < np; ++v)
				    atomicExch(&I.heads[v], 0ull);
			    __threadfence();
			    return ok;
		    }))
			return;
		choose_body(I.P, ((long long)rank * kResThreads + tid) >> 5,
		            (long long)nc * (kResThreads / 32));
		if (!group_barrier(I, G))
			return;
		if (leader && body)
			kept_scan_body<kResBodyThreads>(I.P, X.s_ll, X.tile);
		if (!group_barrier(I, G))
			return;
		if (body)
			emit_body(I.P, rank, nc, X.inv);
		if (!group_barrier(I, G))
			return;
		if (leader && tid == 0)
			finish_body(I.P);
		if (leader)
			__syncthreads();
	}
}

__global__ void __launch_bounds__(kResThreads)
    resident_kernel(const ResInst *__restrict__ insts, int K, const int16_t *__restrict__ cta_inst,
                    ResGlobal *G)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const int g = cta_inst[blockIdx.x]; // -1: a CTA outside every group
	if (g >= 0) {
		const ResInst &I = insts[g];
		run_instance(I, int(blockIdx.x) - I.first_cta, G, smem);
		__syncthreads();
		if (threadIdx.x == 0 && int(blockIdx.x) == I.first_cta) {
			__threadfence();
			atomicAdd(&G->finished, 1u);
		}
	}
	const int g0 = g >= 0 ? g : int(blockIdx.x) % K; // where its search for fathers starts
	// then help the instances still running, until every one has ended
	__shared__ int s_go;
	__shared__ unsigned long long s_ph;
	__shared__ int s_j;
	int staged_for = g;
	const unsigned long long t_idle0 = gtimer();
	unsigned long long t_idle = t_idle0;
	for (int round = 0;; ++round) {
		if (threadIdx.x == 0) {
			s_go = 0;
			if (!vload(&G->abort) && vload(&G->finished) < unsigned(K)) {
				s_go = 1;
				s_j = -1;
				for (int k = 1; k <= K; ++k) {
					const int j = (g0 + k + round) % K;
					const unsigned long long ph = vload(&insts[j].sync->phase);
					if (ph) {
						s_j = j;
						s_ph = ph;
						break;
					}
				}
				// nothing open for longer than the wait limit while instances
				// are still running: a group has stopped answering
				if (s_j < 0 && gtimer() - t_idle > 4 * G->wait_ns) {
					atomicExch(&G->abort, 1);
					s_go = 0;
				}
			}
		}
		__syncthreads();
		if (!s_go)
			break;
		const int j = s_j;
		if (j < 0) {
			if (threadIdx.x == 0)
				__nanosleep(200);
			continue;
		}
		if (threadIdx.x == 0)
			t_idle = gtimer();
		__threadfence(); // the phase was seen open: read its fathers after that
		const ResInst &J = insts[j];
		if (staged_for != j) {
			__syncthreads();
			staged::staged_load_tables(J.bp, J.tpack, J.jobposT, J.L, smem);
			staged_for = j;
		}
		bound_phase(J, s_ph, int(blockIdx.x), smem);
		__syncthreads();
	}
}

}  // namespace
}  // namespace wsbb

using namespace wsbb::host;

// ---------------------------------------------------------------------------
// wsbb_explore_resident: the search of one or many instances in one
// cooperative launch of resident CTAs (resident_kernel above).

namespace {

// Whether a context's instance can run in the resident search (the staged
// family bounds: packed tables, 16-bit staircase paths, P <= 192 pairs).
bool resident_eligible(const wsbb_ctx *ctx)
{
	return ctx->tables.tpack && ctx->bp.span16 && ctx->bp.P <= wsbb::staged::kWalkThreads;
}

}  // namespace

extern "C" int wsbb_explore_resident(wsbb_ctx *const *ctxs, int count,
                                     const wsbb_explore_cfg *cfgs,
                                     const wsbb_resident_opts *opts, wsbb_stats *stats,
                                     void *stream_v)
{
	using namespace wsbb;
	if (!ctxs || count <= 0 || count > 32767 || !cfgs || !stats)
		return WSBB_ERR_ARG;
	for (int k = 0; k < count; ++k)
		if (!ctxs[k])
			return WSBB_ERR_ARG;
	wsbb_ctx *c0 = ctxs[0];
	const int device = c0->device;
	for (int k = 0; k < count; ++k) {
		wsbb_ctx *ctx = ctxs[k];
		if (ctx->device != device)
			return wsbb_set_error(c0, WSBB_ERR_ARG, "resident search: contexts on different devices");
		if (!resident_eligible(ctx))
			return wsbb_set_error(ctx, WSBB_ERR_ARG,
			                      "resident search: the instance needs the chunked family bounds "
			                      "(a time above 127, m above 20 or paths above 16 bits)");
		if (cfgs[k].flags & (WSBB_EXPLORE_RESUME | WSBB_EXPLORE_CHILD_LB2))
			return wsbb_set_error(ctx, WSBB_ERR_ARG,
			                      "resident search: no resume, no per-child bounds");
		for (int q = 0; q < k; ++q)
			if (ctxs[q] == ctx)
				return wsbb_set_error(ctx, WSBB_ERR_ARG, "resident search: a context twice");
	}
	cudaError_t e = cudaSetDevice(device);
	if (e != cudaSuccess)
		return ex_fail(c0, e, "cudaSetDevice");
	const int wait_ms = opts && opts->wait_ms > 0 ? opts->wait_ms : 2000;
	const int self_test = opts ? opts->self_test : 0;

	int max_optin = 0;
	e = cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
	if (e != cudaSuccess)
		return ex_fail(c0, e, "device attribute");

	// search states and layouts
	std::vector<ResInst> H((size_t)count);
	size_t smem = 0;
	for (int k = 0; k < count; ++k) {
		wsbb_ctx *ctx = ctxs[k];
		int window = 0;
		long long cap = 0, region_cap = 0;
		int rc = search_shape(ctx, &cfgs[k], window, cap, region_cap);
		if (rc == WSBB_OK)
			rc = search_state(ctx, window, cap, region_cap);
		if (rc != WSBB_OK)
			return rc;
		ExploreState *X = ctx->ex;
		X->P.log_rec = nullptr;
		X->P.log_cap = 0;
		ResInst &I = H[size_t(k)];
		std::memset(&I, 0, sizeof(I));
		I.P = X->P;
		I.bp = ctx->bp;
		I.FA.fathers = X->P.tmp_rec;
		I.FA.ridx = X->P.father_ridx;
		I.FA.child_off = X->P.child_off;
		I.FA.child_lb = X->P.child_lb;
		I.FA.child_job = X->P.child_job;
		I.FA.stride = X->P.stride;
		I.tpack = ctx->tables.tpack;
		I.jobposT = ctx->tables.jobposT;
		// the family groups: as many as fit one CTA's shared memory, with
		// the single-CTA phases' scratch in the first group's region when
		// it is large enough, else after the groups
		for (int groups = kResGroups; groups >= 1; --groups) {
			I.L = staged::staged_layout(ctx->bp.n, ctx->bp.m, ctx->bp.P, ctx->tables.Pp, groups);
			I.scratch_off = I.L.grp_bytes >= sizeof(ResScratch)
			                    ? unsigned(I.L.off_grp)
			                    : unsigned((I.L.bytes + 15) & ~size_t(15));
			if (std::max(I.L.bytes, size_t(I.scratch_off) + sizeof(ResScratch)) + 1024 <=
			    size_t(max_optin))
				break;
		}
		smem = std::max(smem, std::max(I.L.bytes, size_t(I.scratch_off) + sizeof(ResScratch)));
		I.max_iters = cfgs[k].max_iters;
		I.max_bounded = cfgs[k].max_bounded;
		I.wide = ctx->bp.n > 64;
	}
	if (smem > size_t(max_optin))
		return wsbb_set_error(c0, WSBB_ERR_ARG, "resident search: instances too large for one CTA");
	e = allow_max_dynamic_smem(resident_kernel);
	int occ = 0;
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, resident_kernel, kResThreads, smem);
	if (e != cudaSuccess)
		return ex_fail(c0, e, "resident occupancy");
	const int grid = c0->num_sms * std::max(occ, 1);
	if (occ < 1 || grid < count)
		return wsbb_set_error(c0, WSBB_ERR_ARG,
		                      "resident search: more instances than resident CTAs (" +
		                          std::to_string(grid) + ")");
	// groups: an equal share of the CTAs per instance, at most group_ctas
	// when the caller sets it; the CTAs left over take fathers from every
	// instance's bound phase (for one instance the whole grid in its group
	// is the fastest: its bound phase gains more than its barriers lose)
	const int group_cap = opts && opts->group_ctas > 0 ? opts->group_ctas : grid;
	std::vector<int16_t> cta_inst((size_t)grid, int16_t(-1));
	int at = 0;
	const int heads = kMaxPools * count;
	for (int k = 0; k < count; ++k) {
		const int nc = std::min(grid / count + (k < grid % count ? 1 : 0), group_cap);
		H[size_t(k)].first_cta = at;
		H[size_t(k)].num_ctas = nc;
		for (int b = 0; b < nc; ++b)
			cta_inst[size_t(at + b)] = int16_t(k);
		at += nc;
	}
	// device copies: instances, their sync words and pool counters, the
	// CTA map, the launch's own words
	auto a256 = [](size_t v) { return (v + 255) & ~size_t(255); };
	const size_t off_sync = a256(sizeof(ResInst) * size_t(count));
	const size_t off_heads = off_sync + a256(sizeof(ResSync) * size_t(count));
	const size_t off_map = off_heads + a256(8 * size_t(heads));
	const size_t off_glob = off_map + a256(2 * size_t(grid));
	const size_t bytes = off_glob + a256(sizeof(ResGlobal));
	uint8_t *mem = nullptr;
	e = cudaMalloc(&mem, bytes);
	if (e != cudaSuccess)
		return wsbb_set_error(c0, WSBB_ERR_NOMEM, "resident search buffers");
	ResSync *d_sync = reinterpret_cast<ResSync *>(mem + off_sync);
	unsigned long long *d_heads = reinterpret_cast<unsigned long long *>(mem + off_heads);
	for (int k = 0; k < count; ++k) {
		H[size_t(k)].sync = d_sync + k;
		H[size_t(k)].heads = d_heads + size_t(k) * kMaxPools;
	}
	ResGlobal glob{};
	glob.self_test = self_test;
	glob.wait_ns = (unsigned long long)wait_ms * 1000000ull;
	cudaStream_t s = stream_v ? static_cast<cudaStream_t>(stream_v) : c0->stream;
	if (!stream_v)
		e = wait_for_legacy(s, c0->legacy_ev);
	if (e == cudaSuccess)
		e = cudaMemsetAsync(mem + off_sync, 0, off_map - off_sync, s);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(mem, H.data(), sizeof(ResInst) * size_t(count), cudaMemcpyHostToDevice, s);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(mem + off_map, cta_inst.data(), 2 * size_t(grid),
		                    cudaMemcpyHostToDevice, s);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(mem + off_glob, &glob, sizeof(glob), cudaMemcpyHostToDevice, s);
	for (int k = 0; k < count && e == cudaSuccess; ++k) {
		ExploreState *X = ctxs[k]->ex;
		init_kernel<<<1, 128, 0, s>>>(X->P, cfgs[k].ub0, cfgs[k].best, window_min_of(X->window),
		                              X->window, cfgs[k].max_iters > 0 || cfgs[k].max_bounded > 0);
		e = cudaGetLastError();
	}
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;
	if (e == cudaSuccess)
		e = cudaEventCreate(&ev0);
	if (e == cudaSuccess)
		e = cudaEventCreate(&ev1);
	if (e == cudaSuccess)
		e = cudaEventRecord(ev0, s);
	if (e == cudaSuccess) {
		const ResInst *a_insts = reinterpret_cast<const ResInst *>(mem);
		int a_count = count;
		const int16_t *a_map = reinterpret_cast<const int16_t *>(mem + off_map);
		ResGlobal *a_glob = reinterpret_cast<ResGlobal *>(mem + off_glob);
		void *args[] = {&a_insts, &a_count, &a_map, &a_glob};
		e = cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(resident_kernel), grid,
		                                kResThreads, args, smem, s);
	}
	if (e == cudaSuccess)
		e = cudaEventRecord(ev1, s);
	if (e == cudaSuccess)
		e = cudaEventSynchronize(ev1);
	float ms = 0;
	if (e == cudaSuccess)
		cudaEventElapsedTime(&ms, ev0, ev1);
	std::vector<ResSync> hs((size_t)count);
	if (e == cudaSuccess)
		e = cudaMemcpy(hs.data(), d_sync, sizeof(ResSync) * size_t(count), cudaMemcpyDeviceToHost);
	int rc = WSBB_OK;
	for (int k = 0; k < count && e == cudaSuccess; ++k) {
		ExploreState *X = ctxs[k]->ex;
		ExDev h{};
		std::vector<int16_t> best_rec(size_t(ctxs[k]->bp.stride / 2));
		e = cudaMemcpy(&h, X->P.dev, sizeof(ExDev), cudaMemcpyDeviceToHost);
		if (e == cudaSuccess)
			e = cudaMemcpy(best_rec.data(), X->P.best_rec, size_t(ctxs[k]->bp.stride),
			               cudaMemcpyDeviceToHost);
		if (e != cudaSuccess)
			break;
		const int status = h.done ? 0 : 1;
		if (hs[size_t(k)].watchdog && !h.error)
			h.error = WSBB_ERR_WATCHDOG;
		fill_stats(h, best_rec.data(), ctxs[k]->inst.n, status, ms * 1e-3, 1,
		           ctxs[k]->bp.stride, &stats[k]);
		if (h.error) {
			rc = rc == WSBB_OK || h.error == WSBB_ERR_WATCHDOG ? h.error : rc;
			wsbb_set_error(ctxs[k], h.error,
			               h.error == WSBB_ERR_WATCHDOG
			                   ? "resident search: a wait between CTAs ran out"
			                   : "search pool capacity exceeded");
		} else if (!h.done && !hs[size_t(k)].stopped) {
			// the launch aborted on another instance's watchdog
			stats[k].status = WSBB_ERR_WATCHDOG;
			rc = WSBB_ERR_WATCHDOG;
			wsbb_set_error(ctxs[k], WSBB_ERR_WATCHDOG,
			               "resident search: the launch stopped on a watchdog");
		}
	}
	if (ev0)
		cudaEventDestroy(ev0);
	if (ev1)
		cudaEventDestroy(ev1);
	cudaFree(mem);
	if (e != cudaSuccess)
		return ex_fail(c0, e, "resident search");
	return rc;
}

