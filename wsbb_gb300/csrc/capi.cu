// C-ABI entry points (include/wsbb_gb300.h): context set-up (instance
// precompute + device tables), pool bounds on device or host buffers.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>

#include <mutex>
#include <set>
#include <utility>

#include "wsbb_internal.h"

int wsbb_set_error(wsbb_ctx *ctx, int code, const std::string &msg)
{
	if (ctx)
		ctx->last_error = msg;
	return code;
}

namespace {

int cuda_fail(wsbb_ctx *ctx, cudaError_t e, const char *what)
{
	return wsbb_set_error(ctx, WSBB_ERR_CUDA,
	                      std::string(what) + ": " + cudaGetErrorString(e));
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int pool_call(wsbb_ctx *ctx, const void *recs, int64_t count, int32_t *out, void *stream,
              int mode)
{
	if (!ctx)
		return WSBB_ERR_ARG;
	if (count < 0 || (count > 0 && (!recs || !out)))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "null buffer or negative count");
	if (!aligned16(recs))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "records must be 16-byte aligned");
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "cudaSetDevice");
	e = wsbb::launch_pool_bounds(ctx->bp, recs, count, out, mode, ctx->num_sms,
	                             static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "bound kernel launch");
	return WSBB_OK;
}

}  // namespace

extern "C" int wsbb_ctx_create(const int32_t *p, int n, int m, int device, wsbb_ctx **out)
{
	if (!out || !p)
		return WSBB_ERR_ARG;
	*out = nullptr;
	wsbb_ctx *ctx = new (std::nothrow) wsbb_ctx();
	if (!ctx)
		return WSBB_ERR_NOMEM;
	std::string err = wsbb::build_instance(p, n, m, ctx->inst);
	if (!err.empty()) {
		fprintf(stderr, "wsbb_ctx_create: %s\n", err.c_str());
		delete ctx;
		return WSBB_ERR_ARG;
	}
	wsbb::HostTables H = wsbb::pack_tables(ctx->inst, err);
	if (!err.empty()) {
		fprintf(stderr, "wsbb_ctx_create: %s\n", err.c_str());
		delete ctx;
		return WSBB_ERR_RANGE;
	}
	ctx->device = device;
	wsbb::DeviceTables &T = ctx->tables;
	T.bytes = H.img8.size() + H.img16.size() + H.imgT.size() + H.imgPos.size();
	const size_t off_pack = (T.bytes + 255) & ~size_t(255);
	if (!H.imgPack.empty())
		T.bytes = off_pack + H.imgPack.size();
	cudaError_t e = cudaSetDevice(device);
	if (e == cudaSuccess)
		e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
	if (e == cudaSuccess)
		e = cudaMalloc(&T.mem, T.bytes);
	uint8_t *base = static_cast<uint8_t *>(T.mem);
	if (e == cudaSuccess)
		e = cudaMemcpy(base, H.img8.data(), H.img8.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && !H.img16.empty())
		e = cudaMemcpy(base + H.img8.size(), H.img16.data(), H.img16.size(),
		               cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMemcpy(base + H.img8.size() + H.img16.size(), H.imgT.data(), H.imgT.size(),
		               cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMemcpy(base + H.img8.size() + H.img16.size() + H.imgT.size(), H.imgPos.data(),
		               H.imgPos.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess && !H.imgPack.empty())
		e = cudaMemcpy(base + off_pack, H.imgPack.data(), H.imgPack.size(),
		               cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMalloc(&ctx->d_claim, sizeof(unsigned long long));
	if (e == cudaSuccess)
		e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess)
		e = cudaEventCreateWithFlags(&ctx->legacy_ev, cudaEventDisableTiming);
	if (e != cudaSuccess) {
		fprintf(stderr, "wsbb_ctx_create: %s\n", cudaGetErrorString(e));
		wsbb_ctx_destroy(ctx);
		return WSBB_ERR_CUDA;
	}
	T.t8 = H.t8;
	T.t8.blob = base;
	T.t16 = H.t16;
	T.t16.blob = H.img16.empty() ? nullptr : base + H.img8.size();
	T.johnsonT = reinterpret_cast<const uint2 *>(base + H.img8.size() + H.img16.size());
	T.jobposT = base + H.img8.size() + H.img16.size() + H.imgT.size();
	if (!H.imgPack.empty()) {
		T.tpack = reinterpret_cast<const uint32_t *>(base + off_pack);
		T.Pp = H.Pp;
	}
	wsbb::BoundParams &bp = ctx->bp;
	bp.t8 = T.t8;
	bp.t16 = T.t16;
	bp.n = n;
	bp.m = m;
	bp.P = ctx->inst.P;
	bp.stride = int(wsbb_node_stride(n));
	int64_t total = 0;
	for (int32_t v : ctx->inst.p)
		total += v;
	bp.col16 = total < 32768 ? 1 : 0;
	int32_t pmax = 0;
	for (int32_t v : ctx->inst.p)
		pmax = std::max(pmax, v);
	bp.span16 = int64_t(n + m - 1) * pmax <= 65535 ? 1 : 0;
	*out = ctx;
	return WSBB_OK;
}

void wsbb_explore_release(wsbb_ctx *ctx);

extern "C" void wsbb_ctx_destroy(wsbb_ctx *ctx)
{
	if (!ctx)
		return;
	cudaSetDevice(ctx->device);
	wsbb_explore_release(ctx);
	if (ctx->tables.mem)
		cudaFree(ctx->tables.mem);
	if (ctx->d_recs)
		cudaFree(ctx->d_recs);
	if (ctx->d_out)
		cudaFree(ctx->d_out);
	if (ctx->d_claim)
		cudaFree(ctx->d_claim);
	if (ctx->stream)
		cudaStreamDestroy(ctx->stream);
	if (ctx->legacy_ev)
		cudaEventDestroy(ctx->legacy_ev);
	delete ctx;
}

namespace wsbb {
cudaError_t allow_max_dynamic_smem_fn(const void *kernel)
{
	static std::mutex mu;
	static std::set<std::pair<int, const void *>> done;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess)
		return e;
	std::lock_guard<std::mutex> lock(mu);
	if (done.count({dev, kernel}))
		return cudaSuccess;
	int max_optin = 0;
	e = cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
	// the ceiling covers dynamic shared memory only: the kernel's static
	// shared memory comes off the device's per-block maximum
	cudaFuncAttributes fa;
	if (e == cudaSuccess)
		e = cudaFuncGetAttributes(&fa, kernel);
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         max_optin - int(fa.sharedSizeBytes));
	if (e == cudaSuccess)
		done.insert({dev, kernel});
	return e;
}
}  // namespace wsbb

extern "C" size_t wsbb_ctx_device_bytes(const wsbb_ctx *ctx)
{
	return ctx ? ctx->tables.bytes : 0;
}

extern "C" const char *wsbb_last_error(const wsbb_ctx *ctx)
{
	return ctx ? ctx->last_error.c_str() : "null context";
}

namespace {
int copy_tables(const wsbb::Instance &I, int32_t *mach0, int32_t *mach1, int32_t *lag,
                int32_t *johnson, int32_t *heads, int32_t *tails)
{
	auto put = [](int32_t *dst, const std::vector<int32_t> &src) {
		if (dst)
			std::memcpy(dst, src.data(), src.size() * sizeof(int32_t));
	};
	put(mach0, I.mach0);
	put(mach1, I.mach1);
	put(lag, I.lag);
	put(johnson, I.johnson);
	put(heads, I.heads);
	put(tails, I.tails);
	return WSBB_OK;
}
}  // namespace

extern "C" int wsbb_ctx_tables(const wsbb_ctx *ctx, int32_t *mach0, int32_t *mach1,
                               int32_t *lag, int32_t *johnson, int32_t *heads, int32_t *tails)
{
	if (!ctx)
		return WSBB_ERR_ARG;
	return copy_tables(ctx->inst, mach0, mach1, lag, johnson, heads, tails);
}

extern "C" int wsbb_precompute(const int32_t *p, int n, int m, int32_t *mach0, int32_t *mach1,
                               int32_t *lag, int32_t *johnson, int32_t *heads, int32_t *tails)
{
	if (!p)
		return WSBB_ERR_ARG;
	wsbb::Instance I;
	if (!wsbb::build_instance(p, n, m, I).empty())
		return WSBB_ERR_ARG;
	return copy_tables(I, mach0, mach1, lag, johnson, heads, tails);
}

extern "C" int wsbb_lb2_eval(wsbb_ctx *ctx, const void *recs, int64_t count, int32_t *out,
                             void *stream)
{
	return pool_call(ctx, recs, count, out, stream, 0);
}

extern "C" int wsbb_lb1_eval(wsbb_ctx *ctx, const void *recs, int64_t count, int32_t *out,
                             void *stream)
{
	return pool_call(ctx, recs, count, out, stream, 1);
}

extern "C" int wsbb_makespan_eval(wsbb_ctx *ctx, const void *recs, int64_t count,
                                  int32_t *out, void *stream)
{
	return pool_call(ctx, recs, count, out, stream, 2);
}

extern "C" int wsbb_lb2_eval_host(wsbb_ctx *ctx, const void *host_recs, int64_t count,
                                  int32_t *host_out)
{
	if (!ctx)
		return WSBB_ERR_ARG;
	if (count < 0 || (count > 0 && (!host_recs || !host_out)))
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "null buffer or negative count");
	if (count == 0)
		return WSBB_OK;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "cudaSetDevice");
	const size_t stride = size_t(ctx->bp.stride);
	if (count > ctx->host_cap) {
		if (ctx->d_recs)
			cudaFree(ctx->d_recs);
		if (ctx->d_out)
			cudaFree(ctx->d_out);
		ctx->d_recs = nullptr;
		ctx->d_out = nullptr;
		ctx->host_cap = 0;
		e = cudaMalloc(&ctx->d_recs, size_t(count) * stride);
		if (e == cudaSuccess)
			e = cudaMalloc(&ctx->d_out, size_t(count) * sizeof(int32_t));
		if (e != cudaSuccess)
			return wsbb_set_error(ctx, WSBB_ERR_NOMEM, "device pool allocation failed");
		ctx->host_cap = count;
	}
	e = cudaMemcpyAsync(ctx->d_recs, host_recs, size_t(count) * stride,
	                    cudaMemcpyHostToDevice, ctx->stream);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "pool upload");
	e = wsbb::launch_pool_bounds(ctx->bp, ctx->d_recs, count, ctx->d_out, 0, ctx->num_sms,
	                             ctx->stream);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "bound kernel launch");
	e = cudaMemcpyAsync(host_out, ctx->d_out, size_t(count) * sizeof(int32_t),
	                    cudaMemcpyDeviceToHost, ctx->stream);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "bound download");
	e = cudaStreamSynchronize(ctx->stream);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "pool round trip");
	return WSBB_OK;
}
