// Integer max-plus issue-rate probe: the denominator of the LB2 kernel's
// roofline. Each thread runs 8 independent chains of x = max(x + a, y)
// (one add and one max per step, the same operation mix as the Johnson
// recurrence); the achieved add+max operations per second, with every SM
// filled, is the measured peak the bench reports against.
#include "wsbb_internal.h"

namespace {

__global__ void __launch_bounds__(256) maxplus_probe_kernel(int iters, int32_t a, int32_t b,
                                                           int32_t *sink)
{
	int32_t x[8], y[8];
#pragma unroll
	for (int c = 0; c < 8; ++c) {
		x[c] = int32_t(threadIdx.x) * (c + 1);
		y[c] = b + c;
	}
	for (int i = 0; i < iters; ++i) {
#pragma unroll
		for (int c = 0; c < 8; ++c)
			x[c] = max(x[c] + a, y[c] - i);
	}
	int32_t s = 0;
#pragma unroll
	for (int c = 0; c < 8; ++c)
		s ^= x[c];
	if (s == 0x7fffffff)
		sink[blockIdx.x] = s;
}

}  // namespace

extern "C" int wsbb_probe_maxplus_peak(int device, double *ops_per_s)
{
	if (!ops_per_s)
		return WSBB_ERR_ARG;
	if (cudaSetDevice(device) != cudaSuccess)
		return WSBB_ERR_CUDA;
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, maxplus_probe_kernel, 256, 0);
	const int grid = sms * (per_sm > 0 ? per_sm : 1);
	const int iters = 1 << 16;
	int32_t *sink = nullptr;
	if (cudaMalloc(&sink, sizeof(int32_t) * grid) != cudaSuccess)
		return WSBB_ERR_NOMEM;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	maxplus_probe_kernel<<<grid, 256>>>(iters / 8, 3, 1000, sink); // warm-up
	float best_ms = 1e30f;
	for (int r = 0; r < 3; ++r) {
		cudaEventRecord(e0);
		maxplus_probe_kernel<<<grid, 256>>>(iters, 3, 1000, sink);
		cudaEventRecord(e1);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best_ms)
			best_ms = ms;
	}
	cudaError_t e = cudaGetLastError();
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(sink);
	if (e != cudaSuccess)
		return WSBB_ERR_CUDA;
	const double ops = double(grid) * 256.0 * double(iters) * 8.0 * 2.0;
	*ops_per_s = ops / (double(best_ms) * 1e-3);
	return WSBB_OK;
}
