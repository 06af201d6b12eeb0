// Device helpers shared by the feature kernels: a node record's front and
// back times (the max-plus recurrences of src/bound_flowshop.cpp:841-895,
// back times for every start machine from one reversed pass) and its
// learned-selector features.
#pragma once

#include <cuda_bf16.h>

#include "wsbb_internal.h"

namespace wsbb {

// Raw front times Fr[k] over job[0..l1] and reversed back times Gr[q] (the
// makespan of job[l2..n-1] on machines m-1-q .. m-1); zeros when empty.
__device__ __forceinline__ void node_times(const int16_t *rec, int n, int m, const int32_t *pt,
                                           int32_t *Fr, int32_t *Gr)
{
	const int l1 = rec[n], l2 = rec[n + 1];
	for (int k = 0; k < m; ++k) {
		Fr[k] = 0;
		Gr[k] = 0;
	}
	for (int j = 0; j <= l1; ++j) {
		const int job = rec[j];
		Fr[0] += pt[job];
		for (int k = 1; k < m; ++k)
			Fr[k] = max(Fr[k], Fr[k - 1]) + pt[k * n + job];
	}
	for (int j = n - 1; j >= l2; --j) {
		const int job = rec[j];
		Gr[0] += pt[(m - 1) * n + job];
		for (int q = 1; q < m; ++q)
			Gr[q] = max(Gr[q], Gr[q - 1]) + pt[(m - 1 - q) * n + job];
	}
}

__device__ __forceinline__ void free_mask(const int16_t *rec, int n, uint32_t (&mask)[4])
{
	const int l1 = rec[n], l2 = rec[n + 1];
	mask[0] = mask[1] = mask[2] = mask[3] = 0;
	for (int j = l1 + 1; j < l2; ++j)
		mask[rec[j] >> 5] |= 1u << (rec[j] & 31);
}

// Features of a node with effective heads He[k] and tails Te[k] (what LB2
// starts from) and free-job mask `mask`: He / scale, Te / scale and the
// remaining work of each machine over the free jobs / scale, each rounded
// to bf16, then the mask as 0/1, zero padding up to D.
__device__ __forceinline__ void write_features(const int32_t *He, const int32_t *Te,
                                               const uint32_t (&mask)[4], int n, int m,
                                               const int32_t *pt, float inv_scale, int D,
                                               float *x)
{
	for (int k = 0; k < m; ++k) {
		int32_t work = 0;
		for (int j = 0; j < n; ++j)
			if ((mask[j >> 5] >> (j & 31)) & 1u)
				work += pt[k * n + j];
		x[k] = __bfloat162float(__float2bfloat16_rn(float(He[k]) * inv_scale));
		x[m + k] = __bfloat162float(__float2bfloat16_rn(float(Te[k]) * inv_scale));
		x[2 * m + k] = __bfloat162float(__float2bfloat16_rn(float(work) * inv_scale));
	}
	for (int j = 0; j < n; ++j)
		x[3 * m + j] = (mask[j >> 5] >> (j & 31)) & 1u ? 1.f : 0.f;
	for (int d = 3 * m + n; d < D; ++d)
		x[d] = 0.f;
}

}  // namespace wsbb
