// Internal declarations shared by the host precompute (instance.cpp), the
// bound kernels (bound_kernels.cu), the search (explore.cu) and the C-ABI
// layer (capi.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/wsbb_gb300.h"

namespace wsbb {

// Host precompute of one instance (the reference's initialiserVar,
// src/bound_flowshop.cpp:556-576, restricted to what LB2 reads).
struct Instance {
	int n = 0, m = 0, P = 0;
	std::vector<int32_t> p;        // m x n, machine-major
	std::vector<int32_t> mach0;    // P: first machine of pair i
	std::vector<int32_t> mach1;    // P: second machine of pair i
	std::vector<int32_t> lag;      // P x n
	std::vector<int32_t> johnson;  // P x n: job order of pair i
	std::vector<int32_t> heads;    // m: minTempsArr
	std::vector<int32_t> tails;    // m: minTempsDep
};

// Fills `inst` from p (m x n). Returns an error message, empty on success.
std::string build_instance(const int32_t *p_mxn, int n, int m, Instance &inst);

// Device image of the bound tables. Each CTA stages it into shared memory
// with one linear copy, so it is a single contiguous blob:
//   uint2   johnson_packed[P * n]  pair-major, Johnson order:
//                                  x = job | p[m1][job] << 16
//                                  y = p[m2][job] | lag << 16
//   int32   pt[m * n]              p, machine-major
//   int32   pairs[P]               m1 | m2 << 8
//   int32   heads[m], tails[m]
struct DeviceTables {
	void *blob = nullptr;
	size_t bytes = 0;       // blob size, multiple of 16
	uint32_t off_pt = 0;    // byte offsets inside the blob
	uint32_t off_pairs = 0;
	uint32_t off_heads = 0;
	uint32_t off_tails = 0;
};

std::vector<uint8_t> pack_tables(const Instance &inst, DeviceTables &layout,
                                 std::string &err);

struct BoundParams {
	const uint8_t *tables; // device blob
	uint32_t table_bytes;
	uint32_t off_pt, off_pairs, off_heads, off_tails;
	int n, m, P;
	int stride; // record stride in bytes
};

// Kernel launchers (bound_kernels.cu). `mode`: 0 = LB2, 1 = LB1,
// 2 = makespan of the full permutation.
cudaError_t launch_pool_bounds(const BoundParams &bp, const void *recs,
                               int64_t count, int32_t *out, int mode,
                               int num_sms, cudaStream_t stream);
size_t pool_bounds_smem(const BoundParams &bp, int threads);

}  // namespace wsbb

struct wsbb_ctx {
	int device = 0;
	int num_sms = 0;
	wsbb::Instance inst;
	wsbb::DeviceTables tables;
	wsbb::BoundParams bp;
	std::string last_error;
	// host-buffer path scratch (grown on demand)
	void *d_recs = nullptr;
	int32_t *d_out = nullptr;
	int64_t host_cap = 0;
	cudaStream_t stream = nullptr;
	// search state (explore.cu)
	struct ExploreState *ex = nullptr;
};

int wsbb_set_error(wsbb_ctx *ctx, int code, const std::string &msg);
