// Learned machine-pair selector: a 3-layer MLP that reads a node's features
// and ranks the machine pairs most likely to bind its LB2, so a search can
// try K pairs first and settle most children without the other P - K.
//
//   features  x[0..m)      effective heads / scale (front times if jobs are
//                          fixed at the front, else the static heads — what
//                          LB2 itself starts from)
//             x[m..2m)     effective tails / scale (back times or static
//                          tails)
//             x[2m..3m)    remaining work of each machine over the free
//                          jobs / scale (where the bottleneck is)
//             x[3m..3m+n)  1 for each job still free
//             padded with zeros to D = round_up(3m + n, 16); scale = the
//             largest machine load of the instance
//   network   D -> 128 -> 128 -> P logits (ReLU), bf16 operands with fp32
//             accumulation; logits are padded to O = round_up(P, 8)
//   label     the binding pair of the node's LB2 (the first pair reaching
//             the maximum, the order the reference's own binding-pair
//             statistic uses, src/bound_flowshop.cpp:150-153)
//
// Training runs on the GPU with these kernels: fp32 tiled GEMMs (forward
// operands rounded to bf16 exactly as inference sees them, straight-through
// for the gradient), softmax cross-entropy, ReLU backward, bias sums and
// Adam. Inference is one fused kernel per tile of 16 nodes per warp: three
// bf16 mma.sync layers with fp32 accumulators, then top-K of the P logits.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "node_features.cuh"
#include "wsbb_internal.h"

namespace wsbb {
namespace {

constexpr int kHidden = 128;

__device__ __forceinline__ float round_bf16(float x)
{
	return __bfloat162float(__float2bfloat16_rn(x));
}

// ---------------------------------------------------------------- features

// Per node record: effective heads and tails (the values LB2 starts from),
// the free-job mask, optionally the binding pair. One thread per record;
// tables read through the 8-byte image (data preparation, not the hot path).
__global__ void features_kernel(BoundParams bp, const uint8_t *__restrict__ recs, long long count,
                                float inv_scale, int D, float *__restrict__ X,
                                int32_t *__restrict__ labels)
{
	const int n = bp.n, m = bp.m, P = bp.P;
	const uint8_t *tb = bp.t8.blob;
	const int32_t *pt = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pt);
	const int32_t *pairs = reinterpret_cast<const int32_t *>(tb + bp.t8.off_pairs);
	const int32_t *heads = reinterpret_cast<const int32_t *>(tb + bp.t8.off_heads);
	const int32_t *tails = reinterpret_cast<const int32_t *>(tb + bp.t8.off_tails);
	const uint2 *tj = reinterpret_cast<const uint2 *>(tb);
	for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < count;
	     r += (long long)gridDim.x * blockDim.x) {
		const int16_t *rec = reinterpret_cast<const int16_t *>(recs + r * bp.stride);
		const int l1 = rec[n], l2 = rec[n + 1];
		int32_t F[WSBB_MAX_MACHINES], G[WSBB_MAX_MACHINES], R[WSBB_MAX_MACHINES];
		node_times(rec, n, m, pt, F, G);
		for (int k = 0; k < m; ++k) {
			F[k] = l1 >= 0 ? F[k] : heads[k];
			R[k] = l2 < n ? G[m - 1 - k] : tails[k];
		}
		uint32_t mask[4];
		free_mask(rec, n, mask);
		write_features(F, R, mask, n, m, pt, inv_scale, D, X + r * D);
		if (!labels)
			continue;
		if (l2 - l1 == 1) {
			labels[r] = -1;
			continue;
		}
		int32_t lb = 0, arg = -1;
		for (int i = 0; i < P; ++i) {
			const int a = pairs[i] & 0xff, c = pairs[i] >> 8;
			int32_t t0 = F[a], t1 = F[c];
			for (int q = 0; q < n; ++q) {
				const uint2 v = tj[i * n + q];
				const int job = int(v.x & 0xffu);
				if ((mask[job >> 5] >> (job & 31)) & 1u) {
					t0 += int32_t(v.x >> 16);
					t1 = max(t1, t0 + int32_t(v.y >> 16)) + int32_t(v.y & 0xffffu);
				}
			}
			const int32_t val = l2 < n ? max(t1 + R[c], t0 + R[a]) : t1 + tails[c];
			if (val > lb) {
				lb = val;
				arg = i;
			}
		}
		labels[r] = arg;
	}
}

// ------------------------------------------------------------ SIMT GEMM (fp32)

// C[M x N] = A[M x K] * B[K x N] with arbitrary element strides (so that
// transposed operands need no copy), then optional bias (per column), ReLU,
// bf16 rounding of the result, and accumulation into C.
struct GemmArgs {
	const float *A;
	long long sam, sak;
	const float *B;
	long long sbk, sbn;
	float *C;
	long long ldc;
	const float *bias;
	int M, N, K;
	int relu, round_out, accumulate;
};

constexpr int kTM = 64, kTN = 64, kTK = 16;

__global__ void __launch_bounds__(256) gemm_kernel(GemmArgs g)
{
	__shared__ float As[kTK][kTM + 4];
	__shared__ float Bs[kTK][kTN + 4];
	const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
	const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
	float acc[4][4] = {};
	for (int k0 = 0; k0 < g.K; k0 += kTK) {
		for (int i = threadIdx.x; i < kTK * kTM; i += 256) {
			const int kk = i / kTM, mm = i % kTM;
			const int gm = m0 + mm, gk = k0 + kk;
			As[kk][mm] = (gm < g.M && gk < g.K) ? g.A[gm * g.sam + gk * g.sak] : 0.f;
		}
		for (int i = threadIdx.x; i < kTK * kTN; i += 256) {
			const int kk = i / kTN, nn = i % kTN;
			const int gn = n0 + nn, gk = k0 + kk;
			Bs[kk][nn] = (gn < g.N && gk < g.K) ? g.B[gk * g.sbk + gn * g.sbn] : 0.f;
		}
		__syncthreads();
#pragma unroll
		for (int kk = 0; kk < kTK; ++kk) {
			float a[4], b[4];
#pragma unroll
			for (int i = 0; i < 4; ++i) {
				a[i] = As[kk][ty * 4 + i];
				b[i] = Bs[kk][tx * 4 + i];
			}
#pragma unroll
			for (int i = 0; i < 4; ++i)
#pragma unroll
				for (int j = 0; j < 4; ++j)
					acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
		}
		__syncthreads();
	}
#pragma unroll
	for (int i = 0; i < 4; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
			if (gm >= g.M || gn >= g.N)
				continue;
			float v = acc[i][j];
			if (g.bias)
				v += g.bias[gn];
			if (g.relu)
				v = fmaxf(v, 0.f);
			if (g.round_out)
				v = round_bf16(v);
			float *c = g.C + gm * g.ldc + gn;
			*c = g.accumulate ? *c + v : v;
		}
}

void gemm(cudaStream_t s, const float *A, long long sam, long long sak, const float *B,
          long long sbk, long long sbn, float *C, long long ldc, int M, int N, int K,
          const float *bias = nullptr, int relu = 0, int round_out = 0, int accumulate = 0)
{
	GemmArgs g{A, sam, sak, B, sbk, sbn, C, ldc, bias, M, N, K, relu, round_out, accumulate};
	dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM);
	gemm_kernel<<<grid, 256, 0, s>>>(g);
}

// Softmax cross-entropy over the first P of O logits; writes dZ = (softmax -
// onehot) / B (zero on padding) and adds the batch's loss sum to *loss.
// Rows whose label is outside [0, P) contribute nothing. One warp per row.
__global__ void softmax_xent_kernel(const float *Z, const int32_t *y, int B, int O, int P,
                                    float inv_b, float *dZ, float *loss)
{
	const int lane = threadIdx.x & 31;
	const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	if (row >= B)
		return;
	const float *z = Z + (long long)row * O;
	float *dz = dZ + (long long)row * O;
	const int label = y[row] < P ? y[row] : -1;
	float mx = -INFINITY;
	for (int o = lane; o < P; o += 32)
		mx = fmaxf(mx, z[o]);
	for (int d = 16; d > 0; d >>= 1)
		mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
	float se = 0.f;
	for (int o = lane; o < P; o += 32)
		se += expf(z[o] - mx);
	for (int d = 16; d > 0; d >>= 1)
		se += __shfl_xor_sync(0xffffffffu, se, d);
	for (int o = lane; o < O; o += 32) {
		float g = 0.f;
		if (label >= 0 && o < P)
			g = (expf(z[o] - mx) / se - (o == label ? 1.f : 0.f)) * inv_b;
		dz[o] = g;
	}
	if (lane == 0 && label >= 0)
		atomicAdd(loss, logf(se) + mx - z[label]);
}

// dA *= (H > 0): the ReLU backward on a (rows x cols) activation.
__global__ void relu_back_kernel(float *dA, const float *H, long long count)
{
	for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
	     i += (long long)gridDim.x * blockDim.x)
		if (!(H[i] > 0.f))
			dA[i] = 0.f;
}

// Column sums (bias gradients): out[c] = sum_r M[r, c]. One thread per column.
__global__ void colsum_kernel(const float *Mx, int rows, int cols, float *out)
{
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= cols)
		return;
	float s = 0.f;
	for (int r = 0; r < rows; ++r)
		s += Mx[(long long)r * cols + c];
	out[c] = s;
}

__global__ void round_copy_kernel(const float *src, float *dst, long long count)
{
	for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
	     i += (long long)gridDim.x * blockDim.x)
		dst[i] = round_bf16(src[i]);
}

__global__ void adam_kernel(float *w, const float *g, float *mo, float *ve, long long count,
                            float lr, float b1, float b2, float eps, float c1, float c2)
{
	for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
	     i += (long long)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * mo[i] + (1.f - b1) * gi;
		const float vi = b2 * ve[i] + (1.f - b2) * gi * gi;
		mo[i] = mi;
		ve[i] = vi;
		w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
	}
}

// Gather rows idx[r] of src (cols wide) into dst.
__global__ void gather_rows_kernel(const float *src, const int32_t *ysrc, const long long *idx,
                                   int rows, int cols, float *dst, int32_t *ydst)
{
	const int r = blockIdx.x;
	if (r >= rows)
		return;
	const long long s = idx[r];
	for (int c = threadIdx.x; c < cols; c += blockDim.x)
		dst[(long long)r * cols + c] = src[s * cols + c];
	if (threadIdx.x == 0)
		ydst[r] = ysrc[s];
}

// Weights for inference: bf16, each layer transposed to [out][in].
__global__ void pack_infer_kernel(const float *w, int D, int O, __nv_bfloat16 *w1t,
                                  __nv_bfloat16 *w2t, __nv_bfloat16 *w3t)
{
	const int H = kHidden;
	const float *W1 = w, *W2 = w + D * H + H, *W3 = W2 + H * H + H;
	const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	const long long n1 = (long long)H * D, n2 = (long long)H * H, n3 = (long long)O * H;
	if (tid < n1) {
		const int o = int(tid / D), i = int(tid % D);
		w1t[tid] = __float2bfloat16_rn(W1[i * H + o]);
	} else if (tid < n1 + n2) {
		const long long t = tid - n1;
		const int o = int(t / H), i = int(t % H);
		w2t[t] = __float2bfloat16_rn(W2[i * H + o]);
	} else if (tid < n1 + n2 + n3) {
		const long long t = tid - n1 - n2;
		const int o = int(t / H), i = int(t % H);
		w3t[t] = __float2bfloat16_rn(W3[i * O + o]);
	}
}

// ------------------------------------------------------- fused inference

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1)
{
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
	    "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
	    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p)
{
	return *reinterpret_cast<const uint32_t *>(p);
}

// One 16-row layer on the tensor cores: out[16][N] = act(in[16][K] * W^T + b)
// with W given as wt[N][K] (bf16, global), in from shared memory (bf16,
// row stride lda), out written to shared memory as bf16 (hidden layers) or
// fp32 (logits). N is processed in blocks of 64 columns (8 n-tiles).
template <bool kLogits>
__device__ void mma_layer(const __nv_bfloat16 *in, int lda, int K, const __nv_bfloat16 *wt,
                          const float *bias, int N, void *out, int ldo)
{
	const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
	for (int nb = 0; nb < N; nb += 64) {
		float acc[8][4];
#pragma unroll
		for (int t = 0; t < 8; ++t)
			acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
		for (int k0 = 0; k0 < K; k0 += 16) {
			uint32_t a[4];
			a[0] = ld_pair(in + g * lda + k0 + tq * 2);
			a[1] = ld_pair(in + (g + 8) * lda + k0 + tq * 2);
			a[2] = ld_pair(in + g * lda + k0 + 8 + tq * 2);
			a[3] = ld_pair(in + (g + 8) * lda + k0 + 8 + tq * 2);
#pragma unroll
			for (int t = 0; t < 8; ++t) {
				const int ncol = nb + t * 8 + g;
				if (nb + t * 8 >= N)
					break;
				const uint32_t b0 = ld_pair(wt + (long long)ncol * K + k0 + tq * 2);
				const uint32_t b1 = ld_pair(wt + (long long)ncol * K + k0 + 8 + tq * 2);
				mma_bf16(acc[t], a, b0, b1);
			}
		}
#pragma unroll
		for (int t = 0; t < 8; ++t) {
			if (nb + t * 8 >= N)
				break;
			const int c = nb + t * 8 + tq * 2;
			float v[4] = {acc[t][0] + bias[c], acc[t][1] + bias[c + 1], acc[t][2] + bias[c],
			              acc[t][3] + bias[c + 1]};
			if (kLogits) {
				float *o = static_cast<float *>(out);
				o[g * ldo + c] = v[0];
				o[g * ldo + c + 1] = v[1];
				o[(g + 8) * ldo + c] = v[2];
				o[(g + 8) * ldo + c + 1] = v[3];
			} else {
				__nv_bfloat16 *o = static_cast<__nv_bfloat16 *>(out);
				o[g * ldo + c] = __float2bfloat16_rn(fmaxf(v[0], 0.f));
				o[g * ldo + c + 1] = __float2bfloat16_rn(fmaxf(v[1], 0.f));
				o[(g + 8) * ldo + c] = __float2bfloat16_rn(fmaxf(v[2], 0.f));
				o[(g + 8) * ldo + c + 1] = __float2bfloat16_rn(fmaxf(v[3], 0.f));
			}
		}
	}
	__syncwarp();
}

struct InferArgs {
	const float *X;       // [rows][D] features (bf16-representable fp32)
	long long rows;
	const long long *rows_dev;
	int D, O, P, K;
	const __nv_bfloat16 *w1t, *w2t, *w3t;
	const float *b1, *b2, *b3;
	int16_t *topk;        // [rows][K] pair indices, best first
	float *logits;        // optional [rows][O]
};

constexpr int kInferWarps = 4;

// Shared memory per warp: act0 [16][D] and act1/act2 [16][128] bf16, logits
// [16][O] fp32.
__host__ __device__ inline size_t infer_warp_bytes(int D, int O)
{
	return size_t(16) * D * 2 + size_t(16) * kHidden * 2 * 2 + size_t(16) * O * 4;
}

__global__ void __launch_bounds__(kInferWarps * 32) mlp_infer_kernel(InferArgs a)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const long long rows = a.rows_dev ? *a.rows_dev : a.rows;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint8_t *wb = smem + warp * infer_warp_bytes(a.D, a.O);
	__nv_bfloat16 *act0 = reinterpret_cast<__nv_bfloat16 *>(wb);
	__nv_bfloat16 *act1 = act0 + 16 * a.D;
	__nv_bfloat16 *act2 = act1 + 16 * kHidden;
	float *lg = reinterpret_cast<float *>(act2 + 16 * kHidden);
	const long long tiles = (rows + 15) / 16;
	for (long long tile = (long long)blockIdx.x * kInferWarps + warp; tile < tiles;
	     tile += (long long)gridDim.x * kInferWarps) {
		const long long r0 = tile * 16;
		for (int i = lane; i < 16 * a.D; i += 32) {
			const long long r = r0 + i / a.D;
			act0[i] = __float2bfloat16_rn(r < rows ? a.X[r * a.D + i % a.D] : 0.f);
		}
		__syncwarp();
		mma_layer<false>(act0, a.D, a.D, a.w1t, a.b1, kHidden, act1, kHidden);
		mma_layer<false>(act1, kHidden, kHidden, a.w2t, a.b2, kHidden, act2, kHidden);
		mma_layer<true>(act2, kHidden, kHidden, a.w3t, a.b3, a.O, lg, a.O);
		for (int rr = 0; rr < 16; ++rr) {
			const long long r = r0 + rr;
			if (r >= rows)
				break;
			float *z = lg + rr * a.O;
			if (a.logits)
				for (int o = lane; o < a.O; o += 32)
					a.logits[r * a.O + o] = z[o];
			// top-K by repeated warp argmax (ties: lower pair index first)
			for (int k = 0; k < a.K; ++k) {
				float best = -INFINITY;
				int bi = 0x7fffffff;
				for (int o = lane; o < a.P; o += 32)
					if (z[o] > best || (z[o] == best && o < bi)) {
						best = z[o];
						bi = o;
					}
				for (int d = 16; d > 0; d >>= 1) {
					const float ob = __shfl_xor_sync(0xffffffffu, best, d);
					const int oi = __shfl_xor_sync(0xffffffffu, bi, d);
					if (ob > best || (ob == best && oi < bi)) {
						best = ob;
						bi = oi;
					}
				}
				if (lane == 0) {
					a.topk[r * a.K + k] = int16_t(bi < a.P ? bi : 0);
					z[bi < a.P ? bi : 0] = -INFINITY;
				}
				__syncwarp();
			}
		}
		__syncwarp();
	}
}

}  // namespace
}  // namespace wsbb

// ---------------------------------------------------------------- the model

struct wsbb_model {
	int n = 0, m = 0, P = 0, D = 0, O = 0;
	long long nparams = 0;
	float *w = nullptr;       // fp32 master weights: W1, b1, W2, b2, W3, b3
	float *grad = nullptr;
	float *adam_m = nullptr, *adam_v = nullptr;
	float *wr = nullptr;      // bf16-rounded copy used by the training forward
	__nv_bfloat16 *w1t = nullptr, *w2t = nullptr, *w3t = nullptr; // inference
	long long step = 0;
	// training scratch, grown on demand
	float *act = nullptr;
	long long act_rows = 0;
	float *d_loss = nullptr;
	cudaStream_t stream = nullptr;
	std::string last_error;
};

namespace {

struct Offsets {
	long long W1, b1, W2, b2, W3, b3, total;
};

Offsets offsets_of(int D, int O)
{
	const long long H = wsbb::kHidden;
	Offsets o;
	o.W1 = 0;
	o.b1 = o.W1 + D * H;
	o.W2 = o.b1 + H;
	o.b2 = o.W2 + H * H;
	o.W3 = o.b2 + H;
	o.b3 = o.W3 + H * O;
	o.total = o.b3 + O;
	return o;
}

int model_fail(wsbb_model *md, int code, const std::string &msg)
{
	if (md)
		md->last_error = msg;
	return code;
}

// Forward + backward on rows [0, B) of (X, y) already on the device;
// gradients into md->grad, loss sum into md->d_loss.
cudaError_t forward_backward(wsbb_model *md, const float *X, const int32_t *y, int B,
                             cudaStream_t s)
{
	using namespace wsbb;
	const int D = md->D, H = kHidden, O = md->O, P = md->P;
	const Offsets of = offsets_of(D, O);
	if (md->act_rows < B) {
		if (md->act)
			cudaFree(md->act);
		md->act = nullptr;
		cudaError_t e = cudaMalloc(&md->act, sizeof(float) * size_t(B) * (4 * H + 2 * O));
		if (e != cudaSuccess)
			return e;
		md->act_rows = B;
	}
	float *A1 = md->act, *A2 = A1 + (size_t)B * H, *Z3 = A2 + (size_t)B * H;
	float *dZ3 = Z3 + (size_t)B * O, *dA2 = dZ3 + (size_t)B * O, *dA1 = dA2 + (size_t)B * H;
	const float *W1 = md->wr + of.W1, *W2 = md->wr + of.W2, *W3 = md->wr + of.W3;
	float *G = md->grad;
	round_copy_kernel<<<256, 256, 0, s>>>(md->w, md->wr, md->nparams);
	// forward (operands bf16, fp32 accumulation)
	gemm(s, X, D, 1, W1, H, 1, A1, H, B, H, D, md->w + of.b1, 1, 1);
	gemm(s, A1, H, 1, W2, H, 1, A2, H, B, H, H, md->w + of.b2, 1, 1);
	gemm(s, A2, H, 1, W3, O, 1, Z3, O, B, O, H, md->w + of.b3, 0, 0);
	softmax_xent_kernel<<<(B * 32 + 255) / 256, 256, 0, s>>>(Z3, y, B, O, P, 1.f / B, dZ3,
	                                                          md->d_loss);
	// backward
	gemm(s, A2, 1, H, dZ3, O, 1, G + of.W3, O, H, O, B);          // dW3 = A2^T dZ3
	colsum_kernel<<<(O + 127) / 128, 128, 0, s>>>(dZ3, B, O, G + of.b3);
	gemm(s, dZ3, O, 1, W3, 1, O, dA2, H, B, H, O);                // dA2 = dZ3 W3^T
	relu_back_kernel<<<256, 256, 0, s>>>(dA2, A2, (long long)B * H);
	gemm(s, A1, 1, H, dA2, H, 1, G + of.W2, H, H, H, B);          // dW2 = A1^T dZ2
	colsum_kernel<<<(H + 127) / 128, 128, 0, s>>>(dA2, B, H, G + of.b2);
	gemm(s, dA2, H, 1, W2, 1, H, dA1, H, B, H, H);                // dA1 = dZ2 W2^T
	relu_back_kernel<<<256, 256, 0, s>>>(dA1, A1, (long long)B * H);
	gemm(s, X, 1, D, dA1, H, 1, G + of.W1, H, D, H, B);           // dW1 = X^T dZ1
	colsum_kernel<<<(H + 127) / 128, 128, 0, s>>>(dA1, B, H, G + of.b1);
	return cudaGetLastError();
}

uint64_t mix64(uint64_t z)
{
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

}  // namespace

extern "C" int wsbb_model_create(int n, int m, uint64_t seed, wsbb_model **out)
{
	if (!out || n < 2 || n > WSBB_MAX_JOBS || m < 2 || m > 20)
		return WSBB_ERR_ARG;
	*out = nullptr;
	wsbb_model *md = new wsbb_model();
	md->n = n;
	md->m = m;
	md->P = m * (m - 1) / 2;
	md->D = (3 * m + n + 15) / 16 * 16;
	md->O = (md->P + 7) / 8 * 8;
	const Offsets of = offsets_of(md->D, md->O);
	md->nparams = of.total;
	// He-style init from a seeded generator; biases zero
	std::vector<float> w(of.total, 0.f);
	uint64_t s = seed;
	auto uni = [&]() {
		s += 0x9E3779B97F4A7C15ULL;
		return double(mix64(s) >> 11) * (1.0 / 9007199254740992.0);
	};
	auto fill = [&](long long off, long long count, int fan_in) {
		const double a = std::sqrt(6.0 / fan_in);
		for (long long i = 0; i < count; ++i)
			w[off + i] = float((2 * uni() - 1) * a);
	};
	fill(of.W1, of.b1 - of.W1, md->D);
	fill(of.W2, of.b2 - of.W2, wsbb::kHidden);
	fill(of.W3, of.b3 - of.W3, wsbb::kHidden);
	const size_t bytes = sizeof(float) * size_t(of.total);
	cudaError_t e = cudaMalloc(&md->w, bytes);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->grad, bytes);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->adam_m, bytes);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->adam_v, bytes);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->wr, bytes);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->w1t, sizeof(__nv_bfloat16) * size_t(wsbb::kHidden) * md->D);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->w2t, sizeof(__nv_bfloat16) * size_t(wsbb::kHidden) * wsbb::kHidden);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->w3t, sizeof(__nv_bfloat16) * size_t(md->O) * wsbb::kHidden);
	if (e == cudaSuccess)
		e = cudaMalloc(&md->d_loss, sizeof(float));
	if (e == cudaSuccess)
		e = cudaStreamCreateWithFlags(&md->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess)
		e = cudaMemcpy(md->w, w.data(), bytes, cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMemset(md->adam_m, 0, bytes);
	if (e == cudaSuccess)
		e = cudaMemset(md->adam_v, 0, bytes);
	if (e != cudaSuccess) {
		wsbb_model_destroy(md);
		return WSBB_ERR_CUDA;
	}
	*out = md;
	return wsbb_model_pack(md);
}

extern "C" void wsbb_model_destroy(wsbb_model *md)
{
	if (!md)
		return;
	for (void *p : {(void *)md->w, (void *)md->grad, (void *)md->adam_m, (void *)md->adam_v,
	                (void *)md->wr, (void *)md->w1t, (void *)md->w2t, (void *)md->w3t,
	                (void *)md->act, (void *)md->d_loss})
		if (p)
			cudaFree(p);
	if (md->stream)
		cudaStreamDestroy(md->stream);
	delete md;
}

extern "C" const char *wsbb_model_last_error(const wsbb_model *md)
{
	return md ? md->last_error.c_str() : "null model";
}

extern "C" int wsbb_model_dims(const wsbb_model *md, int *D, int *O, int64_t *nparams)
{
	if (!md)
		return WSBB_ERR_ARG;
	if (D)
		*D = md->D;
	if (O)
		*O = md->O;
	if (nparams)
		*nparams = md->nparams;
	return WSBB_OK;
}

extern "C" int wsbb_model_pack(wsbb_model *md)
{
	if (!md)
		return WSBB_ERR_ARG;
	const long long H = wsbb::kHidden;
	const long long total = H * md->D + H * H + (long long)md->O * H;
	wsbb::pack_infer_kernel<<<int((total + 255) / 256), 256, 0, md->stream>>>(
	    md->w, md->D, md->O, md->w1t, md->w2t, md->w3t);
	cudaError_t e = cudaStreamSynchronize(md->stream);
	return e == cudaSuccess ? WSBB_OK : model_fail(md, WSBB_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int wsbb_model_get_weights(const wsbb_model *md, float *host, int64_t count)
{
	if (!md || !host || count != md->nparams)
		return WSBB_ERR_ARG;
	return cudaMemcpy(host, md->w, sizeof(float) * count, cudaMemcpyDeviceToHost) == cudaSuccess
	           ? WSBB_OK
	           : WSBB_ERR_CUDA;
}

extern "C" int wsbb_model_set_weights(wsbb_model *md, const float *host, int64_t count)
{
	if (!md || !host || count != md->nparams)
		return WSBB_ERR_ARG;
	if (cudaMemcpy(md->w, host, sizeof(float) * count, cudaMemcpyHostToDevice) != cudaSuccess)
		return WSBB_ERR_CUDA;
	return wsbb_model_pack(md);
}

extern "C" int wsbb_features(wsbb_ctx *ctx, const void *recs, int64_t count, float inv_scale,
                             int D, float *X, int32_t *labels, void *stream)
{
	if (!ctx || count < 0 || (count > 0 && (!recs || !X)))
		return WSBB_ERR_ARG;
	if (D < 3 * ctx->inst.m + ctx->inst.n)
		return wsbb_set_error(ctx, WSBB_ERR_ARG, "feature width below 3m + n");
	if (count == 0)
		return WSBB_OK;
	// no caller stream: the legacy default stream, ordered with the
	// caller's default-stream work on `recs`, `X` and `labels`
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	const int grid = int(std::min<int64_t>((count + 127) / 128, ctx->num_sms * 16));
	wsbb::features_kernel<<<grid, 128, 0, s>>>(ctx->bp, static_cast<const uint8_t *>(recs),
	                                           count, inv_scale, D, X, labels);
	cudaError_t e = cudaGetLastError();
	return e == cudaSuccess ? WSBB_OK : wsbb_set_error(ctx, WSBB_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" float wsbb_feature_scale(const wsbb_ctx *ctx)
{
	// 1 / largest machine load: node times land in about [0, 1]
	int64_t best = 1;
	const wsbb::Instance &I = ctx->inst;
	for (int k = 0; k < I.m; ++k) {
		int64_t s = 0;
		for (int j = 0; j < I.n; ++j)
			s += I.p[k * I.n + j];
		best = std::max(best, s);
	}
	return float(1.0 / double(best));
}

extern "C" int wsbb_model_grads(wsbb_model *md, const float *X, const int32_t *y, int B,
                                float *grad_host, float *loss_host)
{
	if (!md || !X || !y || B <= 0)
		return WSBB_ERR_ARG;
	cudaStream_t s = md->stream;
	cudaError_t e = wsbb::wait_for_legacy(s); // X, y may come from default-stream work
	if (e != cudaSuccess)
		return model_fail(md, WSBB_ERR_CUDA, cudaGetErrorString(e));
	cudaMemsetAsync(md->d_loss, 0, sizeof(float), s);
	e = forward_backward(md, X, y, B, s);
	if (e == cudaSuccess && grad_host)
		e = cudaMemcpyAsync(grad_host, md->grad, sizeof(float) * md->nparams,
		                    cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && loss_host)
		e = cudaMemcpyAsync(loss_host, md->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s);
	return e == cudaSuccess ? WSBB_OK : model_fail(md, WSBB_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int wsbb_model_train(wsbb_model *md, const float *X, const int32_t *y, int64_t count,
                                int epochs, int batch, float lr, uint64_t seed,
                                float *epoch_loss_host)
{
	if (!md || !X || !y || count < batch || batch <= 0 || epochs <= 0)
		return WSBB_ERR_ARG;
	cudaStream_t s = md->stream;
	const int D = md->D;
	float *xb = nullptr;
	int32_t *yb = nullptr;
	long long *idx = nullptr;
	cudaError_t e = wsbb::wait_for_legacy(s); // X, y may come from default-stream work
	if (e == cudaSuccess)
		e = cudaMalloc(&xb, sizeof(float) * size_t(batch) * D);
	if (e == cudaSuccess)
		e = cudaMalloc(&yb, sizeof(int32_t) * batch);
	if (e == cudaSuccess)
		e = cudaMalloc(&idx, sizeof(long long) * batch);
	std::vector<long long> order(count), hidx(batch);
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
		for (long long i = 0; i < count; ++i)
			order[i] = i;
		uint64_t r = seed + 0x1000193ULL * (ep + 1);
		for (long long i = count - 1; i > 0; --i) {
			r += 0x9E3779B97F4A7C15ULL;
			std::swap(order[i], order[mix64(r) % uint64_t(i + 1)]);
		}
		cudaMemsetAsync(md->d_loss, 0, sizeof(float), s);
		const long long nb = count / batch;
		for (long long b = 0; b < nb && e == cudaSuccess; ++b) {
			std::copy(order.begin() + b * batch, order.begin() + (b + 1) * batch, hidx.begin());
			e = cudaMemcpyAsync(idx, hidx.data(), sizeof(long long) * batch,
			                    cudaMemcpyHostToDevice, s);
			if (e != cudaSuccess)
				break;
			wsbb::gather_rows_kernel<<<batch, 128, 0, s>>>(X, y, idx, batch, D, xb, yb);
			e = forward_backward(md, xb, yb, batch, s);
			md->step++;
			const float c1 = 1.f / (1.f - std::pow(b1, float(md->step)));
			const float c2 = 1.f / (1.f - std::pow(b2, float(md->step)));
			wsbb::adam_kernel<<<512, 256, 0, s>>>(md->w, md->grad, md->adam_m, md->adam_v,
			                                      md->nparams, lr, b1, b2, eps, c1, c2);
			// keep the pageable index buffer alive until the copy is done
			if (e == cudaSuccess)
				e = cudaStreamSynchronize(s);
		}
		float lsum = 0;
		if (e == cudaSuccess)
			e = cudaMemcpy(&lsum, md->d_loss, sizeof(float), cudaMemcpyDeviceToHost);
		if (epoch_loss_host)
			epoch_loss_host[ep] = lsum / float(nb * batch);
	}
	cudaFree(xb);
	cudaFree(yb);
	cudaFree(idx);
	if (e != cudaSuccess)
		return model_fail(md, WSBB_ERR_CUDA, cudaGetErrorString(e));
	return wsbb_model_pack(md);
}

namespace wsbb {
cudaError_t launch_mlp_topk(const wsbb_model *md, const float *X, long long rows,
                            const long long *rows_dev, int K, int16_t *topk, float *logits,
                            int num_sms, cudaStream_t s)
{
	InferArgs a;
	a.X = X;
	a.rows = rows;
	a.rows_dev = rows_dev;
	a.D = md->D;
	a.O = md->O;
	a.P = md->P;
	a.K = K;
	a.w1t = md->w1t;
	a.w2t = md->w2t;
	a.w3t = md->w3t;
	const Offsets of = offsets_of(md->D, md->O);
	a.b1 = md->w + of.b1;
	a.b2 = md->w + of.b2;
	a.b3 = md->w + of.b3;
	a.topk = topk;
	a.logits = logits;
	const size_t smem = size_t(kInferWarps) * infer_warp_bytes(md->D, md->O);
	cudaError_t e = allow_max_dynamic_smem(mlp_infer_kernel);
	if (e != cudaSuccess)
		return e;
	const long long tiles = (rows + 15) / 16;
	const int grid = int(std::max<long long>(
	    1, std::min<long long>((tiles + kInferWarps - 1) / kInferWarps, num_sms * 4)));
	mlp_infer_kernel<<<grid, kInferWarps * 32, smem, s>>>(a);
	return cudaGetLastError();
}
}  // namespace wsbb

extern "C" int wsbb_model_topk(wsbb_model *md, const float *X, int64_t rows, int K,
                               int16_t *topk, float *logits, void *stream)
{
	if (!md || rows < 0 || K < 1 || K > md->P || (rows > 0 && (!X || !topk)))
		return WSBB_ERR_ARG;
	if (rows == 0)
		return WSBB_OK;
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	cudaStream_t s = static_cast<cudaStream_t>(stream); // NULL: the legacy default stream
	cudaError_t e = wsbb::launch_mlp_topk(md, X, rows, nullptr, K, topk, logits, sms, s);
	return e == cudaSuccess ? WSBB_OK : model_fail(md, WSBB_ERR_CUDA, cudaGetErrorString(e));
}
