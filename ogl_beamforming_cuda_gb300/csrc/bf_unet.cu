/*
 * bf_unet.cu -- kernels of the learned variant (include/bf_unet.h): 3 x 3 x 3
 * convolutions (forward, gradient of the input, gradient of the weights), 2 x
 * pooling and upsampling, the ReLU derivative, the MSE loss, Adam, and the
 * seeded RF synthesis that makes the training data.
 *
 * Convolution forward of BF16 inputs: bf_unet_tc.cu (tcgen05 implicit GEMM).
 * Convolution forward of FP32 inputs (the input gradient; OGL_BF_UNET_SIMT=1 for
 * every input) here (direct, channels-first): a block computes an 8 x 8 x 32
 * output tile for 8 output channels. Per input channel it stages the tile with
 * its one-voxel halo (10 x 10 x 34 values, FP32) and the 27 x 8 taps in shared
 * memory; each thread owns one (y, x) column of 8 depths, loads the 10 input
 * values of a (ky, kx) column once and applies them to 3 kz x 8 depths x 8
 * output channels (192 FMAs per 16 shared loads), accumulating in FP32.
 * The input gradient is the same kernel on the output gradient with the taps
 * flipped and the channel roles swapped. The weight gradient reduces, per
 * (output, input) channel pair, the products over a 4 x 8 x 32 voxel tile held
 * in shared memory: a thread walks runs of 8 x-consecutive voxels, reusing each
 * loaded input row for the three kx taps, and the block's partial sums are added
 * to the FP32 gradient with one atomic per tap.
 */
#include "bf_kernels.h"
#include "bf_unet.h"

#include <cuda_bf16.h>

#include <algorithm>

namespace bf {
namespace {

__device__ __forceinline__ float ld(const float *p, size_t i) { return __ldg(p + i); }
__device__ __forceinline__ float ld(const __nv_bfloat16 *p, size_t i) { return __bfloat162float(p[i]); }
__device__ __forceinline__ void st(float *p, size_t i, float v) { p[i] = v; }
__device__ __forceinline__ void st(__nv_bfloat16 *p, size_t i, float v) { p[i] = __float2bfloat16_rn(v); }

constexpr int CZ = 8, CY = 8, CX = 32, COB = 8;
constexpr int HZ = CZ + 2, HY = CY + 2, HX = CX + 2;

template <typename TI, typename TO>
__global__ void __launch_bounds__(256)
conv3d_fwd(const TI *__restrict__ in, int cin, const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias,
           const TO *__restrict__ residual, TO *__restrict__ out, int cout, int W, int H, int D, int relu)
{
	__shared__ float s_in[HZ * HY * HX];
	__shared__ __align__(16) float s_w[27 * COB];
	const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
	const int tiles_x = (W + CX - 1) / CX, tiles_y = (H + CY - 1) / CY;
	int b = blockIdx.x;
	const int bx = b % tiles_x;
	b /= tiles_x;
	const int by = b % tiles_y, bz = b / tiles_y;
	const int x0 = bx * CX, y0 = by * CY, z0 = bz * CZ, co0 = blockIdx.y * COB;
	const size_t plane = (size_t)H * W, vol = plane * D;

	float acc[CZ][COB];
	#pragma unroll
	for (int z = 0; z < CZ; z++)
		#pragma unroll
		for (int c = 0; c < COB; c++) acc[z][c] = 0.0f;

	for (int ci = 0; ci < cin; ci++) {
		__syncthreads();
		for (int i = threadIdx.x; i < HZ * HY * HX; i += blockDim.x) {
			const int lx = i % HX, r = i / HX, ly = r % HY, lz = r / HY;
			const int gx = x0 + lx - 1, gy = y0 + ly - 1, gz = z0 + lz - 1;
			float v = 0.0f;
			if (gx >= 0 && gx < W && gy >= 0 && gy < H && gz >= 0 && gz < D)
				v = ld(in, (size_t)ci * vol + (size_t)gz * plane + (size_t)gy * W + gx);
			s_in[i] = v;
		}
		if (threadIdx.x < 27 * COB) {
			const int k = threadIdx.x / COB, c = threadIdx.x % COB;
			s_w[threadIdx.x] = co0 + c < cout ? __bfloat162float(w[((size_t)(co0 + c) * cin + ci) * 27 + k]) : 0.0f;
		}
		__syncthreads();
		#pragma unroll
		for (int ky = 0; ky < 3; ky++)
			#pragma unroll
			for (int kx = 0; kx < 3; kx++) {
				float col[HZ];
				#pragma unroll
				for (int z = 0; z < HZ; z++) col[z] = s_in[(z * HY + ty + ky) * HX + tx + kx];
				#pragma unroll
				for (int kz = 0; kz < 3; kz++) {
					const float4 wa = *(const float4 *)&s_w[((kz * 3 + ky) * 3 + kx) * COB];
					const float4 wb = *(const float4 *)&s_w[((kz * 3 + ky) * 3 + kx) * COB + 4];
					#pragma unroll
					for (int z = 0; z < CZ; z++) {
						const float v = col[z + kz];
						acc[z][0] = fmaf(v, wa.x, acc[z][0]);
						acc[z][1] = fmaf(v, wa.y, acc[z][1]);
						acc[z][2] = fmaf(v, wa.z, acc[z][2]);
						acc[z][3] = fmaf(v, wa.w, acc[z][3]);
						acc[z][4] = fmaf(v, wb.x, acc[z][4]);
						acc[z][5] = fmaf(v, wb.y, acc[z][5]);
						acc[z][6] = fmaf(v, wb.z, acc[z][6]);
						acc[z][7] = fmaf(v, wb.w, acc[z][7]);
					}
				}
			}
	}
	const int gx = x0 + tx, gy = y0 + ty;
	if (gx >= W || gy >= H) return;
	#pragma unroll
	for (int c = 0; c < COB; c++) {
		const int co = co0 + c;
		if (co >= cout) break;
		const float bb = bias ? bias[co] : 0.0f;
		#pragma unroll
		for (int z = 0; z < CZ; z++) {
			const int gz = z0 + z;
			if (gz >= D) break;
			const size_t o = (size_t)co * vol + (size_t)gz * plane + (size_t)gy * W + gx;
			float v = acc[z][c] + bb;
			if (relu) v = fmaxf(v, 0.0f);
			if (residual) v += ld(residual, o);
			st(out, o, v);
		}
	}
}

/* wt[ci][co][k] = w[co][ci][26 - k] */
__global__ void flip_weights(const __nv_bfloat16 *__restrict__ w, __nv_bfloat16 *__restrict__ wt, int cout, int cin)
{
	const int n = cout * cin * 27;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const int k = i % 27, r = i / 27, co = r % cout, ci = r / cout;
		wt[i] = w[((size_t)co * cin + ci) * 27 + (26 - k)];
	}
}

constexpr int GZ = 4, GY = 8, GX = 32, GCO = 8, GCI = 8;
constexpr int GHZ = GZ + 2, GHY = GY + 2, GHX = GX + 2;
constexpr int G_STRIDE = GZ * GY * GX + 1;           /* padded: channels on distinct banks */
constexpr int X_STRIDE = GHZ * GHY * GHX + 1;

template <typename TI>
__global__ void __launch_bounds__(256)
conv3d_wgrad(const float *__restrict__ g, int cout, const TI *__restrict__ in, int cin, int W, int H, int D,
             float *__restrict__ gw, float *__restrict__ gb)
{
	extern __shared__ float sm[];
	float *s_g = sm;                                 /* GCO x G_STRIDE */
	float *s_x = sm + GCO * G_STRIDE;                /* GCI x X_STRIDE */
	float *s_r = sm;                                 /* reduction, 256 x 28, after the tiles are used */
	const int tiles_x = (W + GX - 1) / GX, tiles_y = (H + GY - 1) / GY;
	int b = blockIdx.x;
	const int bx = b % tiles_x;
	b /= tiles_x;
	const int by = b % tiles_y, bz = b / tiles_y;
	const int x0 = bx * GX, y0 = by * GY, z0 = bz * GZ;
	const int co0 = blockIdx.y * GCO, ci0 = blockIdx.z * GCI;
	const size_t plane = (size_t)H * W, vol = plane * D;

	for (int i = threadIdx.x; i < GCO * GZ * GY * GX; i += blockDim.x) {
		const int lx = i % GX, r = i / GX, ly = r % GY, r2 = r / GY, lz = r2 % GZ, c = r2 / GZ;
		const int gx = x0 + lx, gy = y0 + ly, gz = z0 + lz, co = co0 + c;
		float v = 0.0f;
		if (co < cout && gx < W && gy < H && gz < D) v = __ldg(g + (size_t)co * vol + (size_t)gz * plane + (size_t)gy * W + gx);
		s_g[c * G_STRIDE + (lz * GY + ly) * GX + lx] = v;
	}
	for (int i = threadIdx.x; i < GCI * GHZ * GHY * GHX; i += blockDim.x) {
		const int lx = i % GHX, r = i / GHX, ly = r % GHY, r2 = r / GHY, lz = r2 % GHZ, c = r2 / GHZ;
		const int gx = x0 + lx - 1, gy = y0 + ly - 1, gz = z0 + lz - 1, ci = ci0 + c;
		float v = 0.0f;
		if (ci < cin && gx >= 0 && gx < W && gy >= 0 && gy < H && gz >= 0 && gz < D)
			v = ld(in, (size_t)ci * vol + (size_t)gz * plane + (size_t)gy * W + gx);
		s_x[c * X_STRIDE + (lz * GHY + ly) * GHX + lx] = v;
	}
	__syncthreads();

	const int pair = threadIdx.x & 63, part = threadIdx.x >> 6;
	const int col = pair >> 3, cil = pair & 7;      /* output / input channel of the pair */
	float acc[27];
	#pragma unroll
	for (int k = 0; k < 27; k++) acc[k] = 0.0f;
	float bsum = 0.0f;
	/* runs of 8 consecutive x: GZ * GY * (GX / 8) = 128 runs, 32 per part */
	for (int run = part; run < GZ * GY * (GX / 8); run += 4) {
		const int rx = (run % (GX / 8)) * 8, r = run / (GX / 8), ly = r % GY, lz = r / GY;
		float gv[8];
		#pragma unroll
		for (int i = 0; i < 8; i++) gv[i] = s_g[col * G_STRIDE + (lz * GY + ly) * GX + rx + i];
		#pragma unroll
		for (int i = 0; i < 8; i++) bsum += gv[i];
		#pragma unroll
		for (int kz = 0; kz < 3; kz++)
			#pragma unroll
			for (int ky = 0; ky < 3; ky++) {
				float xr[10];
				#pragma unroll
				for (int i = 0; i < 10; i++) xr[i] = s_x[cil * X_STRIDE + ((lz + kz) * GHY + ly + ky) * GHX + rx + i];
				#pragma unroll
				for (int kx = 0; kx < 3; kx++) {
					float a = acc[(kz * 3 + ky) * 3 + kx];
					#pragma unroll
					for (int i = 0; i < 8; i++) a = fmaf(gv[i], xr[i + kx], a);
					acc[(kz * 3 + ky) * 3 + kx] = a;
				}
			}
	}
	__syncthreads();
	#pragma unroll
	for (int k = 0; k < 27; k++) s_r[threadIdx.x * 28 + k] = acc[k];
	s_r[threadIdx.x * 28 + 27] = bsum;
	__syncthreads();
	/* the 4 parts of each pair summed in part order, one atomic per tap */
	for (int i = threadIdx.x; i < 64 * 28; i += blockDim.x) {
		const int pr = i / 28, k = i % 28;
		const float s = s_r[pr * 28 + k] + s_r[(64 + pr) * 28 + k] + s_r[(128 + pr) * 28 + k] + s_r[(192 + pr) * 28 + k];
		const int co = co0 + (pr >> 3), ci = ci0 + (pr & 7);
		if (co >= cout || ci >= cin) continue;
		if (k < 27) atomicAdd(gw + ((size_t)co * cin + ci) * 27 + k, s);
		else if (gb && (pr & 7) == 0 && ci0 == 0) atomicAdd(gb + co, s);
	}
}

__global__ void relu_grad_k(float *__restrict__ g, const __nv_bfloat16 *__restrict__ a, int64_t n)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		if (!(__bfloat162float(a[i]) > 0.0f)) g[i] = 0.0f;
}

/* The pooling and upsampling kernels walk rows: block b takes rows b, b + grid,
 * ... of its output (row = (channel * depth + z) * height + y), a row's threads
 * its x positions, so the index arithmetic runs once per row. */
template <typename TI, typename TO>
__global__ void avgpool2_k(const TI *__restrict__ in, TO *__restrict__ out, int c, int W, int H, int D)
{
	const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
	const int64_t rows = (int64_t)c * d2 * h2;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const int y = (int)(row % h2);
		const int64_t cz = row / h2;
		const int z = (int)(cz % d2);
		const int64_t ch = cz / d2;
		const size_t base = (((size_t)ch * D + 2 * z) * H + 2 * y) * W;
		const size_t plane = (size_t)H * W;
		for (int x = threadIdx.x; x < w2; x += blockDim.x) {
			float s = 0.0f;
			#pragma unroll
			for (int dz = 0; dz < 2; dz++)
				#pragma unroll
				for (int dy = 0; dy < 2; dy++)
					#pragma unroll
					for (int dx = 0; dx < 2; dx++)
						s += ld(in, base + dz * plane + (size_t)dy * W + 2 * x + dx);
			st(out, row * w2 + x, 0.125f * s);
		}
	}
}

__global__ void avgpool2_grad_k(const float *__restrict__ go, float *__restrict__ gi, int c, int W, int H, int D,
                                int accumulate)
{
	const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
	const int64_t rows = (int64_t)c * D * H;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const int y = (int)(row % H);
		const int64_t cz = row / H;
		const int z = (int)(cz % D);
		const int64_t ch = cz / D;
		const float *src = go + (((size_t)ch * d2 + z / 2) * h2 + y / 2) * w2;
		float *dst = gi + row * W;
		for (int x = threadIdx.x; x < W; x += blockDim.x) {
			const float v = 0.125f * src[x / 2];
			dst[x] = accumulate ? dst[x] + v : v;
		}
	}
}

template <typename TI, typename TO>
__global__ void upsample2_k(const TI *__restrict__ in, TO *__restrict__ out, int c, int W, int H, int D)
{
	const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
	const int64_t rows = (int64_t)c * D * H;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const int y = (int)(row % H);
		const int64_t cz = row / H;
		const int z = (int)(cz % D);
		const int64_t ch = cz / D;
		const size_t src = (((size_t)ch * d2 + z / 2) * h2 + y / 2) * w2;
		const size_t dst = (size_t)row * W;
		for (int x = threadIdx.x; x < W; x += blockDim.x) st(out, dst + x, ld(in, src + x / 2));
	}
}

__global__ void upsample2_grad_k(const float *__restrict__ go, float *__restrict__ gi, int c, int W, int H, int D)
{
	const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
	const int64_t rows = (int64_t)c * d2 * h2;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const int y = (int)(row % h2);
		const int64_t cz = row / h2;
		const int z = (int)(cz % d2);
		const int64_t ch = cz / d2;
		const size_t base = (((size_t)ch * D + 2 * z) * H + 2 * y) * W;
		const size_t plane = (size_t)H * W;
		for (int x = threadIdx.x; x < w2; x += blockDim.x) {
			float s = 0.0f;
			#pragma unroll
			for (int dz = 0; dz < 2; dz++)
				#pragma unroll
				for (int dy = 0; dy < 2; dy++)
					#pragma unroll
					for (int dx = 0; dx < 2; dx++)
						s += go[base + dz * plane + (size_t)dy * W + 2 * x + dx];
			gi[row * w2 + x] = s;
		}
	}
}

__global__ void mse_k(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ g,
                      float *__restrict__ loss, int64_t n)
{
	float s = 0.0f;
	const float inv = 1.0f / (float)n;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float d = y[i] - t[i];
		g[i] = 2.0f * d * inv;
		s = fmaf(d * d, inv, s);
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
	if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

__global__ void adam_k(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ w16, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.0f - b1) * gi;
		const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		w[i] = wi;
		w16[i] = __float2bfloat16_rn(wi);
	}
}

__global__ void ema_k(float *__restrict__ e, const float *__restrict__ w, __nv_bfloat16 *__restrict__ e16, int64_t n,
                      float decay)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float ei = decay * e[i] + (1.0f - decay) * w[i];
		e[i] = ei;
		if (e16) e16[i] = __float2bfloat16_rn(ei);
	}
}

template <typename TI, typename TO>
__global__ void convert_k(const TI *__restrict__ x, TO *__restrict__ y, int64_t n, float scale)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		st(y, i, scale * ld(x, i));
}

/* one block per (transmit, receive) trace, accumulated in shared memory */
__global__ void __launch_bounds__(256)
synth_k(const float *__restrict__ pos, const float *__restrict__ amp, int n_scat, float *__restrict__ x, int S, int C,
        int T, float px, float py, float fs, float fc, float c)
{
	extern __shared__ float trace[];
	const int r = blockIdx.x % C, t = blockIdx.x / C;
	for (int i = threadIdx.x; i < S; i += blockDim.x) trace[i] = 0.0f;
	__syncthreads();
	const float ex = r * px, ey = t * py;
	const float sigma = 1.0f / fc / 2.5f;
	const int half = (int)ceilf(3.0f * sigma * fs) + 1;
	const float w0 = 6.283185307f * fc, inv_s2 = 1.0f / (sigma * sigma);
	for (int s = threadIdx.x; s < n_scat; s += blockDim.x) {
		const float qx = pos[3 * s], qy = pos[3 * s + 1], qz = pos[3 * s + 2], a = amp[s];
		const float dx = qx - ex, dy = qy - ey;
		const float tau = (qz + sqrtf(dx * dx + dy * dy + qz * qz)) / c;
		const int n0 = (int)floorf(tau * fs);
		for (int k = -half; k <= half; k++) {
			const int n = n0 + k;
			if (n < 0 || n >= S) continue;
			const float tt = (float)n / fs - tau;
			atomicAdd(&trace[n], a * __cosf(w0 * tt) * __expf(-tt * tt * inv_s2));
		}
	}
	__syncthreads();
	float *dst = x + ((size_t)t * C + r) * S;
	for (int i = threadIdx.x; i < S; i += blockDim.x) dst[i] = trace[i];
}

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sm_count() * 32); }
/* blocks for a row walk over `rows` rows */
int grid_rows(int64_t rows) { return (int)std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t)device_sm_count() * 64)); }

} /* namespace */
} /* namespace bf */

namespace bf {
/* bf_unet_tc.cu: the tensor-core form of the forward convolution for BF16 inputs */
bool conv3d_tc_launch(const void *in, int in_type, int cin, const uint16_t *w, const float *bias, const void *residual, void *out,
                      int out_type, int cout, const int32_t dims[3], int relu, cudaStream_t s, cudaError_t &err);
}

using namespace bf;

#define BF_OK(e) ((e) == cudaSuccess ? 1u : 0u)

extern "C" {

uint32_t bf_unet_conv3d(const void *in, int32_t in_type, int32_t cin, const uint16_t *w, const float *bias,
                        const void *residual, void *out, int32_t out_type, int32_t cout, const int32_t dims[3],
                        int32_t relu, void *stream)
{
	if (!in || !w || !out || cin <= 0 || cout <= 0 || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	if (in_type == BF_UNET_BF16) {
		cudaError_t e = cudaSuccess;
		if (conv3d_tc_launch(in, BF_UNET_BF16, cin, w, bias, residual, out, out_type, cout, dims, relu, s, e))
			return BF_OK(e);
	}
	const int W = dims[0], H = dims[1], D = dims[2];
	dim3 grid(((W + CX - 1) / CX) * ((H + CY - 1) / CY) * ((D + CZ - 1) / CZ), (cout + COB - 1) / COB);
	const __nv_bfloat16 *wb = (const __nv_bfloat16 *)w;
	if (in_type == BF_UNET_BF16 && out_type == BF_UNET_BF16)
		conv3d_fwd<__nv_bfloat16, __nv_bfloat16><<<grid, 256, 0, s>>>((const __nv_bfloat16 *)in, cin, wb, bias,
		    (const __nv_bfloat16 *)residual, (__nv_bfloat16 *)out, cout, W, H, D, relu);
	else if (in_type == BF_UNET_BF16 && out_type == BF_UNET_F32)
		conv3d_fwd<__nv_bfloat16, float><<<grid, 256, 0, s>>>((const __nv_bfloat16 *)in, cin, wb, bias,
		    (const float *)residual, (float *)out, cout, W, H, D, relu);
	else if (in_type == BF_UNET_F32 && out_type == BF_UNET_F32)
		conv3d_fwd<float, float><<<grid, 256, 0, s>>>((const float *)in, cin, wb, bias, (const float *)residual,
		    (float *)out, cout, W, H, D, relu);
	else
		conv3d_fwd<float, __nv_bfloat16><<<grid, 256, 0, s>>>((const float *)in, cin, wb, bias,
		    (const __nv_bfloat16 *)residual, (__nv_bfloat16 *)out, cout, W, H, D, relu);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_conv3d_grad_input(const float *grad_out, int32_t cout, const uint16_t *w, float *grad_in, int32_t cin,
                                   const int32_t dims[3], uint16_t *w_scratch, void *stream)
{
	if (!grad_out || !w || !grad_in || !w_scratch || cin <= 0 || cout <= 0) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	flip_weights<<<grid_for((int64_t)cout * cin * 27), 256, 0, s>>>((const __nv_bfloat16 *)w, (__nv_bfloat16 *)w_scratch,
	                                                               cout, cin);
	g_kernel_launches++;
	if (cudaGetLastError() != cudaSuccess) return 0;
	if (dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0) {
		cudaError_t e = cudaSuccess;
		if (conv3d_tc_launch(grad_out, BF_UNET_F32, cout, w_scratch, nullptr, nullptr, grad_in, BF_UNET_F32, cin, dims, 0,
		                     s, e))
			return BF_OK(e);
	}
	return bf_unet_conv3d(grad_out, BF_UNET_F32, cout, w_scratch, nullptr, nullptr, grad_in, BF_UNET_F32, cin, dims, 0,
	                      stream);
}

uint32_t bf_unet_conv3d_grad_weight(const float *grad_out, int32_t cout, const void *in, int32_t in_type, int32_t cin,
                                    const int32_t dims[3], float *grad_w, float *grad_b, void *stream)
{
	if (!grad_out || !in || !grad_w || cin <= 0 || cout <= 0 || !dims) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	const int W = dims[0], H = dims[1], D = dims[2];
	dim3 grid(((W + GX - 1) / GX) * ((H + GY - 1) / GY) * ((D + GZ - 1) / GZ), (cout + GCO - 1) / GCO,
	          (cin + GCI - 1) / GCI);
	const size_t smem = sizeof(float) * ((size_t)GCO * G_STRIDE + (size_t)GCI * X_STRIDE);
	static bool attr = false;
	if (!attr) {
		cudaFuncSetAttribute(conv3d_wgrad<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
		cudaFuncSetAttribute(conv3d_wgrad<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
		attr = true;
	}
	if (in_type == BF_UNET_BF16)
		conv3d_wgrad<__nv_bfloat16><<<grid, 256, smem, s>>>(grad_out, cout, (const __nv_bfloat16 *)in, cin, W, H, D,
		                                                    grad_w, grad_b);
	else
		conv3d_wgrad<float><<<grid, 256, smem, s>>>(grad_out, cout, (const float *)in, cin, W, H, D, grad_w, grad_b);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_relu_grad(float *grad, const uint16_t *act, int64_t n, void *stream)
{
	if (!grad || !act || n < 0) return 0;
	relu_grad_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(grad, (const __nv_bfloat16 *)act, n);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_avgpool2(const void *in, int32_t in_type, void *out, int32_t out_type, int32_t c,
                          const int32_t dims_in[3], void *stream)
{
	if (!in || !out || c <= 0 || !dims_in || dims_in[0] % 2 || dims_in[1] % 2 || dims_in[2] % 2) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	const int W = dims_in[0], H = dims_in[1], D = dims_in[2];
	const int g = grid_rows((int64_t)c * (D / 2) * (H / 2)), t = std::min(128, std::max(32, W / 2));
	if (in_type == BF_UNET_BF16 && out_type == BF_UNET_BF16)
		avgpool2_k<<<g, t, 0, s>>>((const __nv_bfloat16 *)in, (__nv_bfloat16 *)out, c, W, H, D);
	else if (in_type == BF_UNET_F32 && out_type == BF_UNET_F32)
		avgpool2_k<<<g, t, 0, s>>>((const float *)in, (float *)out, c, W, H, D);
	else if (in_type == BF_UNET_BF16)
		avgpool2_k<<<g, t, 0, s>>>((const __nv_bfloat16 *)in, (float *)out, c, W, H, D);
	else
		avgpool2_k<<<g, t, 0, s>>>((const float *)in, (__nv_bfloat16 *)out, c, W, H, D);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_avgpool2_grad(const float *grad_out, float *grad_in, int32_t c, const int32_t dims_in[3],
                               int32_t accumulate, void *stream)
{
	if (!grad_out || !grad_in || c <= 0 || !dims_in) return 0;
	const int g = grid_rows((int64_t)c * dims_in[2] * dims_in[1]), t = std::min(128, std::max(32, dims_in[0]));
	avgpool2_grad_k<<<g, t, 0, (cudaStream_t)stream>>>(grad_out, grad_in, c, dims_in[0], dims_in[1],
	                                                               dims_in[2], accumulate);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_upsample2(const void *in, int32_t in_type, void *out, int32_t out_type, int32_t c,
                           const int32_t dims_out[3], void *stream)
{
	if (!in || !out || c <= 0 || !dims_out || dims_out[0] % 2 || dims_out[1] % 2 || dims_out[2] % 2) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	const int W = dims_out[0], H = dims_out[1], D = dims_out[2];
	const int g = grid_rows((int64_t)c * D * H), t = std::min(128, std::max(32, W));
	if (in_type == BF_UNET_BF16 && out_type == BF_UNET_BF16)
		upsample2_k<<<g, t, 0, s>>>((const __nv_bfloat16 *)in, (__nv_bfloat16 *)out, c, W, H, D);
	else if (in_type == BF_UNET_F32 && out_type == BF_UNET_F32)
		upsample2_k<<<g, t, 0, s>>>((const float *)in, (float *)out, c, W, H, D);
	else if (in_type == BF_UNET_BF16)
		upsample2_k<<<g, t, 0, s>>>((const __nv_bfloat16 *)in, (float *)out, c, W, H, D);
	else
		upsample2_k<<<g, t, 0, s>>>((const float *)in, (__nv_bfloat16 *)out, c, W, H, D);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_upsample2_grad(const float *grad_out, float *grad_in, int32_t c, const int32_t dims_out[3], void *stream)
{
	if (!grad_out || !grad_in || c <= 0 || !dims_out) return 0;
	const int g = grid_rows((int64_t)c * (dims_out[2] / 2) * (dims_out[1] / 2));
	const int t = std::min(128, std::max(32, dims_out[0] / 2));
	upsample2_grad_k<<<g, t, 0, (cudaStream_t)stream>>>(grad_out, grad_in, c, dims_out[0], dims_out[1],
	                                                                dims_out[2]);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_mse(const float *y, const float *t, float *grad, float *loss, int64_t n, void *stream)
{
	if (!y || !t || !grad || !loss || n <= 0) return 0;
	mse_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(y, t, grad, loss, n);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_adam(float *w, const float *grad, float *m, float *v, uint16_t *w16, int64_t n, float lr,
                      float beta1, float beta2, float eps, int32_t step, void *stream)
{
	if (!w || !grad || !m || !v || !w16 || n <= 0 || step < 1) return 0;
	const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
	adam_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, grad, m, v, (__nv_bfloat16 *)w16, n, lr, beta1, beta2, eps,
	                                                     c1, c2);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_ema(float *ema, const float *w, uint16_t *ema16, int64_t n, float decay, void *stream)
{
	if (!ema || !w || n <= 0 || !(decay >= 0.0f && decay <= 1.0f)) return 0;
	ema_k<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(ema, w, (__nv_bfloat16 *)ema16, n, decay);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_unet_convert(const void *x, int32_t x_type, void *y, int32_t y_type, int64_t n, float scale, void *stream)
{
	if (!x || !y || n < 0) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	if (x_type == BF_UNET_F32 && y_type == BF_UNET_BF16)
		convert_k<<<grid_for(n), 256, 0, s>>>((const float *)x, (__nv_bfloat16 *)y, n, scale);
	else if (x_type == BF_UNET_BF16 && y_type == BF_UNET_F32)
		convert_k<<<grid_for(n), 256, 0, s>>>((const __nv_bfloat16 *)x, (float *)y, n, scale);
	else if (x_type == BF_UNET_F32)
		convert_k<<<grid_for(n), 256, 0, s>>>((const float *)x, (float *)y, n, scale);
	else
		convert_k<<<grid_for(n), 256, 0, s>>>((const __nv_bfloat16 *)x, (__nv_bfloat16 *)y, n, scale);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

uint32_t bf_synth_traces(const float *pos, const float *amp, int32_t n_scat, float *x, int32_t samples,
                         int32_t channels, int32_t transmits, float pitch_x, float pitch_y, float fs, float fc,
                         float c, void *stream)
{
	if (!pos || !amp || !x || n_scat < 0 || samples <= 0 || channels <= 0 || transmits <= 0) return 0;
	if ((size_t)samples * sizeof(float) > 200 * 1024) return 0;
	static bool attr = false;
	if (!attr) {
		cudaFuncSetAttribute(synth_k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
		attr = true;
	}
	synth_k<<<channels * transmits, 256, (size_t)samples * sizeof(float), (cudaStream_t)stream>>>(
	    pos, amp, n_scat, x, samples, channels, transmits, pitch_x, pitch_y, fs, fc, c);
	g_kernel_launches++;
	return BF_OK(cudaGetLastError());
}

} /* extern "C" */
