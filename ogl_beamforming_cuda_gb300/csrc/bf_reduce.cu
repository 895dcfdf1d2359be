/*
 * bf_reduce.cu -- frame averaging and the min/max pyramid.
 *
 * Sum (reference: shaders/sum.glsl:7-12, do_sum_shader beamformer.c:218-235):
 * the reference clears the output and runs one dispatch per input frame,
 * reading and rewriting the whole output each time (n+1 reads and n writes of
 * the volume). Here one streaming pass reads each input once and writes the
 * output once: out = ((0 + k*in_0) + k*in_1) + ... evaluated with explicit
 * round-to-nearest so the result is bit-equal to the reference's sequence. The
 * reference's dispatch covers x < 32*max(1, X/32), y < max(1, Y),
 * z < 32*max(1, Z/32); voxels outside stay zero, as there.
 *
 * MinMax (reference: shaders/min_max.glsl:9-24, beamformer.c:595-607): level l
 * holds (min over a 2x2x2 block of level l-1's .x, max of its .y), reads
 * outside level l-1 give 0, initial values (1e9, 0). Texels the reference's
 * dispatch never writes are set to NaN. min_max_fused builds up to four levels
 * per launch: a block reads the 2^k x 2^k x 2^k texels of level L0 under one
 * level-(L0 + k) texel once into shared memory (outside level L0: 0), then
 * makes each coarser level of that subtree from the previous one on chip and
 * writes it (a texel outside its level is kept as 0 for the next level, one
 * outside the dispatch as NaN, as the reference's texture holds them). A
 * 128 x 128 x 256 frame's eight levels take two launches instead of eight.
 */
#include "bf_kernels.h"

#include <algorithm>

namespace bf {

struct SumInputs { const float2 *in[16]; };

__global__ void __launch_bounds__(256)
sum_frames(float2 *out, SumInputs ins, int count, float k, int X, int Y, int Z, int cx, int cy, int cz)
{
	const int64_t n = (int64_t)X * Y * Z;
	for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
		int x = (int)(v % X), y = (int)((v / X) % Y), z = (int)(v / ((int64_t)X * Y));
		float2 acc = make_float2(0.0f, 0.0f);
		if (x < cx && y < cy && z < cz) {
			for (int i = 0; i < count; i++) {
				float2 a = ins.in[i] ? __ldcs(ins.in[i] + v) : make_float2(0.0f, 0.0f);
				acc.x = __fadd_rn(acc.x, __fmul_rn(k, a.x));
				acc.y = __fadd_rn(acc.y, __fmul_rn(k, a.y));
			}
		}
		out[v] = acc;
	}
}

struct MipLevels {
	int32_t X[16], Y[16], Z[16];      /* level dims, max(1, d >> l); l = 0 is the frame */
	int32_t cx[16], cy[16], cz[16];   /* the reference's dispatch bounds per level */
	int64_t off[16];                  /* texel offset of level l >= 1 in the levels array */
};

constexpr int MM_MAX_K = 4;
constexpr int MM_SMEM = 4096 + 512 + 64 + 8 + 1;   /* texels of a depth-4 subtree */

__global__ void __launch_bounds__(256)
min_max_fused(const float2 *__restrict__ src, float2 *__restrict__ levels, const __grid_constant__ MipLevels m,
              int L0, int k)
{
	__shared__ float2 t[MM_SMEM];
	const int S = 1 << k;
	const int pX = m.X[L0], pY = m.Y[L0], pZ = m.Z[L0];
	float2 *prev = t;
	/* edges are powers of two: coordinates by shifts and masks */
	for (int q = threadIdx.x; q < S * S * S; q += blockDim.x) {
		const int i = q & (S - 1), j = (q >> k) & (S - 1), kk = q >> (2 * k);
		const int x = blockIdx.x * S + i, y = blockIdx.y * S + j, z = blockIdx.z * S + kk;
		prev[q] = (x < pX && y < pY && z < pZ) ? __ldg(src + ((int64_t)z * pY + y) * pX + x) : make_float2(0.0f, 0.0f);
	}
	__syncthreads();
	int edge = S;
	for (int lev = 1; lev <= k; lev++) {
		const int l = L0 + lev, pe = edge, le = k - lev;   /* edge = 1 << le */
		edge >>= 1;
		float2 *cur = prev + pe * pe * pe;
		const int X = m.X[l], Y = m.Y[l], Z = m.Z[l];
		for (int q = threadIdx.x; q < edge * edge * edge; q += blockDim.x) {
			const int i = q & (edge - 1), j = (q >> le) & (edge - 1), kk = q >> (2 * le);
			const int x = blockIdx.x * edge + i, y = blockIdx.y * edge + j, z = blockIdx.z * edge + kk;
			float2 v = make_float2(0.0f, 0.0f);
			if (x < X && y < Y && z < Z) {
				if (x < m.cx[l] && y < m.cy[l] && z < m.cz[l]) {
					float mn = 1000000000.0f, mx = 0.0f;
					#pragma unroll
					for (int c = 0; c < 8; c++) {
						const float2 w = prev[((2 * kk + (c >> 2)) * pe + 2 * j + ((c >> 1) & 1)) * pe + 2 * i + (c & 1)];
						mn = fminf(mn, w.x);
						mx = fmaxf(mx, w.y);
					}
					v = make_float2(mn, mx);
				} else {
					v = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
				}
				levels[m.off[l] + ((int64_t)z * Y + y) * X + x] = v;
			}
			cur[q] = v;
		}
		__syncthreads();
		prev = cur;
	}
}

static int grid_for(int64_t n)
{
	int64_t g = (n + 255) / 256;
	const int64_t most = (int64_t)device_sm_count() * 16;
	return (int)(g < most ? (g < 1 ? 1 : g) : most);
}

static int orone(int x) { return x ? x : 1; }

cudaError_t launch_sum(float2 *out, const float2 *const *ins, int count, float prescale, const int32_t dims[3],
                       cudaStream_t s)
{
	if (count > 16) return cudaErrorInvalidValue;
	SumInputs si = {};
	for (int i = 0; i < count; i++) si.in[i] = ins[i];
	const int X = dims[0], Y = dims[1], Z = dims[2];
	const int64_t n = (int64_t)X * Y * Z;
	sum_frames<<<grid_for(n), 256, 0, s>>>(out, si, count, prescale, X, Y, Z, 32 * orone(X / 32), orone(Y),
	                                        32 * orone(Z / 32));
	g_kernel_launches++;
	return cudaGetLastError();
}

cudaError_t launch_min_max(const float2 *level0, const int32_t dims[3], int mips, float2 *levels, cudaStream_t s)
{
	if (mips <= 1) return cudaSuccess;
	if (mips > 16) return cudaErrorInvalidValue;
	MipLevels m{};
	int64_t off = 0;
	for (int l = 0; l < mips; l++) {
		const unsigned w = (unsigned)dims[0] >> l, h = (unsigned)dims[1] >> l, d = (unsigned)dims[2] >> l;
		m.X[l] = w ? (int)w : 1;
		m.Y[l] = h ? (int)h : 1;
		m.Z[l] = d ? (int)d : 1;
		m.cx[l] = 32 * orone((int)w / 32);
		m.cy[l] = orone((int)h);
		m.cz[l] = 32 * orone((int)d / 32);
		if (l >= 1) {
			m.off[l] = off;
			off += (int64_t)m.X[l] * m.Y[l] * m.Z[l];
		}
	}
	for (int L0 = 0; L0 < mips - 1; L0 += MM_MAX_K) {
		const int k = mips - 1 - L0 < MM_MAX_K ? mips - 1 - L0 : MM_MAX_K;
		/* blocks: enough subtrees to cover every level written by this launch */
		int gx = 1, gy = 1, gz = 1;
		for (int lev = 1; lev <= k; lev++) {
			const int sh = k - lev, l = L0 + lev;
			gx = std::max(gx, (m.X[l] + (1 << sh) - 1) >> sh);
			gy = std::max(gy, (m.Y[l] + (1 << sh) - 1) >> sh);
			gz = std::max(gz, (m.Z[l] + (1 << sh) - 1) >> sh);
		}
		const float2 *src = L0 == 0 ? level0 : levels + m.off[L0];
		min_max_fused<<<dim3(gx, gy, gz), 256, 0, s>>>(src, levels, m, L0, k);
		g_kernel_launches++;
		const cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	return cudaSuccess;
}

} /* namespace bf */

namespace bf {

/* Shared-memory streaming probe (the measured peak of the L1/shared-memory data
 * path that bounds delay-and-sum): every warp reads 32 consecutive 16-byte words
 * per LDS.128 (conflict-free, 128 bytes per quarter-warp wavefront), eight loads
 * in flight per thread, two logic operations per load to keep them alive. */
__global__ void __launch_bounds__(256) shared_stream(int iters, unsigned *sink)
{
	__shared__ uint4 buf[2048];                                  /* 32 KB */
	for (int i = threadIdx.x; i < 2048; i += blockDim.x)
		buf[i] = make_uint4(i, 3u * i + 1u, 5u * i + 2u, 7u * i + 3u);
	__syncthreads();
	unsigned a = 0, b = 0;
	int k = threadIdx.x;
	for (int it = 0; it < iters; it++) {
		const uint4 *q = buf + (k & 1023);
		#pragma unroll
		for (int u = 0; u < 8; u++) {
			const uint4 v = q[u * 128];
			a ^= v.x ^ v.y;
			b ^= v.z ^ v.w;
		}
		k += 32;
	}
	if ((a ^ b) == 0x9E3779B9u) atomicAdd(sink, 1u);
}

cudaError_t measure_shared_bandwidth(double *bytes_per_second, cudaStream_t s)
{
	constexpr int ITERS = 20000, THREADS = 256;
	const int blocks = device_sm_count() * 4;
	unsigned *sink = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	cudaError_t e = cudaMalloc(&sink, sizeof(unsigned));
	if (e == cudaSuccess) e = cudaEventCreate(&e0);
	if (e == cudaSuccess) e = cudaEventCreate(&e1);
	float best = 0.0f;
	for (int rep = 0; rep < 8 && e == cudaSuccess; rep++) {
		cudaEventRecord(e0, s);
		shared_stream<<<blocks, THREADS, 0, s>>>(ITERS, sink);
		g_kernel_launches++;
		cudaEventRecord(e1, s);
		if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
		float ms = 0.0f;
		if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
		if (rep >= 2 && (best == 0.0f || ms < best)) best = ms;     /* two warm-up runs */
	}
	if (e == cudaSuccess) e = cudaGetLastError();
	if (e == cudaSuccess)
		*bytes_per_second = (double)blocks * THREADS * ITERS * 8 * 16 / (best * 1e-3);
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (sink) cudaFree(sink);
	return e;
}

} /* namespace bf */
