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
 * outside level l-1 give 0, initial values (1e9, 0). One launch per level; the
 * first level carries almost all of the traffic. Texels the reference's
 * dispatch never writes are set to NaN.
 */
#include "bf_kernels.h"

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

__global__ void __launch_bounds__(256)
min_max_level(const float2 *prev, int pX, int pY, int pZ, float2 *cur, int X, int Y, int Z, int cx, int cy, int cz)
{
	const int64_t n = (int64_t)X * Y * Z;
	for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
		int x = (int)(o % X), y = (int)((o / X) % Y), z = (int)(o / ((int64_t)X * Y));
		if (!(x < cx && y < cy && z < cz)) {
			cur[o] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
			continue;
		}
		float mn = 1000000000.0f, mx = 0.0f;
		#pragma unroll
		for (int k = 0; k < 8; k++) {
			int ix = 2 * x + (k & 1), iy = 2 * y + ((k >> 1) & 1), iz = 2 * z + (k >> 2);
			float2 v = make_float2(0.0f, 0.0f);
			if (ix < pX && iy < pY && iz < pZ) v = __ldg(prev + ((int64_t)iz * pY + iy) * pX + ix);
			mn = fminf(mn, v.x);
			mx = fmaxf(mx, v.y);
		}
		cur[o] = make_float2(mn, mx);
	}
}

static int grid_for(int64_t n)
{
	int64_t g = (n + 255) / 256;
	return (int)(g < 152 * 16 ? (g < 1 ? 1 : g) : 152 * 16);
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
	const float2 *prev = level0;
	int pX = dims[0], pY = dims[1], pZ = dims[2];
	float2 *cur = levels;
	for (int l = 1; l < mips; l++) {
		unsigned w = (unsigned)dims[0] >> l, h = (unsigned)dims[1] >> l, d = (unsigned)dims[2] >> l;
		int X = w ? (int)w : 1, Y = h ? (int)h : 1, Z = d ? (int)d : 1;
		int64_t n = (int64_t)X * Y * Z;
		min_max_level<<<grid_for(n), 256, 0, s>>>(prev, pX, pY, pZ, cur, X, Y, Z, 32 * orone((int)w / 32),
		                                           orone((int)h), 32 * orone((int)d / 32));
		g_kernel_launches++;
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		prev = cur;
		pX = X; pY = Y; pZ = Z;
		cur += n;
	}
	return cudaSuccess;
}

} /* namespace bf */
