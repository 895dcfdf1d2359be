/*
 * bf_decode.cu -- Hadamard decode (reference: shaders/decode.glsl:57-105 and the
 * two dispatches of beamformer.c:534-561).
 *
 * y[c][t][s] = (sum_i H[t][i] * x[map(c)][i][s]) / N.
 *
 * The reference gathers the raw RF into a [channel][sample][transmit] scratch
 * buffer in a first pass and runs an N-term dot product per output in a second.
 * Here the channel-mapped gather is fused into the load and no scratch buffer
 * exists:
 *   - decode_fwht_i16<N>: int16 RF, Sylvester order N <= 32 (64 and 128:
 *     decode_fwht_i16_split, two threads per column). One thread owns one
 *     (channel, sample) column of N transmits in registers and applies the fast
 *     Walsh-Hadamard transform (log2 N butterfly stages, N log2 N integer adds
 *     instead of N^2 multiply-adds). Integer sums are exact; the final scale by
 *     1/N is exact for powers of two, so the result equals the reference's float
 *     accumulation bit for bit. The kernel is bound by HBM traffic: 2 bytes read
 *     and 4 (real) or 8 (complex) bytes written per output sample.
 *   - decode_generic: any order (Kronecker 12*2^k / 20*2^k included), any input
 *     kind, and decode mode NONE. A 32-sample strip of all transmits is staged in
 *     shared memory and each output is the dot product in the reference's order
 *     (i ascending; h*x is exact for h = +-1), divided once by N.
 */
#include "bf_kernels.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace bf {

uint64_t g_kernel_launches = 0;

template <int N>
__device__ __forceinline__ void fwht(int (&v)[N])
{
	constexpr int LOG2N = N <= 1 ? 0 : 31 - __builtin_clz(N);
	#pragma unroll
	for (int st = 0; st < LOG2N; st++) {
		const int h = 1 << st;
		#pragma unroll
		for (int k = 0; k < N / 2; k++) {
			const int j = ((k >> st) << (st + 1)) | (k & (h - 1));
			const int a = v[j], b = v[j + h];
			v[j]     = a + b;
			v[j + h] = a - b;
		}
	}
}

template <int N>
__global__ void __launch_bounds__(128)
decode_fwht_i16(DecodeParams p)
{
	uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t c = blockIdx.y;
	if (s >= p.samples) return;
	uint32_t mc = p.channel_map ? (uint32_t)(int32_t)p.channel_map[c] : c;
	const int16_t *raw = (const int16_t *)p.in;
	uint64_t base = (uint64_t)p.st.in_channel * mc + (uint64_t)p.st.in_sample * s;

	const bool gathered = s < p.in_limit;
	int v[N];
	#pragma unroll
	for (int t = 0; t < N; t++) {
		uint64_t idx = base + (uint64_t)p.st.in_transmit * t;
		v[t] = (gathered && idx < p.in_elems) ? (int)__ldg(raw + idx) : 0;
	}
	fwht<N>(v);

	const float inv_n = 1.0f / (float)N;   /* exact: N is a power of two */
	if (p.output == DEC_OUT_REAL_F16 || p.output == DEC_OUT_REAL_BF16) {
		/* real pairs layout, 16-bit elements: the value rounded once from the exact
		 * f32 decode */
		uint64_t pair = s >> 1;
		uint16_t *o16 = (uint16_t *)p.out;
		#pragma unroll
		for (int t = 0; t < N; t++) {
			uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t + (uint64_t)p.st.out_sample * pair;
			const float y = __fmul_rn((float)v[t], inv_n);
			if (o < p.out_vec2)
				o16[2 * o + (s & 1)] = p.output == DEC_OUT_REAL_F16 ? __half_as_ushort(__float2half_rn(y))
				                                                     : __bfloat16_as_ushort(__float2bfloat16_rn(y));
		}
	} else if (p.output == DEC_OUT_REAL_PAIRS) {
		uint64_t pair = s >> 1;
		#pragma unroll
		for (int t = 0; t < N; t++) {
			uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t + (uint64_t)p.st.out_sample * pair;
			if (o < p.out_vec2) p.out[2 * o + (s & 1)] = __fmul_rn((float)v[t], inv_n);
		}
	} else {
		float2 *out = (float2 *)p.out;
		#pragma unroll
		for (int t = 0; t < N; t++) {
			uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t + (uint64_t)p.st.out_sample * s;
			if (o < p.out_vec2) out[o] = make_float2(__fmul_rn((float)v[t], inv_n), 0.0f);
		}
	}
}

/* Orders N = 64, 128: two threads per (channel, sample) column, each holding N/2
 * transmits (lanes 0-15 of a warp the first half, 16-31 the second half, of 16
 * columns), so a thread needs half the registers and twice the warps fit per SM.
 * The FWHT stages inside a half run in registers; the last stage pairs transmit t
 * with t + N/2 across the two lanes through one shuffle. Integer sums: exact in
 * any order. Loads and stores: each half-warp moves 16 consecutive samples of one
 * transmit row. */
template <int N>
__global__ void __launch_bounds__(128, 6)
decode_fwht_i16_split(DecodeParams p)
{
	constexpr int H = N / 2;
	const uint32_t lane = threadIdx.x & 31, q = lane >> 4;
	const uint32_t s = blockIdx.x * 64 + (threadIdx.x >> 5) * 16 + (lane & 15);
	const uint32_t c = blockIdx.y;
	const bool live = s < p.samples;
	const uint32_t mc = p.channel_map ? (uint32_t)(int32_t)p.channel_map[c] : c;
	const int16_t *raw = (const int16_t *)p.in;
	const uint64_t base = (uint64_t)p.st.in_channel * mc + (uint64_t)p.st.in_sample * s +
	                      (uint64_t)p.st.in_transmit * (q * H);
	const bool gathered = live && s < p.in_limit;
	int v[H];
	#pragma unroll
	for (int k = 0; k < H; k++) {
		const uint64_t idx = base + (uint64_t)p.st.in_transmit * k;
		v[k] = (gathered && idx < p.in_elems) ? (int)__ldg(raw + idx) : 0;
	}
	fwht<H>(v);
	#pragma unroll
	for (int k = 0; k < H; k++) {
		const int other = __shfl_xor_sync(0xffffffffu, v[k], 16);
		v[k] = q ? other - v[k] : v[k] + other;
	}
	if (!live) return;

	const float inv_n = 1.0f / (float)N;   /* exact: N is a power of two */
	const uint32_t t0 = q * H;
	if (p.output == DEC_OUT_REAL_F16 || p.output == DEC_OUT_REAL_BF16) {
		const uint64_t pair = s >> 1;
		uint16_t *o16 = (uint16_t *)p.out;
		#pragma unroll
		for (int k = 0; k < H; k++) {
			const uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * (t0 + k) +
			                   (uint64_t)p.st.out_sample * pair;
			const float y = __fmul_rn((float)v[k], inv_n);
			if (o < p.out_vec2)
				o16[2 * o + (s & 1)] = p.output == DEC_OUT_REAL_F16 ? __half_as_ushort(__float2half_rn(y))
				                                                     : __bfloat16_as_ushort(__float2bfloat16_rn(y));
		}
	} else if (p.output == DEC_OUT_REAL_PAIRS) {
		const uint64_t pair = s >> 1;
		#pragma unroll
		for (int k = 0; k < H; k++) {
			const uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * (t0 + k) +
			                   (uint64_t)p.st.out_sample * pair;
			if (o < p.out_vec2) p.out[2 * o + (s & 1)] = __fmul_rn((float)v[k], inv_n);
		}
	} else {
		float2 *out = (float2 *)p.out;
		#pragma unroll
		for (int k = 0; k < H; k++) {
			const uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * (t0 + k) +
			                   (uint64_t)p.st.out_sample * s;
			if (o < p.out_vec2) out[o] = make_float2(__fmul_rn((float)v[k], inv_n), 0.0f);
		}
	}
}

__device__ __forceinline__ float2 load_input(const DecodeParams &p, uint64_t e)
{
	if (e >= p.in_elems) return make_float2(0.0f, 0.0f);
	switch (p.input) {
	case DEC_IN_I16:  return make_float2((float)__ldg((const int16_t *)p.in + e), 0.0f);
	case DEC_IN_I16C: {
		uint32_t w = __ldg((const uint32_t *)p.in + e);
		return make_float2((float)(int16_t)(w & 0xFFFFu), (float)(int16_t)(w >> 16));
	}
	case DEC_IN_F32:  return make_float2(__ldg((const float *)p.in + e), 0.0f);
	default:          return __ldg((const float2 *)p.in + e);
	}
}

__device__ __forceinline__ void store_output(const DecodeParams &p, uint32_t c, uint32_t t, uint32_t s, float2 y)
{
	if (p.output == DEC_OUT_REAL_PAIRS) {
		uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t + (uint64_t)p.st.out_sample * (s >> 1);
		if (o < p.out_vec2) p.out[2 * o + (s & 1)] = y.x;
	} else {
		uint64_t o = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t + (uint64_t)p.st.out_sample * s;
		if (o < p.out_vec2) ((float2 *)p.out)[o] = y;
	}
}

/* block: 32 samples x 8 transmit lanes; shared: N x 32 float2 */
__global__ void __launch_bounds__(256)
decode_generic(DecodeParams p)
{
	extern __shared__ float2 xs[];
	const uint32_t sx = threadIdx.x, ty = threadIdx.y;
	const uint32_t s = blockIdx.x * 32 + sx, c = blockIdx.y;
	const uint32_t N = p.transmits;
	uint32_t ch = (p.first_stage && p.channel_map) ? (uint32_t)(int32_t)p.channel_map[c] : c;
	uint64_t base = (uint64_t)p.st.in_channel * ch + (uint64_t)p.st.in_sample * s;
	for (uint32_t i = ty; i < N; i += blockDim.y)
		xs[i * 32 + sx] = (s < p.samples && s < p.in_limit) ? load_input(p, base + (uint64_t)p.st.in_transmit * i) : make_float2(0.0f, 0.0f);
	__syncthreads();
	if (s >= p.samples) return;
	for (uint32_t t = ty; t < N; t += blockDim.y) {
		float2 y;
		if (p.hadamard_mode) {
			float ax = 0.0f, ay = 0.0f;
			const int8_t *h = p.hadamard + (uint64_t)t * N;
			for (uint32_t i = 0; i < N; i++) {
				float hv = (float)__ldg(h + i);
				float2 x = xs[i * 32 + sx];
				ax = __fadd_rn(ax, __fmul_rn(hv, x.x));
				ay = __fadd_rn(ay, __fmul_rn(hv, x.y));
			}
			y = make_float2(__fdiv_rn(ax, (float)N), __fdiv_rn(ay, (float)N));
		} else {
			y = xs[t * 32 + sx];
		}
		store_output(p, c, t, s, y);
	}
}

cudaError_t launch_decode(const DecodeParams &p, cudaStream_t s)
{
	if (p.samples == 0 || p.channels == 0 || p.transmits == 0) return cudaSuccess;
	bool fwht_ok = p.hadamard_mode && p.first_stage && p.input == DEC_IN_I16 && p.base == 1 &&
	               p.transmits == p.sylvester && p.transmits <= 128;
	if (fwht_ok && (p.transmits == 64 || p.transmits == 128)) {
		dim3 grid((p.samples + 63) / 64, p.channels), block(128);
		if (p.transmits == 64) decode_fwht_i16_split<64><<<grid, block, 0, s>>>(p);
		else                   decode_fwht_i16_split<128><<<grid, block, 0, s>>>(p);
		g_kernel_launches++;
		return cudaGetLastError();
	}
	if (fwht_ok) {
		dim3 grid((p.samples + 127) / 128, p.channels), block(128);
		switch (p.transmits) {
		case 1:   decode_fwht_i16<1><<<grid, block, 0, s>>>(p); break;
		case 2:   decode_fwht_i16<2><<<grid, block, 0, s>>>(p); break;
		case 4:   decode_fwht_i16<4><<<grid, block, 0, s>>>(p); break;
		case 8:   decode_fwht_i16<8><<<grid, block, 0, s>>>(p); break;
		case 16:  decode_fwht_i16<16><<<grid, block, 0, s>>>(p); break;
		case 32:  decode_fwht_i16<32><<<grid, block, 0, s>>>(p); break;
		default:  fwht_ok = false; break;
		}
		if (fwht_ok) {
			g_kernel_launches++;
			return cudaGetLastError();
		}
	}
	if (p.output == DEC_OUT_REAL_F16 || p.output == DEC_OUT_REAL_BF16) return cudaErrorInvalidValue;
	size_t smem = (size_t)p.transmits * 32 * sizeof(float2);
	static bool attr_set = false;
	if (!attr_set) {
		cudaFuncSetAttribute(decode_generic, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
		attr_set = true;
	}
	if (smem > 160 * 1024) return cudaErrorInvalidValue;
	dim3 grid((p.samples + 31) / 32, p.channels), block(32, 8);
	decode_generic<<<grid, block, smem, s>>>(p);
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
