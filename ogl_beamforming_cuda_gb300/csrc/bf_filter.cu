/*
 * bf_filter.cu -- demodulation + decimating FIR, and the complex FIR filter
 * (reference: shaders/filter.glsl:29-91, dispatched by beamformer.c:571-594).
 *
 * Reference semantics, per output n of a (channel, transmit) row:
 *   y[n] = sum_{k=0}^{L-1} w[n*D - L + k] * h[L-1-k]        (w[j<0] = 0)
 * with, for demodulation, w[j] = sqrt(2) * R(-j) (x_j.re, -x_j.im), R the
 * rotation by the demodulation phase of sample j, and for the Filter stage
 * w[j] = x[j] (its rotation of every input by +n and of the sum by -n cancel).
 *
 * GB300 form: a block owns 128*R consecutive outputs of one row. Its input
 * window is read once, coalesced, pre-rotated once per input sample (the phasor
 * of index j comes from a host table, computed with the same float expression as
 * the reference), and stored in shared memory split into D polyphase components,
 * each component "transposed" so that a warp's reads are conflict free. Each
 * thread then produces R consecutive outputs with a register sliding window:
 *   y[n] = sum_phase sum_q w_phase[n - Lp + q] * hp_phase[q],  Lp = ceil(L / D),
 * which reads every staged sample (2R-1)/R times per tap block instead of once
 * per tap. FP32 accumulation (the order differs from the reference's by
 * rounding only).
 *
 * fir_reg<L, D, R, DEMOD> (the float kinds, taps padded to L in {16, 32, 64, 128},
 * decimation D in {1, 2, 4}): a block of 64 threads owns 64 * R consecutive
 * outputs of one row. The rotated input window is staged once in shared memory as
 * pairs of consecutive inputs, transposed so that the lanes' 16-byte reads (two
 * inputs each) are conflict free. Each thread makes R = 8
 * consecutive outputs in one fully unrolled pass over its (R - 1) D + L window
 * inputs: every staged input is read once per thread, and the taps travel by
 * value in the kernel's parameter space, so each product is one FMA with its tap
 * from the constant bank. The other kinds and longer filters take fir_polyphase.
 */
#include "bf_kernels.h"

namespace bf {

constexpr int FIR_THREADS = 128;
constexpr int FIR_R = 4;                       /* outputs per thread */
constexpr int FIR_NB = FIR_THREADS * FIR_R;    /* outputs per block */

__device__ __forceinline__ float snorm_unpack(int16_t v)
{
	float f = (float)v / 32767.0f;
	return fminf(fmaxf(f, -1.0f), 1.0f);
}
__device__ __forceinline__ uint32_t snorm_pack2(float x, float y)
{
	int16_t a = (int16_t)roundf(fminf(fmaxf(x, -1.0f), 1.0f) * 32767.0f);
	int16_t b = (int16_t)roundf(fminf(fmaxf(y, -1.0f), 1.0f) * 32767.0f);
	return (uint32_t)(uint16_t)a | ((uint32_t)(uint16_t)b << 16);
}

/* shared layout: [phase][rr][g] with window element m = g*R + rr */
__global__ void __launch_bounds__(FIR_THREADS)
fir_polyphase(FilterParams p, uint32_t Lp, uint32_t stride)
{
	extern __shared__ float smem[];
	const uint32_t D = p.decimation;
	float2 *w  = (float2 *)smem;                                   /* D * R * stride */
	float  *hp = smem + 2 * (size_t)D * FIR_R * stride;            /* D * Lp taps */

	const uint32_t c = blockIdx.y, t = blockIdx.z;
	const int64_t n0 = (int64_t)blockIdx.x * FIR_NB;
	const uint32_t in_ch = p.map_channels ? (uint32_t)(int32_t)p.channel_map[c] : c;
	const uint64_t in_row  = (uint64_t)p.st.in_channel * in_ch + (uint64_t)p.st.in_transmit * t;
	const uint64_t out_row = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t;

	for (uint32_t i = threadIdx.x; i < D * Lp; i += FIR_THREADS) hp[i] = __ldg(p.taps + i);

	/* window: m in [n0 - Lp, n0 + NB + R), j = m*D + phase; the last R entries only
	 * meet zero taps but must hold finite values */
	const uint32_t M = FIR_NB + Lp + FIR_R;
	const int64_t j0 = (n0 - (int64_t)Lp) * (int64_t)D;
	for (uint32_t q = threadIdx.x; q < M * D; q += FIR_THREADS) {
		int64_t j = j0 + q;                 /* consecutive threads -> consecutive inputs */
		uint32_t m = q / D, ph = q - m * D;
		float2 v = make_float2(0.0f, 0.0f);
		if (j >= 0 && j < (int64_t)p.in_samples) {
			uint64_t e = in_row + (uint64_t)p.st.in_sample * (uint64_t)j;
			if (e < p.in_elems) {
				if (p.kind == FILT_DEMOD_I16) {
					uint32_t word = __ldg((const uint32_t *)p.in + e);
					v = make_float2(snorm_unpack((int16_t)(word & 0xFFFFu)), snorm_unpack((int16_t)(word >> 16)));
				} else {
					v = __ldg((const float2 *)p.in + e);
				}
			}
			if (p.kind != FILT_COMPLEX) {
				/* sqrt(2) * rotate_iq(v * (1, -1), -j) */
				float2 ph2 = __ldg(p.phasor + j);
				float x0 = v.x, y0 = -v.y;
				float qx = ph2.x * x0 + ph2.y * y0;
				float qy = -ph2.y * x0 + ph2.x * y0;
				v = make_float2(1.41421356f * qx, 1.41421356f * qy);
			}
		}
		w[((size_t)ph * FIR_R + (m % FIR_R)) * stride + m / FIR_R] = v;
	}
	__syncthreads();

	float2 acc[FIR_R];
	#pragma unroll
	for (int r = 0; r < FIR_R; r++) acc[r] = make_float2(0.0f, 0.0f);

	const uint32_t th = threadIdx.x;
	for (uint32_t ph = 0; ph < D; ph++) {
		const float2 *wp = w + (size_t)ph * FIR_R * stride;
		const float  *hq = hp + (size_t)ph * Lp;
		for (uint32_t q0 = 0; q0 < Lp; q0 += FIR_R) {
			float2 x[2 * FIR_R - 1];
			#pragma unroll
			for (int k = 0; k < 2 * FIR_R - 1; k++) {
				uint32_t m = th * FIR_R + q0 + k;              /* window index */
				x[k] = wp[(m % FIR_R) * stride + m / FIR_R];
			}
			#pragma unroll
			for (int qq = 0; qq < FIR_R; qq++) {
				float h = (q0 + qq < Lp) ? hq[q0 + qq] : 0.0f;
				#pragma unroll
				for (int r = 0; r < FIR_R; r++) {
					acc[r].x = fmaf(x[r + qq].x, h, acc[r].x);
					acc[r].y = fmaf(x[r + qq].y, h, acc[r].y);
				}
			}
		}
	}

	#pragma unroll
	for (int r = 0; r < FIR_R; r++) {
		int64_t n = n0 + (int64_t)th * FIR_R + r;
		if (n >= (int64_t)p.out_samples) break;
		uint64_t o = out_row + (uint64_t)p.st.out_sample * (uint64_t)n;
		if (o >= p.out_elems) continue;
		if (p.kind == FILT_DEMOD_I16) ((uint32_t *)p.out)[o] = snorm_pack2(acc[r].x, acc[r].y);
		else                          ((float2 *)p.out)[o] = acc[r];
	}
}

/* ---------------- register-blocked FIR (float kinds) ---------------- */

constexpr int FIRR_THREADS = 64;
constexpr int FIRR_MAX_TAPS = 128;
struct FirTaps { float h[FIRR_MAX_TAPS]; };      /* h[0 .. L), zero beyond the filter */

template <int L, int D, int R, bool DEMOD>
__global__ void __launch_bounds__(FIRR_THREADS)
fir_reg(FilterParams p, const __grid_constant__ FirTaps taps)
{
	constexpr int NB = FIRR_THREADS * R;          /* outputs per block */
	constexpr int RD = R * D;
	constexpr int HD = RD / 2;                    /* input pairs per thread step */
	constexpr int WIN = NB * D + L;               /* inputs j in [n0 D - L, (n0 + NB) D) */
	/* input pairs (m, m + 1), m even, as float4: pair P at [(P % HD) S + P / HD]; the odd
	 * stride keeps the staging stores and the lanes' LDS.128 reads conflict free */
	constexpr int S = ((WIN / 2 + HD - 1) / HD + 1) | 1;
	static_assert(RD % 2 == 0, "pairs of inputs per thread step");
	__shared__ float4 w[HD * S];

	const uint32_t c = blockIdx.y, t = blockIdx.z;
	const int64_t n0 = (int64_t)blockIdx.x * NB;
	const int64_t j0 = n0 * D - L;
	const uint32_t in_ch = p.map_channels ? (uint32_t)(int32_t)p.channel_map[c] : c;
	const uint64_t in_row  = (uint64_t)p.st.in_channel * in_ch + (uint64_t)p.st.in_transmit * t;
	const uint64_t out_row = (uint64_t)p.st.out_channel * c + (uint64_t)p.st.out_transmit * t;

	/* staging in groups of G inputs per thread: all loads of a group are issued
	 * before its rotations and stores, so G input (and phasor) loads are in flight */
	constexpr int PER = (WIN + FIRR_THREADS - 1) / FIRR_THREADS, G = 6;
	#pragma unroll
	for (int k0 = 0; k0 < PER; k0 += G) {
		float2 v[G], ph[G];
		#pragma unroll
		for (int k = 0; k < G; k++) {
			const int q = threadIdx.x + (k0 + k) * FIRR_THREADS;
			const int64_t j = j0 + q;
			const bool in_win = k0 + k < PER && q < WIN && j >= 0 && j < (int64_t)p.in_samples;
			const uint64_t e = in_row + (uint64_t)p.st.in_sample * (uint64_t)j;
			v[k] = in_win && e < p.in_elems ? __ldg((const float2 *)p.in + e) : make_float2(0.0f, 0.0f);
			if (DEMOD) ph[k] = in_win ? __ldg(p.phasor + j) : make_float2(0.0f, 0.0f);
		}
		#pragma unroll
		for (int k = 0; k < G; k++) {
			const int q = threadIdx.x + (k0 + k) * FIRR_THREADS;
			if (k0 + k >= PER || q >= WIN) break;
			float2 x = v[k];
			if (DEMOD) {
				/* sqrt(2) * rotate_iq(v * (1, -1), -j) */
				const float x0 = x.x, y0 = -x.y;
				x = make_float2(1.41421356f * (ph[k].x * x0 + ph[k].y * y0), 1.41421356f * (ph[k].x * y0 - ph[k].y * x0));
			}
			const int P = q / 2;
			((float2 *)w)[2 * ((P % HD) * S + P / HD) + (q & 1)] = x;
		}
	}
	__syncthreads();

	/* output n0 + th R + r reads inputs e = th R D + r D + k, k < L, with tap h[L - 1 - k];
	 * one LDS.128 brings inputs 2 i2 and 2 i2 + 1 (the window's last pair may hold one
	 * input past the taps, which no output uses) */
	const int th = threadIdx.x;
	float2 acc[R];
	#pragma unroll
	for (int r = 0; r < R; r++) acc[r] = make_float2(0.0f, 0.0f);
	#pragma unroll
	for (int i2 = 0; i2 < ((R - 1) * D + L + 1) / 2; i2++) {
		const float4 xx = w[(i2 % HD) * S + th + i2 / HD];
		#pragma unroll
		for (int h = 0; h < 2; h++) {
			const int i = 2 * i2 + h;
			const float2 x = h ? make_float2(xx.z, xx.w) : make_float2(xx.x, xx.y);
			#pragma unroll
			for (int r = 0; r < R; r++) {
				const int k = i - r * D;
				if (k >= 0 && k < L) {
					acc[r].x = fmaf(x.x, taps.h[L - 1 - k], acc[r].x);
					acc[r].y = fmaf(x.y, taps.h[L - 1 - k], acc[r].y);
				}
			}
		}
	}
	#pragma unroll
	for (int r = 0; r < R; r++) {
		const int64_t n = n0 + (int64_t)th * R + r;
		if (n >= (int64_t)p.out_samples) break;
		const uint64_t o = out_row + (uint64_t)p.st.out_sample * (uint64_t)n;
		if (o < p.out_elems) ((float2 *)p.out)[o] = acc[r];
	}
}

template <int L, int D>
static void launch_fir_reg(const FilterParams &p, const FirTaps &taps, cudaStream_t s)
{
	constexpr int R = 8;
	const dim3 grid((p.out_samples + FIRR_THREADS * R - 1) / (FIRR_THREADS * R), p.channels, p.transmits);
	if (p.kind == FILT_COMPLEX) fir_reg<L, D, R, false><<<grid, FIRR_THREADS, 0, s>>>(p, taps);
	else                        fir_reg<L, D, R, true><<<grid, FIRR_THREADS, 0, s>>>(p, taps);
}

template <int D>
static bool launch_fir_reg_d(const FilterParams &p, const FirTaps &taps, cudaStream_t s)
{
	const uint32_t L = p.taps_len;
	if (L <= 16)       launch_fir_reg<16, D>(p, taps, s);
	else if (L <= 32)  launch_fir_reg<32, D>(p, taps, s);
	else if (L <= 64)  launch_fir_reg<64, D>(p, taps, s);
	else if (L <= 128) launch_fir_reg<128, D>(p, taps, s);
	else return false;
	return true;
}

/* the register-blocked FIR for float kinds, decimation 1, 2 or 4 and up to 128
 * taps; false where it does not apply */
static bool try_fir_reg(const FilterParams &p, cudaStream_t s)
{
	if (p.kind == FILT_DEMOD_I16 || !p.host_taps || p.taps_len == 0 || p.taps_len > FIRR_MAX_TAPS) return false;
	if (p.kind != FILT_COMPLEX && !p.phasor) return false;
	const uint32_t D = p.decimation ? p.decimation : 1;
	if (D != 1 && D != 2 && D != 4) return false;
	/* taps padded at the high end to the kernel's length: h[i] = 0 for i >= taps_len
	 * (the window then starts earlier, and the padded taps weigh the extra inputs
	 * by zero) */
	FirTaps taps{};
	for (uint32_t i = 0; i < p.taps_len; i++) taps.h[i] = p.host_taps[i];
	if (D == 1) return launch_fir_reg_d<1>(p, taps, s);
	if (D == 2) return launch_fir_reg_d<2>(p, taps, s);
	return launch_fir_reg_d<4>(p, taps, s);
}

cudaError_t launch_filter(const FilterParams &p, cudaStream_t s)
{
	if (p.out_samples == 0 || p.channels == 0 || p.transmits == 0) return cudaSuccess;
	if (try_fir_reg(p, s)) {
		g_kernel_launches++;
		return cudaGetLastError();
	}
	const uint32_t D = p.decimation ? p.decimation : 1;
	const uint32_t Lp = (p.taps_len + D - 1) / D;
	const uint32_t M = FIR_NB + Lp + FIR_R;
	const uint32_t stride = (M + FIR_R - 1) / FIR_R + 1;
	size_t smem = sizeof(float2) * (size_t)D * FIR_R * stride + sizeof(float) * (size_t)D * Lp;
	static bool attr_set = false;
	if (!attr_set) {
		cudaFuncSetAttribute(fir_polyphase, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
		attr_set = true;
	}
	if (smem > 200 * 1024) return cudaErrorInvalidValue;
	FilterParams q = p;
	q.decimation = D;
	dim3 grid((p.out_samples + FIR_NB - 1) / FIR_NB, p.channels, p.transmits);
	fir_polyphase<<<grid, FIR_THREADS, smem, s>>>(q, Lp, stride);
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
