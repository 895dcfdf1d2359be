/*
 * bf_hilbert.cu -- the CudaHilbert stage: the analytic signal of every channel
 * row (reference: BeamformerShaderKind_CudaHilbert, dispatched to the external
 * cuda_toolkit plugin's cuda_hilbert(input, output) at beamformer.c:567-570 and
 * kept by the planner only when no Demodulate stage exists, beamformer.c:314-340;
 * the plugin's source is not part of the reference).
 *
 * For a row x of N real samples (the real parts of the row in the channel
 * buffer, [channel][transmit][sample] complex, N = samples per row) the output
 * row is the discrete analytic signal z = x + i H{x} (Marple, "Computing the
 * discrete-time analytic signal via FFT", IEEE Trans. Signal Processing 47(9),
 * 1999): Z = FFT(x); Z[0] and Z[N/2] kept, Z[1 .. N/2-1] doubled, Z[N/2+1 ..]
 * zeroed; z = IFFT(Z) = conj(FFT(conj(Z))) / N.
 *
 * The row is read once from HBM into shared memory and written once; both
 * transforms stay on chip. N <= 8192: the real-input form (two N/2-point
 * transforms, see analytic_rows_stockham) with a Stockham autosort FFT (natural
 * order in and out, no bit reversal; Govindaraju et al., "High performance
 * discrete Fourier transforms on graphics processors", SC 2008) in radix-8 passes
 * and one radix-4 or radix-2 pass, ping-pong between two shared buffers whose
 * index is padded by one element per 32 (the strided writes of the early passes
 * then spread over the banks). Rows shorter than 4096 samples share a CTA. N = 16384:
 * in-place radix-2 (bit-reversed load, decimation in time forward, decimation in
 * frequency inverse), 128 KB of shared memory. Twiddles w[m] = exp(-2 pi i m / N),
 * m < N / 2, come from a table the host computes in double precision.
 */
#include "bf_kernels.h"

#include <cmath>

namespace bf {

static __device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
	return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void __launch_bounds__(256)
analytic_rows(const float2 *__restrict__ in, float2 *__restrict__ out, int64_t rows, int log2n,
              const float2 *__restrict__ tw)
{
	extern __shared__ float2 a[];
	const int n = 1 << log2n, half = n >> 1;
	const int shift = 32 - log2n;
	const float scale = 1.0f / (float)n;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const float2 *src = in + row * n;
		float2 *dst = out + row * n;
		for (int s = threadIdx.x; s < n; s += blockDim.x)
			a[__brev((unsigned)s) >> shift] = make_float2(__ldcs(src + s).x, 0.0f);
		__syncthreads();
		/* forward, decimation in time: stage of length len uses w^(j n / len) */
		for (int len = 2, ts = half; len <= n; len <<= 1, ts >>= 1) {
			const int hl = len >> 1;
			for (int k = threadIdx.x; k < half; k += blockDim.x) {
				const int j = k & (hl - 1), i0 = 2 * (k - j) + j, i1 = i0 + hl;
				const float2 t = cmul(__ldg(tw + j * ts), a[i1]);
				const float2 u = a[i0];
				a[i0] = make_float2(u.x + t.x, u.y + t.y);
				a[i1] = make_float2(u.x - t.x, u.y - t.y);
			}
			__syncthreads();
		}
		/* one-sided spectrum */
		for (int s = threadIdx.x; s < n; s += blockDim.x) {
			const float g = (s == 0 || s == half) ? 1.0f : (s < half ? 2.0f : 0.0f);
			a[s] = make_float2(a[s].x * g, a[s].y * g);
		}
		__syncthreads();
		/* inverse, decimation in frequency with conj(w): natural in, bit-reversed out */
		for (int len = n, ts = 1; len >= 2; len >>= 1, ts <<= 1) {
			const int hl = len >> 1;
			for (int k = threadIdx.x; k < half; k += blockDim.x) {
				const int j = k & (hl - 1), i0 = 2 * (k - j) + j, i1 = i0 + hl;
				const float2 w = __ldg(tw + j * ts);
				const float2 u = a[i0], v = a[i1];
				a[i0] = make_float2(u.x + v.x, u.y + v.y);
				a[i1] = cmul(make_float2(u.x - v.x, u.y - v.y), make_float2(w.x, -w.y));
			}
			__syncthreads();
		}
		for (int s = threadIdx.x; s < n; s += blockDim.x) {
			const float2 z = a[__brev((unsigned)s) >> shift];
			__stcs(dst + s, make_float2(z.x * scale, z.y * scale));
		}
		__syncthreads();
	}
}

/* ---------------- Stockham radix-8/4/2 (N <= 8192) ---------------- */

static __device__ __forceinline__ int pad(int e) { return e + (e >> 5); }

static __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
static __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
/* a * (-i) */
static __device__ __forceinline__ float2 cmi(float2 a) { return make_float2(a.y, -a.x); }

static __device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
	const float2 t = a;
	a = cadd(t, b);
	b = csub(t, b);
}

/* forward 4-point DFT (exp(-2 pi i / 4) = -i) */
static __device__ __forceinline__ void dft4(float2 &a, float2 &b, float2 &c, float2 &d)
{
	const float2 t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(b, d), t3 = cmi(csub(b, d));
	a = cadd(t0, t2);
	c = csub(t0, t2);
	b = cadd(t1, t3);
	d = csub(t1, t3);
}

/* forward 8-point DFT: two 4-point DFTs of the even and odd inputs, combined with
 * exp(-2 pi i k / 8) */
static __device__ __forceinline__ void dft8(float2 *v)
{
	const float h = 0.70710678118654752f;
	dft4(v[0], v[2], v[4], v[6]);
	dft4(v[1], v[3], v[5], v[7]);
	const float2 o1 = make_float2(h * (v[3].x + v[3].y), h * (v[3].y - v[3].x));     /* * exp(-i pi/4) */
	const float2 o2 = cmi(v[5]);                                                    /* * -i */
	const float2 o3 = make_float2(h * (v[7].y - v[7].x), -h * (v[7].x + v[7].y));   /* * exp(-3 i pi/4) */
	const float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
	v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
	v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
	v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
	v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}

/* One Stockham pass of radix R over E / N rows of N elements: sub-transforms of
 * length Ns become length Ns * R. */
template <int R>
static __device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst, int E,
                                                     int N, int Ns, const float2 *__restrict__ tw, int tw_n)
{
	const int per_row = N / R;
	const int tstep = tw_n / (Ns * R);                 /* tw[m] = exp(-2 pi i m / tw_n) */
	for (int g = threadIdx.x; g < E / R; g += blockDim.x) {
		const int row = g / per_row, j = g - row * per_row;
		const int base = row * N, k = j % Ns;
		const float2 w1 = __ldg(tw + k * tstep);
		float2 v[R];
		float2 w = w1;
		v[0] = src[pad(base + j)];
		#pragma unroll
		for (int r = 1; r < R; r++) {
			v[r] = cmul(src[pad(base + j + r * per_row)], w);
			w = cmul(w, w1);
		}
		if (R == 8) dft8(v);
		else if (R == 4) dft4(v[0], v[1], v[2], v[3]);
		else dft2(v[0], v[1]);
		const int d = base + (j / Ns) * Ns * R + k;
		#pragma unroll
		for (int r = 0; r < R; r++) dst[pad(d + r * Ns)] = v[r];
	}
}

/* forward N-point FFT of every row of b0 (twiddles from a table for tw_n >= N
 * points); returns the buffer holding the result */
static __device__ float2 *stockham_fft(float2 *b0, float2 *b1, int E, int N, const float2 *__restrict__ tw, int tw_n)
{
	int Ns = 1;
	while (N / Ns >= 8) {
		stockham_pass<8>(b0, b1, E, N, Ns, tw, tw_n);
		__syncthreads();
		float2 *t = b0; b0 = b1; b1 = t;
		Ns *= 8;
	}
	if (N / Ns == 4) {
		stockham_pass<4>(b0, b1, E, N, Ns, tw, tw_n);
		__syncthreads();
		float2 *t = b0; b0 = b1; b1 = t;
	} else if (N / Ns == 2) {
		stockham_pass<2>(b0, b1, E, N, Ns, tw, tw_n);
		__syncthreads();
		float2 *t = b0; b0 = b1; b1 = t;
	}
	return b0;
}

static __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
static __device__ __forceinline__ float2 cscale(float2 a, float k) { return make_float2(a.x * k, a.y * k); }
/* a * (-i/2): the 1/(2i) of the even/odd split */
static __device__ __forceinline__ float2 cmhalfi(float2 a) { return make_float2(0.5f * a.y, -0.5f * a.x); }

/* Real-input form (N = 2M): y[m] = x[2m] + i x[2m+1] is transformed with M points,
 * Y = FFT_M(y). Each pair (k, M - k) of Y gives X[k] = E[k] + W^k O[k] with
 * E[k] = (Y[k] + conj Y[M-k]) / 2, O[k] = (Y[k] - conj Y[M-k]) / (2i), W = exp(-2 pi
 * i / N), for X[k] and X[M-k] at once. The Hilbert spectrum H[k] = -i X[k]
 * (0 < k < M; H[0] = H[M] = 0) is Hermitian, so its real inverse h = H{x} comes
 * from one more M-point transform of V[k] = (H[k] + conj H[M-k]) / 2 +
 * i (H[k] - conj H[M-k]) W^-k / 2: h[2m] + i h[2m+1] = IFFT_M(V)[m]. The output is
 * z = x + i h, whose real part is x itself. */
__global__ void __launch_bounds__(256)
analytic_rows_stockham(const float2 *__restrict__ in, float2 *__restrict__ out, int64_t rows, int n, int rows_per_cta,
                       const float2 *__restrict__ tw)
{
	extern __shared__ float2 smem[];
	const int m = n >> 1;
	const int lm = 31 - __clz(m);                 /* m = 1 << lm */
	const int E = m * rows_per_cta, padded = E + (E >> 5);
	float2 *b0 = smem, *b1 = smem + padded;
	const float scale = 1.0f / (float)m;
	const int P = (m >> 1) + 1;                   /* pairs (k, m - k) per row, k = 0 .. m/2 */
	for (int64_t row0 = (int64_t)blockIdx.x * rows_per_cta; row0 < rows; row0 += (int64_t)gridDim.x * rows_per_cta) {
		const float2 *src = in + row0 * n;
		float2 *dst = out + row0 * n;
		const int64_t avail = rows - row0;
		const int E_rows = (int)(avail < rows_per_cta ? avail : rows_per_cta) * m;
		for (int e = threadIdx.x; e < E; e += blockDim.x) {
			float2 y = make_float2(0.0f, 0.0f);
			if (e < E_rows) {
				const float4 v = __ldg((const float4 *)(src + 2 * (int64_t)e));   /* samples 2k and 2k + 1 */
				y = make_float2(v.x, v.z);
			}
			b0[pad(e)] = y;
		}
		__syncthreads();
		float2 *f = stockham_fft(b0, b1, E, m, tw, n);
		float2 *o = f == b0 ? b1 : b0;
		for (int q = threadIdx.x; q < rows_per_cta * P; q += blockDim.x) {
			const int r = q / P, k = q - r * P, kk = (m - k) & (m - 1);
			const int base = r << lm;
			const float2 Yk = f[pad(base + k)], Ykk = f[pad(base + kk)];
			const float2 Wk = __ldg(tw + k), Wkk = __ldg(tw + kk);
			const float2 Xk  = cadd(cscale(cadd(Yk, cconj(Ykk)), 0.5f), cmul(Wk, cmhalfi(csub(Yk, cconj(Ykk)))));
			const float2 Xkk = cadd(cscale(cadd(Ykk, cconj(Yk)), 0.5f), cmul(Wkk, cmhalfi(csub(Ykk, cconj(Yk)))));
			const float2 Hk  = k == 0 ? make_float2(0.0f, 0.0f) : cmi(Xk);
			const float2 Hkk = kk == 0 ? make_float2(0.0f, 0.0f) : cmi(Xkk);
			const float2 HMk = k == 0 ? make_float2(0.0f, 0.0f) : Hkk;      /* H[M - k] */
			const float2 HMkk = kk == 0 ? make_float2(0.0f, 0.0f) : Hk;     /* H[M - kk] */
			/* V = (H + conj H') / 2 + i (H - conj H') conj(W) / 2; stored conjugated for the
			 * inverse transform done as a forward one */
			const float2 dk = cmul(csub(Hk, cconj(HMk)), cconj(Wk));
			const float2 Vk = cadd(cscale(cadd(Hk, cconj(HMk)), 0.5f), make_float2(-0.5f * dk.y, 0.5f * dk.x));
			o[pad(base + k)] = cconj(Vk);
			if (kk != k) {
				const float2 dkk = cmul(csub(Hkk, cconj(HMkk)), cconj(Wkk));
				const float2 Vkk = cadd(cscale(cadd(Hkk, cconj(HMkk)), 0.5f), make_float2(-0.5f * dkk.y, 0.5f * dkk.x));
				o[pad(base + kk)] = cconj(Vkk);
			}
		}
		__syncthreads();
		float2 *res = stockham_fft(o, f, E, m, tw, n);
		for (int e = threadIdx.x; e < E_rows; e += blockDim.x) {
			const float2 v = cscale(cconj(res[pad(e)]), scale);                   /* h[2k] + i h[2k + 1] */
			const float4 xin = __ldg((const float4 *)(src + 2 * (int64_t)e));
			__stcs((float4 *)(dst + 2 * (int64_t)e), make_float4(xin.x, v.x, xin.z, v.y));
		}
		__syncthreads();
	}
}

/* rows of n real samples are m = n / 2 complex points on chip; rows shorter than
 * 2048 points share a CTA */
static int stockham_rows_per_cta(uint32_t n) { return n / 2 >= 2048 ? 1 : (int)(2048 / (n / 2)); }

static size_t stockham_smem(uint32_t n)
{
	const size_t E = (size_t)(n / 2) * stockham_rows_per_cta(n);
	return 2 * (E + (E >> 5)) * sizeof(float2);
}

bool analytic_supported(uint32_t samples)
{
	return samples >= 2 && samples <= 16384 && (samples & (samples - 1)) == 0;
}

void analytic_twiddles(uint32_t samples, float2 *host_out)
{
	const double two_pi = 6.283185307179586476925286766559;
	for (uint32_t m = 0; m < samples / 2; m++) {
		const double ang = -two_pi * (double)m / (double)samples;
		host_out[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
	}
}

cudaError_t launch_analytic(const float2 *in, float2 *out, int64_t rows, uint32_t samples, const float2 *twiddles,
                            cudaStream_t s)
{
	if (!analytic_supported(samples) || rows < 0 || !twiddles) return cudaErrorInvalidValue;
	if (rows == 0) return cudaSuccess;
	int log2n = 0;
	while ((1u << log2n) < samples) log2n++;
	if (samples <= 8192) {
		const size_t smem = stockham_smem(samples);
		const int rpc = stockham_rows_per_cta(samples);
		if (smem > 48 * 1024) {
			const cudaError_t e = cudaFuncSetAttribute(analytic_rows_stockham, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                                           (int)smem);
			if (e != cudaSuccess) return e;
		}
		int per_sm = 0;
		cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, analytic_rows_stockham, 256, smem);
		if (e != cudaSuccess) return e;
		if (per_sm < 1) return cudaErrorInvalidConfiguration;
		const int64_t ctas_needed = (rows + rpc - 1) / rpc;
		const int64_t max_blocks = (int64_t)device_sm_count() * per_sm;
		const int blocks = (int)(ctas_needed < max_blocks ? ctas_needed : max_blocks);
		analytic_rows_stockham<<<blocks, 256, smem, s>>>(in, out, rows, (int)samples, rpc, twiddles);
	} else {
		const size_t smem = (size_t)samples * sizeof(float2);
		const cudaError_t e = cudaFuncSetAttribute(analytic_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		const int64_t max_blocks = device_sm_count();
		const int blocks = (int)(rows < max_blocks ? rows : max_blocks);
		analytic_rows<<<blocks, 256, smem, s>>>(in, out, rows, log2n, twiddles);
	}
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
