/*
 * bf_das_hercules.cu -- delay-and-sum for HERCULES acquisitions (das.glsl:
 * HERCULES case of the fast path, dispatched by beamformer.c:608-681), the
 * configuration the reference's 3D volumes are made with.
 *
 * Same accumulation order as das_kernel (one thread per voxel; per receive
 * channel the transmits inside the apodization aperture are summed, then the
 * channel sum is added to the voxel), with the work
 * per (voxel, transmit, receive) term cut to what the reference's arithmetic needs:
 *
 *   - No range test per term. Each voxel first proves, from bounds on its lateral
 *     and axial distances to the array, that every square-root argument and every
 *     divided distance lies inside the ranges where the fast square root and the
 *     reciprocal division were checked equal to IEEE on this device; voxels that
 *     cannot (a depth of 0, absurd distances) take a copy of the loop with IEEE
 *     operations.
 *   - Interpolation reads a table built once per frame from the channel data: for
 *     every sample n the power-basis coefficients of the reference's cubic Hermite
 *     segment between samples n and n + 1 (two float4), or the linear segment (one
 *     float4). A cubic term is then one 32-byte load and a Horner evaluation in the
 *     fraction instead of four 8-byte loads, four weights and eight products.
 *   - The transmit-0 term (weighted by 1/sqrt(T)) is peeled off the loop.
 *   - The apodization cos^2(sqrt(w)) is one degree-5 polynomial in w (five FMAs,
 *     absolute error 6.4e-7) instead of the squared eighth-order cosine series.
 *   - Demodulated data: the phase exp(i 2 pi fc t) of a term at sample index
 *     j + f (t = (j + f) / fs) splits into exp(i theta (j + 1/2)), stored in the
 *     table segment of sample j, and exp(i theta (f - 1/2)), theta = 2 pi fc / fs:
 *     one FMA and the fast sine and cosine of an angle in [-pi, pi] (|theta| <=
 *     2 pi, which covers fc = fs / 4 of the raw data at decimation 2; larger
 *     theta, e.g. 4 pi at decimation 4, adds a two-constant reduction).
 *     This replaces the reference's time division, angle product and range
 *     reduction per term, and is closer to the exact phase than the float angle
 *     of the reference (whose rounding, up to half an ulp of angles of ~10^3 rad,
 *     is the difference). Without the table (nearest), or for |theta| > 256, the
 *     term computes the reference's angle, reduced with the two-constant split of
 *     2 pi (6.28125 exact in 8 bits, the rest rounded to float; off by at most
 *     |k| * 1.1e-11 rad, k < 2^15).
 *
 * Sample indices stay bit-equal to the reference's: the delay chain is the same
 * sequence of round-to-nearest operations as das_kernel's.
 *
 * DAS precision 1 (DasParams::half_table, the precision variant; H in the
 * templates) trades that exactness for speed within about -57 dB of the FP32
 * volume: the table in FP16 pairs scaled by a power of two from the frame's
 * largest channel-data magnitude (chan_absmax), segments evaluated in packed
 * FP16, the sample index sqrt(x) fs / c + io from an approximate reciprocal
 * square root, a degree-3 apodization, and a thread's two depths in packed FP32
 * pairs; sums stay FP32.
 */
#include "bf_kernels.h"
#include "bf_das_math.cuh"
#include "bf_das_hercules.cuh"
#include "bf_das_staged.cuh"

#include <cstdlib>
#include <cstring>

namespace bf {

/* Interpolation tables, one entry per flat channel-data index n < entries
 * (samples outside [0, readable) read as 0, as the reference's bounded reads do).
 * Cubic (das.glsl:36-62): with P1 = s[n], P2 = s[n+1], T1 = (s[n+1] - s[n-1]) / 2,
 * T2 = (s[n+2] - s[n]) / 2 the segment is a0 + a1 f + a2 f^2 + a3 f^3 with
 * a0 = P1, a1 = T1, a2 = 3 (P2 - P1) - 2 T1 - T2, a3 = 2 (P1 - P2) + T1 + T2;
 * stored as float4 (a0, a1) and float4 (a2, a3), complex pairs.
 * Linear: float4 (s[n], s[n+1] - s[n]). Nearest (ROT only): float2 s[n].
 * ROT: every coefficient of the segment starting at sample j = n mod S of its row
 * is multiplied by exp(i theta (j + 1/2)), the demodulation phase at the middle of
 * the segment (nearest: exp(i theta j), rot_half = 0), from its turns
 * (j * rot_step + rot_half) / 2^32 (0.32 fixed point: the product wraps exactly;
 * the phase error is at most (j + 1) * 2^-33 turns). */
/* Largest |component| of the channel data rf[0, n), as float bits into *out
 * (zeroed before; NaN components are skipped): the scale of the FP16 table. */
__global__ void __launch_bounds__(256)
chan_absmax(const float2 *__restrict__ rf, int64_t n, unsigned *__restrict__ out)
{
	float m = 0.0f;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float2 v = __ldg(rf + i);
		m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
	}
	/* non-negative floats order as their bit patterns */
	const unsigned b = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
	if ((threadIdx.x & 31) == 0 && b) atomicMax(out, b);
}

/* H: DAS precision 1, every complex coefficient times 2^k (half_table_shift of
 * *absmax) rounded to an FP16 pair: cubic 16 bytes (a0, a1, a2, a3), linear 8
 * bytes (a0, a1), nearest 4 bytes (rotated or not). */
template <int INTERP, bool ROT, bool H = false>
__global__ void __launch_bounds__(256)
interp_table(const float2 *__restrict__ rf, int64_t entries, int64_t readable, int32_t S, uint32_t rot_step,
             uint32_t rot_half, const unsigned *__restrict__ absmax, float4 *__restrict__ out)
{
	const float2 zero = make_float2(0.0f, 0.0f);
	const float hs = H ? pow2f(half_table_shift(__ldg(absmax))) : 1.0f;
	auto h2 = [&](float2 a) {
		const __half2 h = __floats2half2_rn(a.x * hs, a.y * hs);
		unsigned u;
		memcpy(&u, &h, sizeof(u));
		return u;
	};
	for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < entries; n += (int64_t)gridDim.x * blockDim.x) {
		const float2 s1 = n < readable ? rf[n] : zero;
		const float2 s2 = n + 1 < readable ? rf[n + 1] : zero;
		float cs = 1.0f, sn = 0.0f;
		if (ROT) {
			const uint32_t u = (uint32_t)(n % S) * rot_step + rot_half;
			sincospif((float)(int32_t)u * 0x1p-31f, &sn, &cs);
		}
		/* (x + i y) exp(i phi) */
		auto rot = [&](float x, float y) { return make_float2(cs * x - sn * y, sn * x + cs * y); };
		if (INTERP == INTERP_NEAREST) {
			const float2 a0 = ROT ? rot(s1.x, s1.y) : s1;
			if (H) ((unsigned *)out)[n] = h2(a0);
			else   ((float2 *)out)[n] = a0;
			continue;
		}
		if (INTERP == INTERP_LINEAR) {
			const float2 a0 = ROT ? rot(s1.x, s1.y) : s1;
			const float2 a1 = ROT ? rot(s2.x - s1.x, s2.y - s1.y) : make_float2(s2.x - s1.x, s2.y - s1.y);
			if (H) ((uint2 *)out)[n] = make_uint2(h2(a0), h2(a1));
			else   out[n] = make_float4(a0.x, a0.y, a1.x, a1.y);
			continue;
		}
		const float2 s0 = n > 0 && n - 1 < readable ? rf[n - 1] : zero;
		const float2 s3 = n + 2 < readable ? rf[n + 2] : zero;
		const float t1x = 0.5f * (s2.x - s0.x), t1y = 0.5f * (s2.y - s0.y);
		const float t2x = 0.5f * (s3.x - s1.x), t2y = 0.5f * (s3.y - s1.y);
		const float dx = s2.x - s1.x, dy = s2.y - s1.y;
		float2 a0 = s1, a1 = make_float2(t1x, t1y);
		float2 a2 = make_float2(3.0f * dx - 2.0f * t1x - t2x, 3.0f * dy - 2.0f * t1y - t2y);
		float2 a3 = make_float2(t1x + t2x - 2.0f * dx, t1y + t2y - 2.0f * dy);
		if (ROT) {
			a0 = rot(a0.x, a0.y);
			a1 = rot(a1.x, a1.y);
			a2 = rot(a2.x, a2.y);
			a3 = rot(a3.x, a3.y);
		}
		if (H) {
			((uint4 *)out)[n] = make_uint4(h2(a0), h2(a1), h2(a2), h2(a3));
		} else {
			out[2 * n]     = make_float4(a0.x, a0.y, a1.x, a1.y);
			out[2 * n + 1] = make_float4(a2.x, a2.y, a3.x, a3.y);
		}
	}
}

/* 128-thread blocks, 8 per SM (64 registers); 256-thread volume blocks measured
 * slower (96.4 against 94.9 ms per 128 x 128 x 256 cubic frame) */
template <int TY> __host__ __device__ constexpr int herc_threads() { return 128; }

template <int INTERP, int TY, bool H>
__global__ void __launch_bounds__(herc_threads<TY>(), 1024 / herc_threads<TY>())
das_hercules(DasParams p, const float4 *__restrict__ tab)
{
	const int yt = blockIdx.y / p.groups;
	hercules_tile<INTERP, TY, herc_threads<TY>(), H>(p, tab, blockIdx.x, yt, blockIdx.z, blockIdx.y - yt * p.groups);
}

/* The staged form (bf_das_staged.cuh): cubic and linear tables, 8 blocks of 128
 * threads per SM with about 27 KB of shared memory each. */
template <int INTERP, int TY, bool H>
__global__ void __launch_bounds__(128, 8)
das_hercules_staged(DasParams p, const float4 *__restrict__ tab)
{
	extern __shared__ __align__(128) uint8_t stg_smem[];
	const int yt = blockIdx.y / p.groups;
	hercules_tile_staged<INTERP, TY, H>(p, tab, blockIdx.x, yt, blockIdx.z, blockIdx.y - yt * p.groups, stg_smem);
}

/* volume tile of the staged kernel: HercTile<4> (4 x 4 x 16) unless
 * OGL_BF_DAS_STAGED_TILE=8 (4 x 8 x 8, for comparisons) */
static int staged_volume_ty()
{
	const char *env = std::getenv("OGL_BF_DAS_STAGED_TILE");
	return env && env[0] == '8' ? 8 : 4;
}

/* the staged kernel runs for FP32 cubic and linear tables (the FP16 table of DAS
 * precision 1 measured faster unstaged: 52.5 against 60.8 ms per 3D frame);
 * OGL_BF_DAS_STAGED=0 keeps hercules_tile (for comparisons), =1 stages the FP16
 * table of volumes too, =require marks blocks that cannot stage with NaN (tests) */
static bool use_staged(const DasParams &p)
{
	const char *env = std::getenv("OGL_BF_DAS_STAGED");
	if (env && env[0] == '0') return false;
	if (p.interp != INTERP_CUBIC && p.interp != INTERP_LINEAR) return false;
	if (p.half_table && !(env && (env[0] == '1' || env[0] == 'r'))) return false;
	if (p.half_table && p.dims[1] < 4) return false;
	return p.wait_error != nullptr && p.T <= 256 && p.loop_end <= 256 && (p.rot_table != 0 || !(p.fc > 0.0f));
}

bool das_hercules_use_staged(const DasParams &p)
{
	return !p.half_table && use_staged(p);
}

template <int INTERP, int TY, bool H>
static int staged_occupancy()
{
	int n = 0;
	const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, das_hercules_staged<INTERP, TY, H>, 128,
	                                                                    stg_smem_bytes<INTERP, TY, H>());
	return e == cudaSuccess && n > 0 ? n : 1;
}

int64_t das_hercules_table_bytes(const DasParams &p)
{
	const int64_t n = (int64_t)p.C * p.T * p.S;
	/* FP32: cubic 32 bytes per sample, linear 16, nearest 8 (only rotated data);
	 * FP16 (precision 1): half of that, nearest always */
	if (p.half_table) return p.interp == INTERP_CUBIC ? 16 * n : p.interp == INTERP_LINEAR ? 8 * n : 4 * n;
	return p.interp == INTERP_CUBIC ? 32 * n : p.interp == INTERP_LINEAR ? 16 * n : p.rot_table ? 8 * n : 0;
}

int64_t das_hercules_tiles(const DasParams &p)
{
	if (p.dims[1] >= 4 && use_staged(p) && staged_volume_ty() == 8) {
		using T = HercTile<8, 128>;
		return (int64_t)((p.dims[0] + T::X - 1) / T::X) * ((p.dims[1] + T::Y - 1) / T::Y) *
		       ((p.dims[2] + T::Z * T::NV - 1) / (T::Z * T::NV));
	}
	if (p.dims[1] >= 4) {
		using T = HercTile<4, herc_threads<4>()>;
		return (int64_t)((p.dims[0] + T::X - 1) / T::X) * ((p.dims[1] + T::Y - 1) / T::Y) *
		       ((p.dims[2] + T::Z * T::NV - 1) / (T::Z * T::NV));
	}
	using T = HercTile<1, herc_threads<1>()>;
	return (int64_t)((p.dims[0] + T::X - 1) / T::X) * p.dims[1] * ((p.dims[2] + T::Z * T::NV - 1) / (T::Z * T::NV));
}

template <int TY, bool H>
static int hercules_occupancy(int interp)
{
	int n = 0;
	cudaError_t e;
	switch (interp) {
	case INTERP_CUBIC:  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, das_hercules<INTERP_CUBIC, TY, H>, herc_threads<TY>(), 0); break;
	case INTERP_LINEAR: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, das_hercules<INTERP_LINEAR, TY, H>, herc_threads<TY>(), 0); break;
	default:            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, das_hercules<INTERP_NEAREST, TY, H>, herc_threads<TY>(), 0); break;
	}
	return e == cudaSuccess && n > 0 ? n : 1024 / herc_threads<TY>();
}

int das_hercules_blocks_per_sm(const DasParams &p)
{
	static int cache[2][3][2] = {}, staged[2][2][2] = {};
	const int ty = p.dims[1] >= 4 ? 1 : 0, ip = p.interp >= 0 && p.interp < 3 ? p.interp : 0, h = p.half_table ? 1 : 0;
	if (use_staged(p)) {
		/* every staged form fits 8 blocks of 128 threads per SM at 64 registers and
		 * about 27 KB of shared memory; the query confirms it per form */
		int &s = staged[ty][p.interp == INTERP_CUBIC ? 1 : 0][h];
		if (!s) {
			if (p.interp == INTERP_CUBIC)
				s = ty ? (h ? staged_occupancy<INTERP_CUBIC, 4, true>() : staged_occupancy<INTERP_CUBIC, 4, false>())
				       : (h ? staged_occupancy<INTERP_CUBIC, 1, true>() : staged_occupancy<INTERP_CUBIC, 1, false>());
			else
				s = ty ? (h ? staged_occupancy<INTERP_LINEAR, 4, true>() : staged_occupancy<INTERP_LINEAR, 4, false>())
				       : (h ? staged_occupancy<INTERP_LINEAR, 1, true>() : staged_occupancy<INTERP_LINEAR, 1, false>());
		}
		return s;
	}
	int &c = cache[ty][ip][h];
	if (!c) c = ty ? (h ? hercules_occupancy<4, true>(p.interp) : hercules_occupancy<4, false>(p.interp))
	               : (h ? hercules_occupancy<1, true>(p.interp) : hercules_occupancy<1, false>(p.interp));
	return c;
}

bool das_hercules_supported(const DasParams &p)
{
	return p.family == DAS_HERCULES && p.fast && !p.sparse_mode && !p.coherency && p.dense_rows &&
	       p.rf_count >= (int64_t)p.C * p.T * p.S && p.loop_end == p.C;
}

template <int SY, bool H>
static void launch_staged(const DasParams &q, const float4 *table, cudaStream_t s)
{
	using STile = HercTile<SY, 128>;
	const dim3 grid((q.dims[0] + STile::X - 1) / STile::X, ((q.dims[1] + STile::Y - 1) / STile::Y) * q.groups,
	                (q.dims[2] + STile::Z * STile::NV - 1) / (STile::Z * STile::NV));
	if (q.interp == INTERP_CUBIC)
		das_hercules_staged<INTERP_CUBIC, SY, H><<<grid, 128, stg_smem_bytes<INTERP_CUBIC, SY, H>(), s>>>(q, table);
	else
		das_hercules_staged<INTERP_LINEAR, SY, H><<<grid, 128, stg_smem_bytes<INTERP_LINEAR, SY, H>(), s>>>(q, table);
}

template <int TY, bool H>
static void launch_hercules_tiles(const DasParams &p, const float4 *table, cudaStream_t s)
{
	constexpr int THREADS = herc_threads<TY>();
	using Tile = HercTile<TY, THREADS>;
	dim3 grid((p.dims[0] + Tile::X - 1) / Tile::X, ((p.dims[1] + Tile::Y - 1) / Tile::Y) * p.groups,
	          (p.dims[2] + Tile::Z * Tile::NV - 1) / (Tile::Z * Tile::NV));
	if (use_staged(p)) {
		DasParams q = p;
		const char *env = std::getenv("OGL_BF_DAS_STAGED");
		q.stage_only = env && std::strcmp(env, "require") == 0;
		if (TY != 1 && staged_volume_ty() == 8) launch_staged<8, H>(q, table, s);
		else                                    launch_staged<TY, H>(q, table, s);
		return;
	}
	switch (p.interp) {
	case INTERP_CUBIC:  das_hercules<INTERP_CUBIC, TY, H><<<grid, THREADS, 0, s>>>(p, table); break;
	case INTERP_LINEAR: das_hercules<INTERP_LINEAR, TY, H><<<grid, THREADS, 0, s>>>(p, table); break;
	default:            das_hercules<INTERP_NEAREST, TY, H><<<grid, THREADS, 0, s>>>(p, table); break;
	}
}

template <bool H>
static void launch_table(const DasParams &p, int64_t entries, int blocks, float4 *table, cudaStream_t s)
{
	const bool rot = p.rot_table != 0;
	const uint32_t step = rot ? p.rot_step : 0, half = rot ? p.rot_half : 0;
	switch (p.interp * 2 + (rot ? 1 : 0)) {
	case INTERP_NEAREST * 2 + 1: interp_table<INTERP_NEAREST, true, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, step, 0, p.absmax, table); break;
	case INTERP_NEAREST * 2:     interp_table<INTERP_NEAREST, false, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, 0, 0, p.absmax, table); break;
	case INTERP_CUBIC * 2 + 1:   interp_table<INTERP_CUBIC, true, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, step, half, p.absmax, table); break;
	case INTERP_CUBIC * 2:       interp_table<INTERP_CUBIC, false, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, 0, 0, p.absmax, table); break;
	case INTERP_LINEAR * 2 + 1:  interp_table<INTERP_LINEAR, true, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, step, half, p.absmax, table); break;
	default:                     interp_table<INTERP_LINEAR, false, H><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, p.S, 0, 0, p.absmax, table); break;
	}
}

cudaError_t launch_das_table(const DasParams &p, float4 *table, cudaStream_t s)
{
	if (das_hercules_table_bytes(p) == 0) return cudaSuccess;
	if (!table || (p.half_table && !p.absmax)) return cudaErrorInvalidValue;
	const int64_t entries = (int64_t)p.C * p.T * p.S;
	const int64_t most = (int64_t)device_sm_count() * 16;
	const int blocks = (int)((entries + 255) / 256 < most ? (entries + 255) / 256 : most);
	if (p.half_table) {
		/* the scale: every sample the table reads, rf[0, min(readable, entries + 2)) */
		const int64_t n = p.rf_count < entries + 2 ? p.rf_count : entries + 2;
		cudaError_t e = cudaMemsetAsync(p.absmax, 0, sizeof(unsigned), s);
		if (e != cudaSuccess) return e;
		chan_absmax<<<blocks, 256, 0, s>>>(p.rf, n, p.absmax);
		g_kernel_launches++;
		launch_table<true>(p, entries, blocks, table, s);
	} else {
		launch_table<false>(p, entries, blocks, table, s);
	}
	g_kernel_launches++;
	return cudaGetLastError();
}

cudaError_t launch_das_hercules(const DasParams &p, float4 *table, cudaStream_t s)
{
	const int64_t n = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	if (n == 0) return cudaSuccess;
	if (!das_hercules_supported(p) || p.groups < 1 || (p.groups > 1 && !p.partial) || p.rx_step < 1 ||
	    (das_hercules_table_bytes(p) > 0 && !table) || (p.half_table && !p.absmax))
		return cudaErrorInvalidValue;
	if (das_hercules_table_bytes(p) > 0) {
		const cudaError_t e = launch_das_table(p, table, s);
		if (e != cudaSuccess) return e;
	}
	if (p.half_table) {
		if (p.dims[1] >= 4) launch_hercules_tiles<4, true>(p, table, s);
		else                launch_hercules_tiles<1, true>(p, table, s);
	} else {
		if (p.dims[1] >= 4) launch_hercules_tiles<4, false>(p, table, s);
		else                launch_hercules_tiles<1, false>(p, table, s);
	}
	g_kernel_launches++;
	if (p.groups > 1) {
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		return launch_das_reduce(p.partial, p.frame, n, p.groups, s);
	}
	return cudaGetLastError();
}

} /* namespace bf */
