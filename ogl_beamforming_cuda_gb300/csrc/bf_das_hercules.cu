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
 *   - The phase reduction drops the third Cody-Waite constant: with the
 *     two-constant split of 2 pi (6.28125 exact in 8 bits, the rest rounded to
 *     float) the reduced angle is off by at most |k| * 1.1e-11 rad, k < 2^15.
 *
 * Sample indices stay bit-equal to the reference's: the delay chain is the same
 * sequence of round-to-nearest operations as das_kernel's.
 */
#include "bf_kernels.h"
#include "bf_das_math.cuh"

namespace bf {

/* Interpolation tables, one entry per flat channel-data index n < entries
 * (samples outside [0, readable) read as 0, as the reference's bounded reads do).
 * Cubic (das.glsl:36-62): with P1 = s[n], P2 = s[n+1], T1 = (s[n+1] - s[n-1]) / 2,
 * T2 = (s[n+2] - s[n]) / 2 the segment is a0 + a1 f + a2 f^2 + a3 f^3 with
 * a0 = P1, a1 = T1, a2 = 3 (P2 - P1) - 2 T1 - T2, a3 = 2 (P1 - P2) + T1 + T2;
 * stored as float4 (a0, a1) and float4 (a2, a3), complex pairs.
 * Linear: float4 (s[n], s[n+1] - s[n]). */
template <int INTERP>
__global__ void __launch_bounds__(256)
interp_table(const float2 *__restrict__ rf, int64_t entries, int64_t readable, float4 *__restrict__ out)
{
	const float2 zero = make_float2(0.0f, 0.0f);
	for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < entries; n += (int64_t)gridDim.x * blockDim.x) {
		const float2 s1 = n < readable ? rf[n] : zero;
		const float2 s2 = n + 1 < readable ? rf[n + 1] : zero;
		if (INTERP == INTERP_LINEAR) {
			out[n] = make_float4(s1.x, s1.y, s2.x - s1.x, s2.y - s1.y);
			continue;
		}
		const float2 s0 = n > 0 && n - 1 < readable ? rf[n - 1] : zero;
		const float2 s3 = n + 2 < readable ? rf[n + 2] : zero;
		const float t1x = 0.5f * (s2.x - s0.x), t1y = 0.5f * (s2.y - s0.y);
		const float t2x = 0.5f * (s3.x - s1.x), t2y = 0.5f * (s3.y - s1.y);
		const float dx = s2.x - s1.x, dy = s2.y - s1.y;
		out[2 * n]     = make_float4(s1.x, s1.y, t1x, t1y);
		out[2 * n + 1] = make_float4(3.0f * dx - 2.0f * t1x - t2x, 3.0f * dy - 2.0f * t1y - t2y,
		                             t1x + t2x - 2.0f * dx, t1y + t2y - 2.0f * dy);
	}
}

/* Quotient x / b from the reciprocal rb = RN(1/b) and one correction FMA: equal
 * to IEEE division wherever launch_verify_division found it so (for the DAS
 * divisors: every |x| in [2^-100, 2^20]; x = 0 gives 0). */
__device__ __forceinline__ float div_rc(float x, float b, float rb)
{
	const float q = __fmul_rn(x, rb);
	const float r = fmaf(-q, b, x);
	return fmaf(r, rb, q);
}

/* The part of one (voxel, transmit t, receive r) term after the lateral distance:
 * lat2 = |lateral offset|^2 of the virtual element (r, t); row = (r * T + t) * S. */
template <int INTERP, bool DEMOD, bool FASTMATH>
__device__ __forceinline__ void term_tail(const DasParams &p, const float4 *__restrict__ tab, float lat2, float dz2,
                                          float ka2, float dtx, float s_lim, int row, float scale, float &ax, float &ay)
{
	const float w    = ka2 * lat2;
	const float x    = __fadd_rn(lat2, dz2);
	const float drx  = FASTMATH ? sqrt_newton(x) : __fsqrt_rn(x);
	const float d    = __fadd_rn(dtx, drx);
	float tt = FASTMATH ? div_rc(d, p.c, p.rc) : __fdiv_rn(d, p.c);
	tt = __fadd_rn(tt, p.toff);
	const float idx = __fmul_rn(tt, p.fs);
	const bool ok = idx >= 0.0f && idx < s_lim && w < HALF_PI_SQ;
	const float a  = ok ? apod_cos2(w) * scale : 0.0f;
	const float ic = ok ? idx : 1.0f;
	float vx, vy;
	if (INTERP == INTERP_NEAREST) {
		const int j = row + (int)roundf(ic);
		const int last = (int)p.rf_count - 1;
		float2 v = __ldg(p.rf + min(j, last));
		vx = j > last ? 0.0f : v.x;
		vy = j > last ? 0.0f : v.y;
	} else {
		const int ii = (int)ic;
		const float f = ic - (float)ii;
		if (INTERP == INTERP_CUBIC) {
			/* one 32-byte load of the segment (the table is 32-byte aligned) */
			const float4 *cp = tab + 2 * (size_t)(unsigned)(row + ii);
			float a0x, a0y, a1x, a1y, a2x, a2y, a3x, a3y;
			asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
			    : "=f"(a0x), "=f"(a0y), "=f"(a1x), "=f"(a1y), "=f"(a2x), "=f"(a2y), "=f"(a3x), "=f"(a3y) : "l"(cp));
			vx = fmaf(fmaf(fmaf(a3x, f, a2x), f, a1x), f, a0x);
			vy = fmaf(fmaf(fmaf(a3y, f, a2y), f, a1y), f, a0y);
		} else {
			const float4 c = __ldg(tab + (size_t)(unsigned)(row + ii));
			vx = fmaf(c.z, f, c.x);
			vy = fmaf(c.w, f, c.y);
		}
	}
	if (DEMOD) {
		const float time = FASTMATH ? div_rc(ic, p.fs, p.rfs) : __fdiv_rn(ic, p.fs);
		const float arg  = __fmul_rn(p.r360_fc, time);
		const float k = rintf(arg * 0.159154943f);
		float rr = fmaf(-k, 6.28125f, arg);
		rr = fmaf(-k, 0x1.fb5444p-10f, rr);
		float sn, cs;
		__sincosf(rr, &sn, &cs);
		const float ca = a * cs, sa = a * sn;
		ax = fmaf(ca, vx, fmaf(-sa, vy, ax));
		ay = fmaf(sa, vx, fmaf(ca, vy, ay));
	} else {
		ax = fmaf(a, vx, ax);
		ay = fmaf(a, vy, ay);
	}
}

/* Per-voxel constants of the term loop. */
struct HercVoxel {
	float q_fix, q_var;     /* lateral coordinates fixed by r and varied by t */
	float dz2, dtx, ka2, lim2;
	bool  fast;             /* every term inside the verified fast-math ranges */
};

__device__ __forceinline__ HercVoxel hercules_setup(const DasParams &p, int vx, int vy, int vz)
{
	HercVoxel v;
	float w[3], q[3];
	m4v(p.M, (float)vx, (float)vy, (float)vz, w);
	m4v(p.X, w[0], w[1], w[2], q);
	v.dz2 = __fmul_rn(q[2], q[2]);
	v.dtx = transmit_distance(p, w, 0);
	const float ka = __fdiv_rn(p.apod_scale, fabsf(q[2]));
	v.ka2 = ka * ka;
	v.lim2 = HALF_PI_SQ / v.ka2;
	/* receive channel r fixes one lateral coordinate, transmit t the other */
	v.q_fix = p.rx_cols ? q[0] : q[1];
	v.q_var = p.rx_cols ? q[1] : q[0];
	const float pitch_fix = p.rx_cols ? p.px : p.py, pitch_var = p.rx_cols ? p.py : p.px;
	/* Bounds over all (r, t): the lateral offsets are linear in r and t, so their
	 * largest magnitudes sit at the first or last element; the square-root argument
	 * lies in [dz2, xmax] and |d| <= |dtx| + sqrt(xmax) (margins cover rounding). */
	const float fa = fabsf(v.q_fix), fb = fabsf(v.q_fix - (float)(p.C - 1) * pitch_fix);
	const float va = fabsf(v.q_var), vb = fabsf(v.q_var - (float)(p.T - 1) * pitch_var);
	const float fm = fmaxf(fa, fb), vm = fmaxf(va, vb);
	const float xmax = (fm * fm + vm * vm + v.dz2) * 1.0001f;
	v.fast = p.fast_sqrt && v.dz2 >= p.sqrt_lo && xmax <= p.sqrt_hi &&
	         fabsf(v.dtx) + sqrtf(xmax) * 1.0001f <= p.c_hi && p.c_lo <= 0x1p-100f &&
	         p.fs_lo <= 0x1p-100f && (float)p.S <= p.fs_hi;
	return v;
}

/* Sum over receive channels [u_begin, u_end) of the channel's transmit sum, for
 * NV voxels that share their lateral coordinates (NV = 2: two depths of one
 * column). The transmit interval is the widest of the voxels' (the deepest:
 * the aperture grows with depth); a voxel's terms outside its own interval weigh
 * exactly 0, so each voxel's sums equal its own loop's bit for bit. */
template <int INTERP, bool DEMOD, bool FASTMATH, int NV>
__device__ __forceinline__ void hercules_column(const DasParams &p, const float4 *__restrict__ tab, const HercVoxel *v,
                                                int u_begin, int u_end, float *sx, float *sy)
{
	constexpr int extra = INTERP == INTERP_CUBIC ? 2 : INTERP == INTERP_LINEAR ? 1 : 0;
	const float s_lim = (float)(p.S - extra);
	const float pitch_fix = p.rx_cols ? p.px : p.py, pitch_var = p.rx_cols ? p.py : p.px;
	const float q_fix = v[0].q_fix, q_var = v[0].q_var;
	float lim2 = v[0].lim2;
	#pragma unroll
	for (int k = 1; k < NV; k++) lim2 = fmaxf(lim2, v[k].lim2);
	for (int r = u_begin; r < u_end; r++) {
		const float df = __fsub_rn(q_fix, __fmul_rn((float)r, pitch_fix));
		const float f2 = __fmul_rn(df, df);
		int t_lo, t_hi;
		aperture_interval(q_var, pitch_var, lim2 - f2, p.T, t_lo, t_hi);
		if (t_lo > t_hi) continue;
		float ax[NV], ay[NV];
		#pragma unroll
		for (int k = 0; k < NV; k++) ax[k] = ay[k] = 0.0f;
		int row = (r * p.T + t_lo) * p.S;
		if (t_lo == 0) {
			/* element 0 sits at 0: dv = q_var - 0 * pitch */
			const float dv = __fsub_rn(q_var, __fmul_rn(0.0f, pitch_var));
			const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
			#pragma unroll
			for (int k = 0; k < NV; k++)
				term_tail<INTERP, DEMOD, FASTMATH>(p, tab, lat2, v[k].dz2, v[k].ka2, v[k].dtx, s_lim, row, p.inv_sqrt_T,
				                                   ax[k], ay[k]);
			t_lo = 1;
			row += p.S;
		}
		float tf = (float)t_lo;
		#pragma unroll (3 - NV)
		for (int t = t_lo; t <= t_hi; t++) {
			const float dv = __fsub_rn(q_var, __fmul_rn(tf, pitch_var));
			const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
			#pragma unroll
			for (int k = 0; k < NV; k++)
				term_tail<INTERP, DEMOD, FASTMATH>(p, tab, lat2, v[k].dz2, v[k].ka2, v[k].dtx, s_lim, row, 1.0f,
				                                   ax[k], ay[k]);
			tf += 1.0f;
			row += p.S;
		}
		#pragma unroll
		for (int k = 0; k < NV; k++) { sx[k] += ax[k]; sy[k] += ay[k]; }
	}
}

/* One voxel on its own, with the fast or the IEEE square root and divisions. */
template <int INTERP>
__device__ __forceinline__ void hercules_single(const DasParams &p, const float4 *__restrict__ tab, const HercVoxel &v,
                                             int u_begin, int u_end, float &sx, float &sy)
{
	const bool demod = p.fc > 0.0f;
	if (v.fast) {
		if (demod) hercules_column<INTERP, true, true, 1>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else       hercules_column<INTERP, false, true, 1>(p, tab, &v, u_begin, u_end, &sx, &sy);
	} else {
		if (demod) hercules_column<INTERP, true, false, 1>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else       hercules_column<INTERP, false, false, 1>(p, tab, &v, u_begin, u_end, &sx, &sy);
	}
}

/* Voxel tiles of a block (128 threads). Volumes: threads 4 x 4 x 8, each thread
 * two adjacent depths, so a block covers 4 x 4 x 16 voxels and a warp 4 x 4 x 4.
 * Planes: threads 8 x 1 x 16, one voxel each. The sample delay moves by ~1.3
 * samples per axial voxel step and by at most ~0.3 per lateral step inside the
 * aperture, so the compact 3D warp reads the fewest distinct table entries per
 * term; the spread of the transmit intervals across its lanes is ~3 elements. */
template <int TY> struct HercTile {
	static constexpr int X = TY == 1 ? 8 : 4, Y = TY, Z = 128 / (X * TY), NV = TY == 1 ? 1 : 2;
};

template <int INTERP, int TY>
__global__ void __launch_bounds__(DAS_THREADS, TY == 1 ? 8 : 6)
das_hercules(DasParams p, const float4 *__restrict__ tab)
{
	using Tile = HercTile<TY>;
	constexpr int NV = Tile::NV;
	const int ytiles = blockIdx.y / p.groups;
	const int grp = blockIdx.y - ytiles * p.groups;
	const int vx = blockIdx.x * Tile::X + (int)(threadIdx.x % Tile::X);
	const int vy = ytiles * Tile::Y + (int)((threadIdx.x / Tile::X) % Tile::Y);
	const int vz0 = (blockIdx.z * Tile::Z + (int)(threadIdx.x / (Tile::X * Tile::Y))) * NV;
	if (vx >= p.dims[0] || vy >= p.dims[1] || vz0 >= p.dims[2]) return;
	const int u_begin = grp * p.per_group;
	const int u_end   = min(p.loop_end, u_begin + p.per_group);

	HercVoxel v[NV] = {};
	float sx[NV], sy[NV];
	int nv = 0;
	#pragma unroll
	for (int k = 0; k < NV; k++) {
		sx[k] = sy[k] = 0.0f;
		if (vz0 + k < p.dims[2]) { v[k] = hercules_setup(p, vx, vy, vz0 + k); nv = k + 1; }
	}
	bool together = nv == NV;
	bool fast = v[0].fast;
	#pragma unroll
	for (int k = 1; k < NV; k++) {
		together = together && v[k].q_fix == v[0].q_fix && v[k].q_var == v[0].q_var;
		fast = fast && v[k].fast;
	}
	if (NV > 1 && together && fast) {
		const bool demod = p.fc > 0.0f;
		if (demod) hercules_column<INTERP, true, true, NV>(p, tab, v, u_begin, u_end, sx, sy);
		else       hercules_column<INTERP, false, true, NV>(p, tab, v, u_begin, u_end, sx, sy);
	} else {
		#pragma unroll
		for (int k = 0; k < NV; k++)
			if (k < nv) hercules_single<INTERP>(p, tab, v[k], u_begin, u_end, sx[k], sy[k]);
	}

	const int64_t nvox = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	#pragma unroll
	for (int k = 0; k < NV; k++) {
		if (k >= nv) break;
		const int64_t o = ((int64_t)(vz0 + k) * p.dims[1] + vy) * p.dims[0] + vx;
		if (p.groups > 1) p.partial[grp * nvox + o] = make_float2(sx[k], sy[k]);
		else              p.frame[o] = make_float2(sx[k], sy[k]);
	}
}

int64_t das_hercules_table_entries(const DasParams &p)
{
	const int64_t n = (int64_t)p.C * p.T * p.S;
	return p.interp == INTERP_CUBIC ? 2 * n : p.interp == INTERP_LINEAR ? n : 0;
}

bool das_hercules_supported(const DasParams &p)
{
	return p.family == DAS_HERCULES && p.fast && !p.sparse_mode && !p.coherency && p.dense_rows &&
	       p.rf_count >= (int64_t)p.C * p.T * p.S && p.loop_end == p.C;
}

template <int TY>
static void launch_hercules_tiles(const DasParams &p, const float4 *table, cudaStream_t s)
{
	using Tile = HercTile<TY>;
	dim3 grid((p.dims[0] + Tile::X - 1) / Tile::X, ((p.dims[1] + Tile::Y - 1) / Tile::Y) * p.groups,
	          (p.dims[2] + Tile::Z * Tile::NV - 1) / (Tile::Z * Tile::NV));
	switch (p.interp) {
	case INTERP_CUBIC:  das_hercules<INTERP_CUBIC, TY><<<grid, DAS_THREADS, 0, s>>>(p, table); break;
	case INTERP_LINEAR: das_hercules<INTERP_LINEAR, TY><<<grid, DAS_THREADS, 0, s>>>(p, table); break;
	default:            das_hercules<INTERP_NEAREST, TY><<<grid, DAS_THREADS, 0, s>>>(p, table); break;
	}
}

cudaError_t launch_das_hercules(const DasParams &p, float4 *table, cudaStream_t s)
{
	const int64_t n = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	if (n == 0) return cudaSuccess;
	if (!das_hercules_supported(p) || p.groups < 1 || (p.groups > 1 && !p.partial) ||
	    (p.interp != INTERP_NEAREST && !table))
		return cudaErrorInvalidValue;
	if (p.interp != INTERP_NEAREST) {
		const int64_t entries = (int64_t)p.C * p.T * p.S;
		const int blocks = (int)((entries + 255) / 256 < 152 * 16 ? (entries + 255) / 256 : 152 * 16);
		if (p.interp == INTERP_CUBIC) interp_table<INTERP_CUBIC><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, table);
		else                          interp_table<INTERP_LINEAR><<<blocks, 256, 0, s>>>(p.rf, entries, p.rf_count, table);
		g_kernel_launches++;
	}
	if (p.dims[1] >= 4) launch_hercules_tiles<4>(p, table, s);
	else                launch_hercules_tiles<1>(p, table, s);
	g_kernel_launches++;
	if (p.groups > 1) {
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		return launch_das_reduce(p.partial, p.frame, n, p.groups, s);
	}
	return cudaGetLastError();
}

} /* namespace bf */
