/*
 * bf_das_hercules.cuh -- device code of the HERCULES delay-and-sum fast path
 * (see bf_das_hercules.cu): the term, the per-voxel set-up and range proof, the
 * column loop over receive channels and transmits, and one voxel tile.
 */
#pragma once
#include <cuda_fp16.h>
#include "bf_kernels.h"
#include "bf_das_math.cuh"

namespace bf {

/* Quotient x / b from the reciprocal rb = RN(1/b) and one correction FMA: equal
 * to IEEE division wherever launch_verify_division found it so (for the DAS
 * divisors: every |x| in [2^-100, 2^20]; x = 0 gives 0). */
__device__ __forceinline__ float div_rc(float x, float b, float rb)
{
	const float q = __fmul_rn(x, rb);
	const float r = fmaf(-q, b, x);
	return fmaf(r, rb, q);
}

/* cos^2(sqrt(w)) on [0, (pi/2)^2] as 1 + w q(w) with q of degree 4 (a weighted
 * least-squares fit iterated towards the minimax error; exact at w = 0, maximum
 * absolute error 6.4e-7 in FP32 Horner form, against 1e-7 for the squared Taylor
 * cosine of the general kernel): five FMAs. A weight enters the sum linearly, so
 * the error is below 1e-6 of the output. */
__device__ __forceinline__ float apod_cos2_p5(float w)
{
	float c = -1.12993468e-04f;
	c = fmaf(c, w, 3.10126483e-03f);
	c = fmaf(c, w, -4.43560816e-02f);
	c = fmaf(c, w, 3.33286583e-01f);
	c = fmaf(c, w, -9.99991953e-01f);
	return fmaf(c, w, 1.0f);
}

/* cos^2(sqrt(w)) on [0, (pi/2)^2] for DAS precision 1: (1 - w / (pi/2)^2)
 * (1 + a w + b w^2) expanded, a and b a weighted least-squares fit iterated towards
 * the minimax error; maximum absolute error 9.6e-4, 1.2e-7 at the aperture edge.
 * Three FMAs. */
__device__ __forceinline__ float apod_cos2_p3(float w)
{
	float c = -0.031044068f;
	c = fmaf(c, w, 0.31450406f);
	c = fmaf(c, w, -0.99229395f);
	return fmaf(c, w, 1.0f);
}

/* Table scale of DAS precision 1: the shift k with m 2^k in [1024, 2048) for the
 * largest channel-data component m (float bits); 0 when m is 0, below 2^-100,
 * above 2^100 or not a number. Each component of a cubic segment's coefficients
 * is at most 1, 1, 9 and 6 m before the rotation, so every rotated coefficient
 * and Horner partial sum is below 17 sqrt(2) m 2^k < 49300, inside FP16's
 * largest finite 65504. */
__device__ __forceinline__ int half_table_shift(unsigned m_bits)
{
	const float m = __uint_as_float(m_bits);
	if (!(m >= 0x1p-100f && m <= 0x1p100f)) return 0;
	const int e = (int)((m_bits >> 23) & 0xffu) - 126;   /* m = f 2^e, f in [1/2, 1) */
	return 11 - e;
}

__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

__device__ __forceinline__ __half2 as_half2(unsigned u)
{
	__half2 h;
	memcpy(&h, &u, sizeof(h));
	return h;
}

/* Precision 1: sample value of one term from the FP16 table at index ic (cubic
 * and linear: ic in [0, s_lim); nearest: round(ic) inside the row), and the
 * fraction the phase rotation needs. */
template <int INTERP>
__device__ __forceinline__ void sample_half(const float4 *__restrict__ tab, int row, float ic, float &f, float &vx,
                                            float &vy)
{
	float2 v;
	if (INTERP == INTERP_NEAREST) {
		const float r = roundf(ic);
		v = __half22float2(__ldg((const __half2 *)tab + (row + (int)r)));
		f = ic - r;
	} else {
		const int ii = (int)ic;
		f = ic - (float)ii;
		const __half2 f2 = __float2half2_rn(f);
		__half2 h;
		if (INTERP == INTERP_CUBIC) {
			const uint4 q = __ldg((const uint4 *)tab + (unsigned)(row + ii));
			h = __hfma2(as_half2(q.w), f2, as_half2(q.z));
			h = __hfma2(h, f2, as_half2(q.y));
			h = __hfma2(h, f2, as_half2(q.x));
		} else {
			const uint2 q = __ldg((const uint2 *)tab + (unsigned)(row + ii));
			h = __hfma2(as_half2(q.y), f2, as_half2(q.x));
		}
		v = __half22float2(h);
	}
	vx = v.x;
	vy = v.y;
}

/* The part of one (voxel, transmit t, receive r) term after the lateral distance:
 * lat2 = |lateral offset|^2 of the virtual element (r, t); row = (r * T + t) * S.
 * ROT: the table is rotated (DasParams::rot_table), the term by theta (f - 1/2)
 * only; ROT = 2 reduces that angle to [-pi, pi] first (|theta| > 2 pi).
 * INR: the voxel's proof that every sample index of its terms lies in [0, s_lim)
 * (HercVoxel::inrange): no range test; the apodization argument is clamped to the
 * aperture edge instead of tested, so a term just outside the aperture weighs the
 * polynomial's value at the edge (|p| < 5e-7) where the reference weighs
 * cos(pi/2)^2 = 2e-15. */
template <int INTERP, bool DEMOD, bool FASTMATH, int ROT, bool INR = false, bool H = false>
__device__ __forceinline__ void term_tail(const DasParams &p, const float4 *__restrict__ tab, float lat2, float dz2,
                                          float ka2, float dtx, float s_lim, int row, float scale, float &ax, float &ay)
{
	const float w    = INR ? fminf(ka2 * lat2, HALF_PI_SQ) : ka2 * lat2;
	const float x    = __fadd_rn(lat2, dz2);
	float idx;
	if (H) {
		/* precision 1: dtx carries the voxel's io = dtx fs_c + toff_fs */
		float drx;
		if (FASTMATH) {
			float r;
			asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
			drx = x * r;
		} else {
			drx = __fsqrt_rn(x);
		}
		idx = fmaf(drx, p.fs_c, dtx);
	} else {
		const float drx = FASTMATH ? sqrt_newton(x) : __fsqrt_rn(x);
		const float d   = __fadd_rn(dtx, drx);
		float tt = FASTMATH ? div_rc(d, p.c, p.rc) : __fdiv_rn(d, p.c);
		tt = __fadd_rn(tt, p.toff);
		idx = __fmul_rn(tt, p.fs);
	}
	const bool ok = INR || (idx >= 0.0f && idx < s_lim && w < HALF_PI_SQ);
	const float a  = ok ? (H ? apod_cos2_p3(w) : apod_cos2_p5(w)) * scale : 0.0f;
	const float ic = ok ? idx : 1.0f;
	float vx, vy, f = 0.0f;
	if (H && INTERP == INTERP_NEAREST && !INR) {
		/* FP16 table, nearest outside the proof: round(idx) may be the sample
		 * after the last row's end, which reads 0 */
		const float r = roundf(ic);
		const int j = row + (int)r;
		const int last = p.C * p.T * p.S - 1;
		const float2 v = __half22float2(__ldg((const __half2 *)tab + min(j, last)));
		vx = j <= last ? v.x : 0.0f;
		vy = j <= last ? v.y : 0.0f;
		f = ic - r;
	} else if (H) {
		sample_half<INTERP>(tab, row, ic, f, vx, vy);
	} else if (INTERP == INTERP_NEAREST && INR) {
		/* round(idx) proven inside the row: no bound check; with ROT the sample
		 * comes pre-rotated by its phase from the table (float2 per sample) */
		const float r = roundf(ic);
		const int j = row + (int)r;
		const float2 v = ROT != 0 ? __ldg((const float2 *)tab + j) : __ldg(p.rf + j);
		vx = v.x;
		vy = v.y;
		f = ic - r;                                         /* in [-1/2, 1/2] */
	} else if (INTERP == INTERP_NEAREST) {
		const int j = row + (int)roundf(ic);
		const int last = (int)p.rf_count - 1;
		float2 v = __ldg(p.rf + min(j, last));
		vx = j > last ? 0.0f : v.x;
		vy = j > last ? 0.0f : v.y;
	} else {
		const int ii = (int)ic;
		f = ic - (float)ii;
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
		float sn, cs;
		if (ROT != 0 && (INTERP != INTERP_NEAREST || INR || H)) {
			/* table interpolation: theta (f - 1/2); nearest: theta (idx - round(idx)) */
			float a = INTERP == INTERP_NEAREST ? __fmul_rn(p.theta, f) : fmaf(p.theta, f, -p.theta_half);
			if (ROT == 2) {
				/* two-constant split of 2 pi: off by at most |k| * 1.1e-11 rad */
				const float k = rintf(a * 0.159154943f);
				a = fmaf(-k, 6.28125f, a);
				a = fmaf(-k, 0x1.fb5444p-10f, a);
			}
			__sincosf(a, &sn, &cs);
		} else {
			const float time = FASTMATH ? div_rc(ic, p.fs, p.rfs) : __fdiv_rn(ic, p.fs);
			const float arg  = __fmul_rn(p.r360_fc, time);
			const float k = rintf(arg * 0.159154943f);
			float rr = fmaf(-k, 6.28125f, arg);
			rr = fmaf(-k, 0x1.fb5444p-10f, rr);
			__sincosf(rr, &sn, &cs);
		}
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
	float io;               /* precision 1: dtx fs_c + toff_fs, the index offset */
	bool  fast;             /* every term inside the verified fast-math ranges */
	bool  inrange;          /* every term's sample index inside [0, S - 2) (cubic), [0, S - 1) (linear), [0, S - 1/2) (nearest) */
};

__device__ __forceinline__ HercVoxel hercules_setup(const DasParams &p, int vx, int vy, int vz)
{
	HercVoxel v;
	float w[3], q[3];
	m4v(p.M, (float)vx, (float)vy, (float)vz, w);
	m4v(p.X, w[0], w[1], w[2], q);
	v.dz2 = __fmul_rn(q[2], q[2]);
	v.dtx = transmit_distance(p, w, 0);
	v.io = fmaf(v.dtx, p.fs_c, p.toff_fs);
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
	/* distance d = dtx + sqrt(lat2 + dz2) lies in [dtx + sqrt(dz2), dtx + sqrt(xmax)]
	 * and idx = (d / c + toff) fs grows with d; the margins (1e-4 relative, 0.01
	 * samples) cover the roundings of the term's chain and of these bounds */
	const float dmin = v.dtx + sqrtf(v.dz2) * 0.9999f, dmax = v.dtx + sqrtf(xmax) * 1.0001f;
	const float imin = (dmin / p.c + p.toff) * p.fs, imax = (dmax / p.c + p.toff) * p.fs;
	/* nearest: round(idx) <= S - 1 needs idx < S - 1/2 */
	const float s_lim = p.interp == INTERP_CUBIC ? (float)(p.S - 2) : p.interp == INTERP_LINEAR ? (float)(p.S - 1)
	                                                                                         : (float)p.S - 0.5f;
	/* precision 1 forms the index as sqrt(x) fs_c + io: its rounding and the
	 * approximate reciprocal square root (relative error < 2^-22) stay below
	 * 4e-6 of the magnitudes summed */
	const float hm = p.half_table ? 4e-6f * (fabsf(v.io) + fabsf(p.toff_fs) + sqrtf(xmax) * 1.0001f * fabsf(p.fs_c))
	                              : 0.0f;
	v.inrange = p.c > 0.0f && p.fs > 0.0f && imin - fabsf(imin) * 1e-4f - hm >= 0.01f &&
	            imax + fabsf(imax) * 1e-4f + hm + 0.01f < s_lim;
	return v;
}

/* Sum over receive channels [u_begin, u_end) of the channel's transmit sum, for
 * NV voxels that share their lateral coordinates (NV = 2: two depths of one
 * column). The transmit interval is the widest of the voxels' (the deepest:
 * the aperture grows with depth); a voxel's terms outside its own interval weigh
 * exactly 0, so each voxel's sums equal its own loop's bit for bit. */
template <int INTERP, bool DEMOD, bool FASTMATH, int ROT, int NV, bool INR = false, bool H = false>
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
	for (int r = u_begin; r < u_end; r += p.rx_step) {
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
				term_tail<INTERP, DEMOD, FASTMATH, ROT, INR, H>(p, tab, lat2, v[k].dz2, v[k].ka2, H ? v[k].io : v[k].dtx,
				                                                s_lim, row, p.inv_sqrt_T, ax[k], ay[k]);
			t_lo = 1;
			row += p.S;
		}
		float tf = (float)t_lo;
		/* two transmits per iteration keep two table loads in flight per voxel
		 * (87.5 against 90.5 ms per 128 x 128 x 256 cubic frame; 3 or 4, or fewer
		 * registers for more blocks per SM, measured slower) */
		#pragma unroll 2
		for (int t = t_lo; t <= t_hi; t++) {
			const float dv = __fsub_rn(q_var, __fmul_rn(tf, pitch_var));
			const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
			#pragma unroll
			for (int k = 0; k < NV; k++)
				term_tail<INTERP, DEMOD, FASTMATH, ROT, INR, H>(p, tab, lat2, v[k].dz2, v[k].ka2, H ? v[k].io : v[k].dtx,
				                                                s_lim, row, 1.0f, ax[k], ay[k]);
			tf += 1.0f;
			row += p.S;
		}
		#pragma unroll
		for (int k = 0; k < NV; k++) { sx[k] += ax[k]; sy[k] += ay[k]; }
	}
}

/* Precision 1, one transmit of two depths of a column (the float2 lanes are the
 * two voxels) whose sample indices are proven in range: the per-voxel arithmetic
 * of term_tail<..., INR, H> in packed FP32 (per component the same IEEE
 * operations as its scalar form; the caller forms the lateral distance with
 * FMAs). ROT != 0 or !DEMOD. */
template <int INTERP, bool DEMOD, int ROT>
__device__ __forceinline__ void term_h2(const DasParams &p, const float4 *__restrict__ tab, float lat2, float2 dz2,
                                        float2 ka2, float2 io, int row, float scale, float2 &ax, float2 &ay)
{
	const float2 l2 = make_float2(lat2, lat2);
	float2 w = __fmul2_rn(ka2, l2);
	w.x = fminf(w.x, HALF_PI_SQ);
	w.y = fminf(w.y, HALF_PI_SQ);
	const float2 x = __fadd2_rn(l2, dz2);
	float r0, r1;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x.x));
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(x.y));
	const float2 idx = __ffma2_rn(__fmul2_rn(x, make_float2(r0, r1)), make_float2(p.fs_c, p.fs_c), io);
	/* apod_cos2_p3 on both voxels */
	float2 a = __ffma2_rn(make_float2(-0.031044068f, -0.031044068f), w, make_float2(0.31450406f, 0.31450406f));
	a = __ffma2_rn(a, w, make_float2(-0.99229395f, -0.99229395f));
	a = __ffma2_rn(a, w, make_float2(1.0f, 1.0f));
	if (scale != 1.0f) a = __fmul2_rn(a, make_float2(scale, scale));
	float2 f, vx, vy;
	sample_half<INTERP>(tab, row, idx.x, f.x, vx.x, vy.x);
	sample_half<INTERP>(tab, row, idx.y, f.y, vx.y, vy.y);
	if (DEMOD) {
		float2 ang = INTERP == INTERP_NEAREST ? __fmul2_rn(make_float2(p.theta, p.theta), f)
		                                      : __ffma2_rn(make_float2(p.theta, p.theta), f,
		                                                   make_float2(-p.theta_half, -p.theta_half));
		if (ROT == 2) {
			const float2 k = make_float2(-rintf(ang.x * 0.159154943f), -rintf(ang.y * 0.159154943f));
			ang = __ffma2_rn(k, make_float2(6.28125f, 6.28125f), ang);
			ang = __ffma2_rn(k, make_float2(0x1.fb5444p-10f, 0x1.fb5444p-10f), ang);
		}
		float2 sn, cs;
		__sincosf(ang.x, &sn.x, &cs.x);
		__sincosf(ang.y, &sn.y, &cs.y);
		const float2 ca = __fmul2_rn(a, cs), sa = __fmul2_rn(a, sn);
		ax = __ffma2_rn(ca, vx, __ffma2_rn(make_float2(-sa.x, -sa.y), vy, ax));
		ay = __ffma2_rn(sa, vx, __ffma2_rn(ca, vy, ay));
	} else {
		ax = __ffma2_rn(a, vx, ax);
		ay = __ffma2_rn(a, vy, ay);
	}
}

/* Precision 1, NV = 2 voxels proven in range: hercules_column with term_h2; the
 * lateral offset of a transmit is one FMA (q - t pitch) and its square plus the
 * fixed offset's another. */
template <int INTERP, bool DEMOD, int ROT>
__device__ __forceinline__ void hercules_column_h2(const DasParams &p, const float4 *__restrict__ tab, const HercVoxel *v,
                                                   int u_begin, int u_end, float *sx, float *sy)
{
	const float pitch_fix = p.rx_cols ? p.px : p.py, pitch_var = p.rx_cols ? p.py : p.px;
	const float q_fix = v[0].q_fix, q_var = v[0].q_var;
	const float lim2 = fmaxf(v[0].lim2, v[1].lim2);
	const float2 dz2 = make_float2(v[0].dz2, v[1].dz2), ka2 = make_float2(v[0].ka2, v[1].ka2);
	const float2 io = make_float2(v[0].io, v[1].io);
	for (int r = u_begin; r < u_end; r += p.rx_step) {
		const float df = fmaf(-(float)r, pitch_fix, q_fix);
		const float f2 = df * df;
		int t_lo, t_hi;
		aperture_interval(q_var, pitch_var, lim2 - f2, p.T, t_lo, t_hi);
		if (t_lo > t_hi) continue;
		float2 ax = make_float2(0.0f, 0.0f), ay = make_float2(0.0f, 0.0f);
		int row = (r * p.T + t_lo) * p.S;
		if (t_lo == 0) {
			term_h2<INTERP, DEMOD, ROT>(p, tab, fmaf(q_var, q_var, f2), dz2, ka2, io, row, p.inv_sqrt_T, ax, ay);
			t_lo = 1;
			row += p.S;
		}
		float tf = (float)t_lo;
		#pragma unroll 2
		for (int t = t_lo; t <= t_hi; t++) {
			const float dv = fmaf(-tf, pitch_var, q_var);
			term_h2<INTERP, DEMOD, ROT>(p, tab, fmaf(dv, dv, f2), dz2, ka2, io, row, 1.0f, ax, ay);
			tf += 1.0f;
			row += p.S;
		}
		sx[0] += ax.x;
		sx[1] += ax.y;
		sy[0] += ay.x;
		sy[1] += ay.y;
	}
}

/* One voxel on its own, with the fast or the IEEE square root and divisions (and,
 * where its sample indices are proven in range, without per-term range tests). */
template <int INTERP, bool H = false>
__device__ __forceinline__ void hercules_single(const DasParams &p, const float4 *__restrict__ tab, const HercVoxel &v,
                                             int u_begin, int u_end, float &sx, float &sy)
{
	const bool demod = p.fc > 0.0f;
	const int rot = p.rot_table;
	if (v.fast && v.inrange) {
		if (demod && rot == 1)      hercules_column<INTERP, true, true, 1, 1, true, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod && rot == 2) hercules_column<INTERP, true, true, 2, 1, true, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod)             hercules_column<INTERP, true, true, 0, 1, true, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else                        hercules_column<INTERP, false, true, 0, 1, true, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
	} else if (v.fast) {
		if (demod && rot == 1)      hercules_column<INTERP, true, true, 1, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod && rot == 2) hercules_column<INTERP, true, true, 2, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod)             hercules_column<INTERP, true, true, 0, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else                        hercules_column<INTERP, false, true, 0, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
	} else {
		if (demod && rot == 1)      hercules_column<INTERP, true, false, 1, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod && rot == 2) hercules_column<INTERP, true, false, 2, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else if (demod)             hercules_column<INTERP, true, false, 0, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
		else                        hercules_column<INTERP, false, false, 0, 1, false, H>(p, tab, &v, u_begin, u_end, &sx, &sy);
	}
}

/* Voxel tiles of a block (128 threads). Volumes: threads 4 x 4 x 8, each thread
 * two adjacent depths, so a block covers 4 x 4 x 16 voxels and a warp 4 x 4 x 4.
 * Planes: threads 8 x 1 x 16, one voxel each. The sample delay moves by ~1.3
 * samples per axial voxel step and by at most ~0.3 per lateral step inside the
 * aperture, so the compact 3D warp reads the fewest distinct table entries per
 * term; the spread of the transmit intervals across its lanes is ~3 elements. */
template <int TY, int THREADS = 128> struct HercTile {
	static constexpr int X = TY == 1 ? 8 : 4, Y = TY, Z = THREADS / (X * TY), NV = TY == 1 ? 1 : 2;
};

/* Thread threadIdx.x of voxel tile (bx, yt, bz), outer-loop group grp: the
 * work of one das_hercules block, also run by the batched launch. */
template <int INTERP, int TY, int THREADS = 128, bool H = false>
__device__ __forceinline__ void hercules_tile(const DasParams &p, const float4 *__restrict__ tab, int bx, int yt, int bz,
                                              int grp)
{
	using Tile = HercTile<TY, THREADS>;
	constexpr int NV = Tile::NV;
	const int vx = bx * Tile::X + (int)(threadIdx.x % Tile::X);
	const int vy = yt * Tile::Y + (int)((threadIdx.x / Tile::X) % Tile::Y);
	const int vz0 = (bz * Tile::Z + (int)(threadIdx.x / (Tile::X * Tile::Y))) * NV;
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
		const int rot = p.rot_table;
		bool inr = true;
		#pragma unroll
		for (int k = 0; k < NV; k++) inr = inr && v[k].inrange;
		if (H && NV == 2 && inr && (rot != 0 || !demod)) {
			if (demod && rot == 1)      hercules_column_h2<INTERP, true, 1>(p, tab, v, u_begin, u_end, sx, sy);
			else if (demod)             hercules_column_h2<INTERP, true, 2>(p, tab, v, u_begin, u_end, sx, sy);
			else                        hercules_column_h2<INTERP, false, 0>(p, tab, v, u_begin, u_end, sx, sy);
		} else if (inr) {
			if (demod && rot == 1)      hercules_column<INTERP, true, true, 1, NV, true, H>(p, tab, v, u_begin, u_end, sx, sy);
			else if (demod && rot == 2) hercules_column<INTERP, true, true, 2, NV, true, H>(p, tab, v, u_begin, u_end, sx, sy);
			else if (demod)             hercules_column<INTERP, true, true, 0, NV, true, H>(p, tab, v, u_begin, u_end, sx, sy);
			else                        hercules_column<INTERP, false, true, 0, NV, true, H>(p, tab, v, u_begin, u_end, sx, sy);
		} else {
			if (demod && rot == 1)      hercules_column<INTERP, true, true, 1, NV, false, H>(p, tab, v, u_begin, u_end, sx, sy);
			else if (demod && rot == 2) hercules_column<INTERP, true, true, 2, NV, false, H>(p, tab, v, u_begin, u_end, sx, sy);
			else if (demod)             hercules_column<INTERP, true, true, 0, NV, false, H>(p, tab, v, u_begin, u_end, sx, sy);
			else                        hercules_column<INTERP, false, true, 0, NV, false, H>(p, tab, v, u_begin, u_end, sx, sy);
		}
	} else {
		#pragma unroll
		for (int k = 0; k < NV; k++)
			if (k < nv) hercules_single<INTERP, H>(p, tab, v[k], u_begin, u_end, sx[k], sy[k]);
	}
	if (H) {
		/* undo the table's power-of-two scale (exact) */
		const float us = pow2f(-half_table_shift(__ldg(p.absmax)));
		#pragma unroll
		for (int k = 0; k < NV; k++) { sx[k] *= us; sy[k] *= us; }
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

} /* namespace bf */
