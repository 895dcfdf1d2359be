/*
 * bf_das_forces.cuh -- device code of the FORCES delay-and-sum fast path
 * (das.glsl:259-277), shared by das_forces (bf_das_forces.cu) and the batched
 * launch (bf_das_batch.cu); see bf_das_forces.cu for the method.
 */
#pragma once
#include "bf_kernels.h"
#include "bf_das_math.cuh"
#include "bf_das_generic.cuh"
#include "bf_das_hercules.cuh"

namespace bf {

/* one FORCES term from the table, its index idx proven in [0, s_lim): the
 * segment at floor(idx) times a, rotated by theta (f - 1/2) (ROT 2: reduced) */
template <int INTERP, bool DEMOD, int ROT>
__device__ __forceinline__ void forces_table_term(const DasParams &p, const float4 *__restrict__ tab, int row,
                                                  float idx, float a, float &ax, float &ay)
{
	const int ii = (int)idx;
	const float f = idx - (float)ii;
	float vx, vy;
	if (INTERP == INTERP_CUBIC) {
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
	if (DEMOD) {
		float an = fmaf(p.theta, f, -p.theta_half);
		if (ROT == 2) {
			const float k = rintf(an * 0.159154943f);
			an = fmaf(-k, 6.28125f, an);
			an = fmaf(-k, 0x1.fb5444p-10f, an);
		}
		float sn, cs;
		__sincosf(an, &sn, &cs);
		const float ca = a * cs, sa = a * sn;
		ax = fmaf(ca, vx, fmaf(-sa, vy, ax));
		ay = fmaf(sa, vx, fmaf(ca, vy, ay));
	} else {
		ax = fmaf(a, vx, ax);
		ay = fmaf(a, vy, ay);
	}
}

/* The fast loop of one proven voxel over receive channels [u_begin, u_end). */
template <int INTERP, bool DEMOD, int ROT>
__device__ __forceinline__ float2 forces_voxel_fast(const DasParams &p, const float4 *__restrict__ tab, const float q[3],
                                                    float dz2, float dy2, float ka, int u_begin, int u_end)
{
	float sx = 0.0f, sy = 0.0f;
	for (int r = u_begin; r < u_end; r++) {
		const float rdx = __fsub_rn(q[0], __fmul_rn((float)r, p.px));
		const float arg = ka * rdx;
		const float wa = arg * arg;
		if (!(wa < HALF_PI_SQ)) continue;
		const float a = apod_cos2(wa);
		const float rd = sqrt_newton(__fadd_rn(__fmul_rn(rdx, rdx), dz2));
		float ax = 0.0f, ay = 0.0f;
		int row = r * p.T * p.S;
		float tf = 0.0f;
		#pragma unroll 2
		for (int t = 0; t < p.T; t++) {
			const float dx = __fsub_rn(q[0], __fmul_rn(p.px, tf));
			const float d = sqrt_newton(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), dy2), dz2));
			float tt = div_rc(__fadd_rn(d, rd), p.c, p.rc);
			tt = __fadd_rn(tt, p.toff);
			forces_table_term<INTERP, DEMOD, ROT>(p, tab, row, __fmul_rn(tt, p.fs), a, ax, ay);
			tf += 1.0f;
			row += p.S;
		}
		sx += ax;
		sy += ay;
	}
	return make_float2(sx, sy);
}

/* FORCES fast path of voxel (vx, vy, vz) over receive channels [u_begin,
 * u_end): the proven loop from the table tab, or das_voxel when the voxel lacks
 * the proof (INTERP cubic or linear; tab built for these parameters). */
template <int INTERP>
__device__ __forceinline__ float2 forces_voxel(const DasParams &p, const float4 *__restrict__ tab, int vx, int vy,
                                               int vz, int u_begin, int u_end)
{
	float w[3], q[3];
	m4v(p.M, (float)vx, (float)vy, (float)vz, w);
	m4v(p.X, w[0], w[1], w[2], q);
	const float dz2 = __fmul_rn(q[2], q[2]);
	const float dy = __fsub_rn(q[1], p.cy_forces), dy2 = __fmul_rn(dy, dy);
	const float ka = __fdiv_rn(p.apod_scale, fabsf(q[2]));

	/* bounds over all (r, t): the lateral offsets are linear in r and t, so their
	 * extremes sit at the end elements (or 0 inside the array); margins cover the
	 * roundings of the chain and of these bounds */
	const float tx_hi = (float)(p.T - 1) * p.px, rx_hi = (float)(p.C - 1) * p.px;
	const float dxm = fmaxf(fabsf(q[0]), fabsf(q[0] - tx_hi));
	const float dxn = q[0] < 0.0f ? -q[0] : q[0] > tx_hi ? q[0] - tx_hi : 0.0f;
	const float rxm = fmaxf(fabsf(q[0]), fabsf(q[0] - rx_hi));
	const float xt_lo = dy2 + dz2 + dxn * dxn, xt_hi = (dy2 + dz2 + dxm * dxm) * 1.0001f;
	const float xr_lo = dz2, xr_hi = (dz2 + rxm * rxm) * 1.0001f;
	const float dmin = (sqrtf(xt_lo) + sqrtf(xr_lo)) * 0.9999f, dmax = (sqrtf(xt_hi) + sqrtf(xr_hi)) * 1.0001f;
	const bool fast = p.fast_sqrt && fminf(xt_lo, xr_lo) >= p.sqrt_lo && fmaxf(xt_hi, xr_hi) <= p.sqrt_hi &&
	                  dmax <= p.c_hi && p.c_lo <= 0x1p-100f && p.fs_lo <= 0x1p-100f && (float)p.S <= p.fs_hi;
	constexpr int extra = INTERP == INTERP_CUBIC ? 2 : 1;
	const float s_lim = (float)(p.S - extra);
	const float imin = (dmin / p.c + p.toff) * p.fs, imax = (dmax / p.c + p.toff) * p.fs;
	const bool inrange = p.c > 0.0f && p.fs > 0.0f && imin - fabsf(imin) * 1e-4f >= 0.01f &&
	                     imax + fabsf(imax) * 1e-4f + 0.01f < s_lim;

	float2 s;
	const bool demod = p.fc > 0.0f;
	if (fast && inrange && (!demod || p.rot_table != 0)) {
		if (demod && p.rot_table == 1) s = forces_voxel_fast<INTERP, true, 1>(p, tab, q, dz2, dy2, ka, u_begin, u_end);
		else if (demod)                s = forces_voxel_fast<INTERP, true, 2>(p, tab, q, dz2, dy2, ka, u_begin, u_end);
		else                           s = forces_voxel_fast<INTERP, false, 0>(p, tab, q, dz2, dy2, ka, u_begin, u_end);
	} else {
		s = das_voxel<DAS_FORCES, INTERP, true>(p, vx, vy, vz, u_begin, u_end);
	}
	return s;
}

} /* namespace bf */
