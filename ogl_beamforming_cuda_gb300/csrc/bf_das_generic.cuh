/*
 * bf_das_generic.cuh -- the general delay-and-sum of one voxel (das.glsl:23-341):
 * every DAS mode, nearest / cubic / linear interpolation, fast and full
 * (coherency-weighted) paths. Shared by das_kernel and the batched launch.
 */
#pragma once
#include "bf_kernels.h"
#include "bf_das_math.cuh"

namespace bf {

/* sample_rf (das.glsl:64-72): interpolated channel sample rotated by the phase
 * of the sample time. Returns false when the reference's validity factor is 0.
 * base = (channel * transmits + transmit) * samples. */
template <int INTERP>
__device__ __forceinline__ bool sample_rf(const DasParams &p, int64_t base, float index, float2 &out)
{
	constexpr int extra = INTERP == INTERP_CUBIC ? 2 : INTERP == INTERP_LINEAR ? 1 : 0;
	if (!(index >= 0.0f) || !(index < 2147483520.0f)) return false;
	const int ii = (int)index;
	if (ii + extra >= p.S) return false;
	float2 v;
	if (INTERP == INTERP_NEAREST) {
		v = rf_at(p, base + (int64_t)roundf(index));
	} else {
		const float t = index - (float)ii;
		if (INTERP == INTERP_CUBIC) {
			float2 s0, s1, s2, s3;
			const int64_t j = base + ii - 1;
			if (j >= 0 && j + 3 < p.rf_count) {
				s0 = __ldg(p.rf + j); s1 = __ldg(p.rf + j + 1); s2 = __ldg(p.rf + j + 2); s3 = __ldg(p.rf + j + 3);
			} else {
				s0 = rf_at(p, j); s1 = rf_at(p, j + 1); s2 = rf_at(p, j + 2); s3 = rf_at(p, j + 3);
			}
			const float t2 = t * t;
			const float w0 = t * fmaf(t, fmaf(t, -0.5f, 1.0f), -0.5f);
			const float w1 = fmaf(t2, fmaf(t, 1.5f, -2.5f), 1.0f);
			const float w2 = t * fmaf(t, fmaf(t, -1.5f, 2.0f), 0.5f);
			const float w3 = t2 * fmaf(t, 0.5f, -0.5f);
			v.x = fmaf(w0, s0.x, fmaf(w1, s1.x, fmaf(w2, s2.x, w3 * s3.x)));
			v.y = fmaf(w0, s0.y, fmaf(w1, s1.y, fmaf(w2, s2.y, w3 * s3.y)));
		} else {
			const float2 s0 = rf_at(p, base + ii), s1 = rf_at(p, base + ii + 1);
			v.x = fmaf(t, s1.x - s0.x, s0.x);
			v.y = fmaf(t, s1.y - s0.y, s0.y);
		}
	}
	if (p.fc > 0.0f) {
		const float time = div_const(index, p.fs, p.rfs, p.fs_lo, p.fs_hi);
		const float arg  = __fmul_rn(p.r360_fc, time);
		/* Cody-Waite reduction of arg modulo 2 pi */
		const float C1 = 6.28125f, C2 = 0x1.fb5444p-10f, C3 = 0x1.68c234p-37f;
		const float k = rintf(arg * 0.159154943f);
		float r = fmaf(-k, C1, arg);
		r = fmaf(-k, C2, r);
		r = fmaf(-k, C3, r);
		float s, c;
		__sincosf(r, &s, &c);
		v = make_float2(c * v.x - s * v.y, s * v.x + c * v.y);
	}
	out = v;
	return true;
}


/* One (voxel, transmit, receive) term: apodization (w = (k lat)^2), receive
 * distance, sample index, interpolated and rotated sample, accumulated with weight
 * a * scale. Returns without contribution outside the aperture or the record. */
template <int INTERP>
__device__ __forceinline__ void accumulate_term(const DasParams &p, float w, float d_rx2, float dtx, int64_t base,
                                                float scale, float &ax, float &ay)
{
	if (!(w < HALF_PI_SQ)) return;
	const float a = apod_cos2(w) * scale;
	const float drx = sqrt_rx(p, d_rx2);
	float2 v;
	if (!sample_rf<INTERP>(p, base, sample_index(p, __fadd_rn(dtx, drx)), v)) return;
	ax = fmaf(a, v.x, ax);
	ay = fmaf(a, v.y, ay);
}

/* HERCULES fast path for one receive channel over transmits [t_lo, t_hi], without
 * branches in the loop body: a term outside the aperture or the record gets weight
 * 0 and a safe in-record index, so consecutive terms' loads can overlap. Requires
 * rf to hold exactly C*T*S samples (every index row + [-1, S] is in bounds except
 * -1, which the cubic path masks). */
template <int INTERP>
__device__ __forceinline__ void hercules_row(const DasParams &p, float q_var, float pitch_var, float f2, float dz2,
                                             float ka2, float dtx, int rbase, int t_lo, int t_hi, float &ax, float &ay)
{
	constexpr int extra = INTERP == INTERP_CUBIC ? 2 : INTERP == INTERP_LINEAR ? 1 : 0;
	const float s_lim = (float)(p.S - extra);
	const int last = (int)p.rf_count - 1;
	#pragma unroll 2
	for (int t = t_lo; t <= t_hi; t++) {
		const float dv = __fsub_rn(q_var, __fmul_rn((float)t, pitch_var));
		const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
		const float w = ka2 * lat2;
		float a = w < HALF_PI_SQ ? apod_cos2(w) : 0.0f;
		a = t == 0 ? a * p.inv_sqrt_T : a;
		const float drx = sqrt_rx(p, __fadd_rn(lat2, dz2));
		const float idx = sample_index(p, __fadd_rn(dtx, drx));
		const bool ok = idx >= 0.0f && idx < s_lim;
		a = ok ? a : 0.0f;
		const float ic = ok ? idx : 1.0f;
		const int ii = (int)ic;
		const int row = rbase + t * p.S;
		float2 v;
		if (INTERP == INTERP_NEAREST) {
			const int j = row + (int)roundf(ic);
			v = __ldg(p.rf + min(j, last));
			if (j > last) v = make_float2(0.0f, 0.0f);
		} else if (INTERP == INTERP_LINEAR) {
			const float f = ic - (float)ii;
			const float2 s0 = __ldg(p.rf + row + ii), s1 = __ldg(p.rf + row + ii + 1);
			v.x = fmaf(f, s1.x - s0.x, s0.x);
			v.y = fmaf(f, s1.y - s0.y, s0.y);
		} else {
			const float f = ic - (float)ii;
			const int j = row + ii - 1;
			float2 s0 = __ldg(p.rf + max(j, 0));
			const float2 s1 = __ldg(p.rf + j + 1), s2 = __ldg(p.rf + j + 2), s3 = __ldg(p.rf + j + 3);
			if (j < 0) s0 = make_float2(0.0f, 0.0f);
			const float f2c = f * f;
			const float w0 = f * fmaf(f, fmaf(f, -0.5f, 1.0f), -0.5f);
			const float w1 = fmaf(f2c, fmaf(f, 1.5f, -2.5f), 1.0f);
			const float w2 = f * fmaf(f, fmaf(f, -1.5f, 2.0f), 0.5f);
			const float w3 = f2c * fmaf(f, 0.5f, -0.5f);
			v.x = fmaf(w0, s0.x, fmaf(w1, s1.x, fmaf(w2, s2.x, w3 * s3.x)));
			v.y = fmaf(w0, s0.y, fmaf(w1, s1.y, fmaf(w2, s2.y, w3 * s3.y)));
		}
		if (p.fc > 0.0f) {
			const float time = div_const(ic, p.fs, p.rfs, p.fs_lo, p.fs_hi);
			const float arg  = __fmul_rn(p.r360_fc, time);
			const float C1 = 6.28125f, C2 = 0x1.fb5444p-10f, C3 = 0x1.68c234p-37f;
			const float k = rintf(arg * 0.159154943f);
			float r = fmaf(-k, C1, arg);
			r = fmaf(-k, C2, r);
			r = fmaf(-k, C3, r);
			float sn, cs;
			__sincosf(r, &sn, &cs);
			const float ca = a * cs, sa = a * sn;
			ax = fmaf(ca, v.x, fmaf(-sa, v.y, ax));
			ay = fmaf(sa, v.x, fmaf(ca, v.y, ay));
		} else {
			ax = fmaf(a, v.x, ax);
			ay = fmaf(a, v.y, ay);
		}
	}
}


/* The voxel (vx, vy, vz) summed over the outer loop range [u_begin, u_end)
 * (receive channels, or transmits for RCA); FAST = DASFast, else the full path. */
template <int FAMILY, int INTERP, bool FAST>
__device__ __forceinline__ float2 das_voxel(const DasParams &p, int vx, int vy, int vz, int u_begin, int u_end)
{
	float w[3], q[3];
	m4v(p.M, (float)vx, (float)vy, (float)vz, w);
	m4v(p.X, w[0], w[1], w[2], q);
	const float dz2 = __fmul_rn(q[2], q[2]);
	const int64_t row = (int64_t)p.S;                      /* samples per (channel, transmit) row */

	float sx = 0.0f, sy = 0.0f, sa = 0.0f;

	if (FAMILY == DAS_HERCULES) {
		const float dtx = transmit_distance(p, w, 0);
		const float ka  = __fdiv_rn(p.apod_scale, fabsf(q[2]));
		const float ka2 = ka * ka;
		const float lim2 = HALF_PI_SQ / ka2;                /* lat^2 bound of the aperture */
		if (FAST && !p.sparse_mode) {
			/* receive channel r fixes one lateral coordinate, transmit t the other */
			const float q_fix = p.rx_cols ? q[0] : q[1], pitch_fix = p.rx_cols ? p.px : p.py;
			const float q_var = p.rx_cols ? q[1] : q[0], pitch_var = p.rx_cols ? p.py : p.px;
			for (int r = u_begin; r < u_end; r += p.rx_step) {
				const float df = __fsub_rn(q_fix, __fmul_rn((float)r, pitch_fix));
				const float f2 = __fmul_rn(df, df);
				int t_lo, t_hi;
				aperture_interval(q_var, pitch_var, lim2 - f2, p.T, t_lo, t_hi);
				if (t_lo > t_hi) continue;
				float ax = 0.0f, ay = 0.0f;
				if (p.dense_rows) {
					hercules_row<INTERP>(p, q_var, pitch_var, f2, dz2, ka2, dtx, r * p.T * p.S, t_lo, t_hi, ax, ay);
					sx += ax;
					sy += ay;
					continue;
				}
				const int64_t rbase = (int64_t)r * p.T * row;
				int t = t_lo;
				if (t == 0) {
					const float dv = q_var;                  /* element 0 sits at 0 */
					const float dv0 = __fsub_rn(dv, __fmul_rn(0.0f, pitch_var));
					const float lat2 = __fadd_rn(f2, __fmul_rn(dv0, dv0));
					accumulate_term<INTERP>(p, ka2 * lat2, __fadd_rn(lat2, dz2), dtx, rbase, p.inv_sqrt_T, ax, ay);
					t = 1;
				}
				for (; t <= t_hi; t++) {
					const float dv = __fsub_rn(q_var, __fmul_rn((float)t, pitch_var));
					const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
					accumulate_term<INTERP>(p, ka2 * lat2, __fadd_rn(lat2, dz2), dtx, rbase + t * row, 1.0f, ax, ay);
				}
				sx += ax;
				sy += ay;
			}
		} else {
			/* sparse elements (UHERCULES) and the full / coherency path: every term */
			const int t_first = p.sparse_mode ? 1 : 0;
			const int outer_end = FAST ? u_end : p.T;
			for (int o = FAST ? u_begin : t_first; o < outer_end; o++) {
				float ax = 0.0f, ay = 0.0f;
				const int inner_begin = FAST ? t_first : 0, inner_end = FAST ? p.T : p.C;
				for (int i = inner_begin; i < inner_end; i++) {
					const int r = FAST ? o : i, t = FAST ? i : o;
					const int tc = p.sparse_mode ? (int)__ldg(p.sparse + t - 1) : t;
					const float ex = p.rx_cols ? __fmul_rn((float)r, p.px) : __fmul_rn((float)tc, p.px);
					const float ey = p.rx_cols ? __fmul_rn((float)tc, p.py) : __fmul_rn((float)r, p.py);
					const float dx = __fsub_rn(q[0], ex), dy = __fsub_rn(q[1], ey);
					const float lat2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
					const int64_t base = ((int64_t)r * p.T + t) * row;
					if (FAST) {
						accumulate_term<INTERP>(p, ka2 * lat2, __fadd_rn(lat2, dz2), dtx, base,
						                        t == 0 ? p.inv_sqrt_T : 1.0f, ax, ay);
					} else {
						float bx = 0.0f, by = 0.0f;
						accumulate_term<INTERP>(p, ka2 * lat2, __fadd_rn(lat2, dz2), dtx, base,
						                        t == 0 ? p.inv_sqrt_T : 1.0f, bx, by);
						sx += bx;
						sy += by;
						sa += sqrtf(bx * bx + by * by);
					}
				}
				if (FAST) { sx += ax; sy += ay; }
			}
		}
	}
	else if (FAMILY == DAS_FORCES) {
		const float ka = __fdiv_rn(p.apod_scale, fabsf(q[2]));
		const int t_first = p.sparse_mode ? 1 : 0;
		const int r0 = FAST ? u_begin : 0, r1 = FAST ? u_end : p.C;
		const float dy = __fsub_rn(q[1], p.cy_forces), dy2 = __fmul_rn(dy, dy);
		for (int r = r0; r < r1; r++) {
			const float rdx = __fsub_rn(q[0], __fmul_rn((float)r, p.px));
			const float arg = ka * rdx;
			const float wa = arg * arg;
			if (!(wa < HALF_PI_SQ)) continue;
			const float a = apod_cos2(wa);
			const float rd = __fsqrt_rn(__fadd_rn(__fmul_rn(rdx, rdx), dz2));
			float ax = 0.0f, ay = 0.0f;
			for (int t = t_first; t < p.T; t++) {
				const int tc = p.sparse_mode ? (int)__ldg(p.sparse + t - 1) : t;
				const float dx = __fsub_rn(q[0], __fmul_rn(p.px, (float)tc));
				const float d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), dy2), dz2));
				float2 v;
				const int64_t base = ((int64_t)r * p.T + (FAST ? t : tc)) * row;
				if (!sample_rf<INTERP>(p, base, sample_index(p, __fadd_rn(d, rd)), v)) continue;
				if (FAST) {
					ax = fmaf(a, v.x, ax);
					ay = fmaf(a, v.y, ay);
				} else {
					const float bx = a * v.x, by = a * v.y;
					sx += bx;
					sy += by;
					sa += sqrtf(bx * bx + by * by);
				}
			}
			if (FAST) { sx += ax; sy += ay; }
		}
	} else if (FAMILY == DAS_RCA) {
		const float q2x = p.rx_rows ? q[1] : q[0], q2y = q[2];
		const float ka = __fdiv_rn(p.apod_scale, fabsf(q2y));
		const float q2y2 = __fmul_rn(q2y, q2y);
		const float pitch = p.rx_rows ? p.py : p.px;
		const int t0 = FAST ? u_begin : 0, t1 = FAST ? u_end : p.T;
		for (int t = t0; t < t1; t++) {
			const float dtx = transmit_distance(p, w, t);
			float ax = 0.0f, ay = 0.0f;
			for (int r = 0; r < p.C; r++) {
				const float rvx = __fsub_rn(q2x, __fmul_rn((float)r, pitch));
				const float arg = ka * rvx;
				const float wa = arg * arg;
				if (!(wa < HALF_PI_SQ)) continue;
				const float a = apod_cos2(wa);
				const float rd = __fsqrt_rn(__fadd_rn(__fmul_rn(rvx, rvx), q2y2));
				float2 v;
				if (!sample_rf<INTERP>(p, ((int64_t)r * p.T + t) * row, sample_index(p, __fadd_rn(dtx, rd)), v)) continue;
				if (FAST) {
					ax = fmaf(a, v.x, ax);
					ay = fmaf(a, v.y, ay);
				} else {
					const float bx = a * v.x, by = a * v.y;
					sx += bx;
					sy += by;
					sa += sqrtf(bx * bx + by * by);
				}
			}
			if (FAST) { sx += ax; sy += ay; }
		}
	}

	if (!FAST && p.coherency) {
		const float den = sa + (sa == 0.0f ? 1.0f : 0.0f);
		sx *= sx / den;
		sy *= sy / den;
	}
	return make_float2(sx, sy);
}

} /* namespace bf */
