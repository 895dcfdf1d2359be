/*
 * bf_das_staged.cuh -- HERCULES delay-and-sum with the interpolation table staged
 * in shared memory (das.glsl:178-215, the fast path; the same terms, order and
 * accumulation as hercules_tile in bf_das_hercules.cuh).
 *
 * Why. The per-term table gather of hercules_tile reads 32 (FP32 cubic) or 16
 * (FP16 cubic) bytes per lane from L1; on the 3D workload it takes about twice
 * the data-pipe wavefronts its bytes need, and that pipe is its bound. A
 * shared-memory LDS.128 serves eight lanes per wavefront when the lanes fall in
 * distinct or identical 16-byte words, which lanes reading neighbouring samples
 * of one (receive, transmit) row do.
 *
 * How. A block of 128 threads covers 4 x 4 x 16 or 4 x 8 x 8 voxels (two depths
 * per thread), or 8 x 1 x 16 for planes. For every row (r, t) it bounds the
 * samples any of its voxels can read: with the block's voxel box mapped to
 * transducer coordinates (centre q_c, circumscribed radius R) and its
 * transmit-distance range [dtx_lo, dtx_hi], every receive distance lies in
 * |q_c - e_rt| -/+ R, so every sample index lies in
 * [((dtx_lo + |q_c - e| - R) / c + toff) fs, ((dtx_hi + |q_c - e| + R) / c + toff) fs]
 * (half a sample of margin each side). A window is therefore at most
 * (dtx_hi - dtx_lo + 2 R) fs / c + 2.3 segments long for every row, and a block
 * checks once that this fits stg_wm; blocks that do not fit, or whose voxels lack
 * the fast in-range proof, run hercules_tile instead.
 * Per receive channel the block stages the rows of its transmit interval (the
 * union of its voxels' apodization intervals) in chunks of stg_rc rows: each of
 * stg_rc threads bounds one row's window and issues one cp.async.bulk copy of it
 * from the table (L2-resident) into shared memory, completing on an mbarrier;
 * the next chunk's copies run while the current chunk is summed (two buffers).
 * Each warp walks the transmits of its lanes' union interval in step, so the
 * lanes of a load read one row. A lane's terms outside its own aperture weigh
 * exactly 0 (the reference weighs them cos(pi/2)^2 ~ 2e-15).
 *
 * FP32 tables only: with the FP16 table (16 bytes per term) the gathers are no
 * longer the bound, and the staging overhead (union intervals, window indices,
 * barriers) made that kernel slower than hercules_tile.
 *
 * Every mbarrier wait is bounded (about one second); a wait that runs out sets
 * DasParams::wait_error, the block drains the copies it issued and stops.
 */
#pragma once
#include "bf_das_hercules.cuh"

namespace bf {

constexpr long long STG_WAIT_CYCLES = 2000000000ll;   /* ~1 s at 2 GHz */

/* bytes of one table segment */
template <int INTERP, bool H> __host__ __device__ constexpr int stg_seg_bytes()
{
	return H ? (INTERP == INTERP_CUBIC ? 16 : 8) : (INTERP == INTERP_CUBIC ? 32 : 16);
}

/* Block tiles of the staged kernel (HercTile<TY>): volumes 4 x 4 x 16 (TY 4) or
 * 4 x 8 x 8 (TY 8), planes 8 x 1 x 16 (TY 1). Segments per staged row window:
 * the 3D workload's 4 x 4 x 16 box spans 19.4 samples, its 4 x 8 x 8 box 11.0,
 * the plane's 8 x 1 x 16 box 20.0. */
template <int TY> __host__ __device__ constexpr int stg_wm() { return TY == 8 ? 14 : 24; }

/* rows per chunk: about 25 KB of windows in two buffers (8 blocks per SM) */
template <int TY, int SEGB> __host__ __device__ constexpr int stg_rc()
{
	return (TY == 8 ? 28 : 16) * 32 / SEGB;
}

/* dynamic shared memory of a block: two buffers of stg_rc windows, their first
 * segments, four mbarriers (full and empty per buffer), the stop word, the box,
 * the block's transmit interval per receive channel (receive channels < 256) */
template <int INTERP, int TY, bool H> __host__ __device__ constexpr int stg_smem_bytes()
{
	return 2 * stg_rc<TY, stg_seg_bytes<INTERP, H>()>() * stg_wm<TY>() * stg_seg_bytes<INTERP, H>() +
	       2 * stg_rc<TY, stg_seg_bytes<INTERP, H>()>() * 4 + 5 * 8 + 8 * 4 + 2 * 256 * 4;
}

__device__ __forceinline__ uint32_t stg_smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool stg_wait(uint32_t bar, uint32_t parity, long long limit = STG_WAIT_CYCLES)
{
	const long long t0 = clock64();
	while (true) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if (clock64() - t0 > limit) return false;
	}
}

/* stg_wait that also gives up when the block's stop word is set; a wait that runs
 * out sets the stop word and the error word */
__device__ __forceinline__ bool stg_wait_or_stop(uint32_t bar, uint32_t parity, volatile int *stop, unsigned *error)
{
	const long long t0 = clock64();
	while (true) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if (*stop) return false;
		if (clock64() - t0 > STG_WAIT_CYCLES) {
			*stop = 1;
			atomicExch(error, 1u);
			return false;
		}
	}
}

/* floor(x) and x - floor(x) for 0 <= x < 2^31 (truncation; the voxels are proven
 * in range, so x >= 0); j_minus is floor(x) minus `lo`. The float/integer
 * conversions run on the special-function unit; doing the same on the FMA pipe
 * (adding 1.5 * 2^23) measured slower, as that pipe is the busier one here. */
__device__ __forceinline__ void stg_floor(float x, int lo, int &j_minus, float &f)
{
	const int i = (int)x;
	j_minus = i - lo;
	f = x - (float)i;
}

__device__ __forceinline__ void stg_floor2(float2 x, int lo, int &j0, int &j1, float2 &f)
{
	const int i0 = (int)x.x, i1 = (int)x.y;
	j0 = i0 - lo;
	j1 = i1 - lo;
	f = __fadd2_rn(x, make_float2(-(float)i0, -(float)i1));
}

/* Geometry of a block's voxel box for the window bounds. */
struct StgBox {
	float qc[3];        /* box centre in transducer coordinates */
	float rq;           /* circumscribed radius in transducer coordinates */
	float dtx_lo, dtx_hi;
};

__device__ __forceinline__ StgBox stg_box(const DasParams &p, int x0, int x1, int y0, int y1, int z0, int z1)
{
	StgBox b;
	float pc[3];
	m4v(p.M, 0.5f * (float)(x0 + x1), 0.5f * (float)(y0 + y1), 0.5f * (float)(z0 + z1), pc);
	m4v(p.X, pc[0], pc[1], pc[2], b.qc);
	float rq = 0.0f, rp = 0.0f, lo = INFINITY, hi = -INFINITY;
	#pragma unroll
	for (int k = 0; k < 8; k++) {
		float w[3], q[3];
		m4v(p.M, (float)((k & 1) ? x1 : x0), (float)((k & 2) ? y1 : y0), (float)((k & 4) ? z1 : z0), w);
		m4v(p.X, w[0], w[1], w[2], q);
		const float dq0 = q[0] - b.qc[0], dq1 = q[1] - b.qc[1], dq2 = q[2] - b.qc[2];
		const float dp0 = w[0] - pc[0], dp1 = w[1] - pc[1], dp2 = w[2] - pc[2];
		rq = fmaxf(rq, dq0 * dq0 + dq1 * dq1 + dq2 * dq2);
		rp = fmaxf(rp, dp0 * dp0 + dp1 * dp1 + dp2 * dp2);
		const float d = transmit_distance(p, w, 0);
		lo = fminf(lo, d);
		hi = fmaxf(hi, d);
	}
	/* a plane wave's distance is linear in the point (extremes at corners); a
	 * cylindrical wave's is convex (maximum at a corner, minimum at least the
	 * centre's minus the box radius) */
	const float4 f = __ldg(p.focal);
	if (f.w == 0.0f) lo = fmaxf(0.0f, transmit_distance(p, pc, 0) - sqrtf(rp) * 1.0001f);
	b.rq = sqrtf(rq) * 1.0001f + 1e-9f;
	b.dtx_lo = lo - fabsf(lo) * 1e-5f;
	b.dtx_hi = hi + fabsf(hi) * 1e-5f;
	return b;
}

/* Window [lo, lo + len) of table segments of row (r, t) for the block's box, with
 * lo + len <= S; len <= WM when stg_box_fits held. Segment counts of the 8-byte
 * forms kept even (16-byte copies; rows of an even sample count). */
template <int SEGB, int WM>
__device__ __forceinline__ void stg_window(const DasParams &p, const StgBox &b, int r, int t, int &lo, int &len)
{
	const float ex = p.rx_cols ? (float)r * p.px : (float)t * p.px;
	const float ey = p.rx_cols ? (float)t * p.py : (float)r * p.py;
	const float dx = b.qc[0] - ex, dy = b.qc[1] - ey;
	const float dc = sqrtf(dx * dx + dy * dy + b.qc[2] * b.qc[2]);
	const float ilo = ((b.dtx_lo + fmaxf(dc - b.rq, 0.0f)) / p.c + p.toff) * p.fs;
	const float ihi = ((b.dtx_hi + dc + b.rq) / p.c + p.toff) * p.fs;
	int a = (int)floorf(ilo - 0.5f - fabsf(ilo) * 1e-4f), e = (int)floorf(ihi + 0.5f + fabsf(ihi) * 1e-4f);
	a = min(max(a, 0), p.S - 1);
	e = min(e, p.S - 1);
	if (SEGB == 8) {
		a &= ~1;
		e |= 1;
		e = min(e, p.S - 1);
	}
	if (e < a) e = a;
	int n = e - a + 1;
	if (SEGB == 8) n = (n + 1) & ~1;
	lo = a;
	len = min(n, WM);
}

/* true when every row's window of the box fits WM segments: a window spans
 * ihi - ilo <= (dtx_hi - dtx_lo + 2 R) fs / c plus its margins (half a sample
 * and 1e-4 of the index, below S, on each side), and floor() adds at most one
 * segment more */
template <int WM>
__device__ __forceinline__ bool stg_box_fits(const DasParams &p, const StgBox &b)
{
	if (!(p.c > 0.0f) || !(p.fs > 0.0f)) return false;
	const float span = (b.dtx_hi - b.dtx_lo + 2.0f * b.rq) / p.c * p.fs;
	return span * 1.0002f + 2.2f + 2e-4f * (float)p.S <= (float)WM;
}

/* One FP32 term from the staged window (a voxel proven in range): the delay chain
 * of term_tail<..., INR> bit for bit; the segment at local index j - lo. */
template <int INTERP, bool DEMOD, int ROT, int WM>
__device__ __forceinline__ void stg_term(const DasParams &p, const float4 *__restrict__ win, int lo, float lat2,
                                         float dz2, float ka2, float dtx, float scale, float &ax, float &ay)
{
	const float w = ka2 * lat2;
	const float x = __fadd_rn(lat2, dz2);
	const float drx = sqrt_newton(x);
	const float d = __fadd_rn(dtx, drx);
	float tt = div_rc(d, p.c, p.rc);
	tt = __fadd_rn(tt, p.toff);
	const float idx = __fmul_rn(tt, p.fs);
	const float a = w < HALF_PI_SQ ? apod_cos2_p5(w) * scale : 0.0f;
	int jm;
	float f;
	stg_floor(idx, lo, jm, f);
	const unsigned jl = min((unsigned)jm, (unsigned)(WM - 1));
	float vx, vy;
	if (INTERP == INTERP_CUBIC) {
		const float4 c0 = win[2 * jl], c1 = win[2 * jl + 1];
		vx = fmaf(fmaf(fmaf(c1.z, f, c1.x), f, c0.z), f, c0.x);
		vy = fmaf(fmaf(fmaf(c1.w, f, c1.y), f, c0.w), f, c0.y);
	} else {
		const float4 c = win[jl];
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

/* Two depths of a column (the float2 lanes are the two voxels) from the staged
 * window, FP32: the delay chain of stg_term in packed FP32 pairs. Per component
 * __fmul2_rn / __fadd2_rn / __ffma2_rn are the IEEE operations of the scalar
 * chain, so sample indices stay bit-equal; the Horner evaluation and the
 * rotation run on (re, im) pairs in the scalar code's order. */
template <int INTERP, bool DEMOD, int ROT, int WM>
__device__ __forceinline__ void stg_term2(const DasParams &p, const float4 *__restrict__ win, int lo, float lat2,
                                          float2 dz2, float2 ka2, float2 dtx, float scale, float2 *acc)
{
	const float2 l2 = make_float2(lat2, lat2);
	const float2 w = __fmul2_rn(ka2, l2);
	const float2 x = __fadd2_rn(l2, dz2);
	float r0, r1;
	asm("rsqrt.approx.f32 %0, %1;" : "=f"(r0) : "f"(x.x));
	asm("rsqrt.approx.f32 %0, %1;" : "=f"(r1) : "f"(x.y));
	const float2 r = make_float2(r0, r1);
	const float2 y = __fmul2_rn(x, r);
	const float2 h = __fmul2_rn(make_float2(0.5f, 0.5f), r);
	const float2 e = __ffma2_rn(make_float2(-y.x, -y.y), y, x);
	const float2 drx = __ffma2_rn(e, h, y);                 /* sqrt_newton */
	const float2 d = __fadd2_rn(dtx, drx);
	const float2 q = __fmul2_rn(d, make_float2(p.rc, p.rc));
	const float2 rr = __ffma2_rn(make_float2(-q.x, -q.y), make_float2(p.c, p.c), d);
	float2 tt = __ffma2_rn(rr, make_float2(p.rc, p.rc), q);  /* div_rc */
	tt = __fadd2_rn(tt, make_float2(p.toff, p.toff));
	const float2 idx = __fmul2_rn(tt, make_float2(p.fs, p.fs));
	/* apod_cos2_p5 on both voxels */
	float2 a = __ffma2_rn(make_float2(-1.12993468e-04f, -1.12993468e-04f), w,
	                      make_float2(3.10126483e-03f, 3.10126483e-03f));
	a = __ffma2_rn(a, w, make_float2(-4.43560816e-02f, -4.43560816e-02f));
	a = __ffma2_rn(a, w, make_float2(3.33286583e-01f, 3.33286583e-01f));
	a = __ffma2_rn(a, w, make_float2(-9.99991953e-01f, -9.99991953e-01f));
	a = __ffma2_rn(a, w, make_float2(1.0f, 1.0f));
	if (scale != 1.0f) a = __fmul2_rn(a, make_float2(scale, scale));
	a.x = w.x < HALF_PI_SQ ? a.x : 0.0f;
	a.y = w.y < HALF_PI_SQ ? a.y : 0.0f;
	int i0, i1;
	float2 f;
	stg_floor2(idx, lo, i0, i1, f);
	const unsigned j0 = min((unsigned)i0, (unsigned)(WM - 1)), j1 = min((unsigned)i1, (unsigned)(WM - 1));
	float2 v0, v1;
	if (INTERP == INTERP_CUBIC) {
		const float4 c00 = win[2 * j0], c01 = win[2 * j0 + 1], c10 = win[2 * j1], c11 = win[2 * j1 + 1];
		const float2 f0 = make_float2(f.x, f.x), f1 = make_float2(f.y, f.y);
		v0 = __ffma2_rn(make_float2(c01.z, c01.w), f0, make_float2(c01.x, c01.y));
		v1 = __ffma2_rn(make_float2(c11.z, c11.w), f1, make_float2(c11.x, c11.y));
		v0 = __ffma2_rn(v0, f0, make_float2(c00.z, c00.w));
		v1 = __ffma2_rn(v1, f1, make_float2(c10.z, c10.w));
		v0 = __ffma2_rn(v0, f0, make_float2(c00.x, c00.y));
		v1 = __ffma2_rn(v1, f1, make_float2(c10.x, c10.y));
	} else {
		const float4 c0 = win[j0], c1 = win[j1];
		v0 = __ffma2_rn(make_float2(c0.z, c0.w), make_float2(f.x, f.x), make_float2(c0.x, c0.y));
		v1 = __ffma2_rn(make_float2(c1.z, c1.w), make_float2(f.y, f.y), make_float2(c1.x, c1.y));
	}
	if (DEMOD) {
		float2 an = __ffma2_rn(make_float2(p.theta, p.theta), f, make_float2(-p.theta_half, -p.theta_half));
		if (ROT == 2) {
			const float2 k = make_float2(-rintf(an.x * 0.159154943f), -rintf(an.y * 0.159154943f));
			an = __ffma2_rn(k, make_float2(6.28125f, 6.28125f), an);
			an = __ffma2_rn(k, make_float2(0x1.fb5444p-10f, 0x1.fb5444p-10f), an);
		}
		float s0, c0, s1, c1;
		__sincosf(an.x, &s0, &c0);
		__sincosf(an.y, &s1, &c1);
		/* (ax, ay) += vy (-sa, ca), then vx (ca, sa): fmaf(ca, vx, fmaf(-sa, vy, ax)) */
		const float2 cs0 = __fmul2_rn(make_float2(a.x, a.x), make_float2(c0, s0));
		const float2 cs1 = __fmul2_rn(make_float2(a.y, a.y), make_float2(c1, s1));
		acc[0] = __ffma2_rn(make_float2(v0.y, v0.y), make_float2(-cs0.y, cs0.x), acc[0]);
		acc[1] = __ffma2_rn(make_float2(v1.y, v1.y), make_float2(-cs1.y, cs1.x), acc[1]);
		acc[0] = __ffma2_rn(make_float2(v0.x, v0.x), cs0, acc[0]);
		acc[1] = __ffma2_rn(make_float2(v1.x, v1.x), cs1, acc[1]);
	} else {
		acc[0] = __ffma2_rn(make_float2(a.x, a.x), v0, acc[0]);
		acc[1] = __ffma2_rn(make_float2(a.y, a.y), v1, acc[1]);
	}
}

/* FP16 segment of the staged window at the index: value and fraction */
template <int INTERP, int WM>
__device__ __forceinline__ void stg_sample_half(const uint8_t *__restrict__ win, int jm, float f, float &vx, float &vy)
{
	const unsigned jl = min((unsigned)jm, (unsigned)(WM - 1));
	const __half2 f2 = __float2half2_rn(f);
	__half2 h;
	if (INTERP == INTERP_CUBIC) {
		const uint4 q = ((const uint4 *)win)[jl];
		h = __hfma2(as_half2(q.w), f2, as_half2(q.z));
		h = __hfma2(h, f2, as_half2(q.y));
		h = __hfma2(h, f2, as_half2(q.x));
	} else {
		const uint2 q = ((const uint2 *)win)[jl];
		h = __hfma2(as_half2(q.y), f2, as_half2(q.x));
	}
	const float2 v = __half22float2(h);
	vx = v.x;
	vy = v.y;
}

/* Precision 1, one transmit of two depths of a column (packed FP32 pairs, as
 * term_h2) from the staged window. */
template <int INTERP, bool DEMOD, int ROT, int WM>
__device__ __forceinline__ void stg_term_h2(const DasParams &p, const uint8_t *__restrict__ win, int lo, float lat2,
                                            float2 dz2, float2 ka2, float2 io, float scale, float2 &ax, float2 &ay)
{
	const float2 l2 = make_float2(lat2, lat2);
	const float2 w = __fmul2_rn(ka2, l2);
	const float2 x = __fadd2_rn(l2, dz2);
	float r0, r1;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x.x));
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(x.y));
	const float2 idx = __ffma2_rn(__fmul2_rn(x, make_float2(r0, r1)), make_float2(p.fs_c, p.fs_c), io);
	float2 a = __ffma2_rn(make_float2(-0.031044068f, -0.031044068f), w, make_float2(0.31450406f, 0.31450406f));
	a = __ffma2_rn(a, w, make_float2(-0.99229395f, -0.99229395f));
	a = __ffma2_rn(a, w, make_float2(1.0f, 1.0f));
	if (scale != 1.0f) a = __fmul2_rn(a, make_float2(scale, scale));
	a.x = w.x < HALF_PI_SQ ? a.x : 0.0f;
	a.y = w.y < HALF_PI_SQ ? a.y : 0.0f;
	int i0, i1;
	float2 f, vx, vy;
	stg_floor2(idx, lo, i0, i1, f);
	stg_sample_half<INTERP, WM>(win, i0, f.x, vx.x, vy.x);
	stg_sample_half<INTERP, WM>(win, i1, f.y, vx.y, vy.y);
	if (DEMOD) {
		float2 ang = __ffma2_rn(make_float2(p.theta, p.theta), f, make_float2(-p.theta_half, -p.theta_half));
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

/* The staged block: receive channels [u_begin, u_end) of voxel tile (bx, yt, bz).
 * Called only when every voxel of the block is fast, proven in range and shares
 * its column's lateral coordinates, and the box fits (uniform over the block). */
template <int INTERP, int TY, bool H, bool DEMOD, int ROT>
__device__ __forceinline__ void hercules_staged_body(const DasParams &p, const float4 *__restrict__ tab, uint8_t *smem,
                                                     const StgBox &box_in, const HercVoxel *v, bool inside, int u_begin,
                                                     int u_end, float *sx, float *sy)
{
	using Tile = HercTile<TY, 128>;
	constexpr int NV = Tile::NV;
	constexpr int SEGB = stg_seg_bytes<INTERP, H>();
	constexpr int WM = stg_wm<TY>(), RC = stg_rc<TY, SEGB>();
	constexpr int BUFB = RC * WM * SEGB;
	uint8_t *bufs = smem;
	int *win_lo = (int *)(smem + 2 * BUFB);
	uint64_t *bars = (uint64_t *)(win_lo + 2 * RC);        /* full[2], empty[2] */
	volatile int *stop = (volatile int *)(bars + 4);
	float *boxs = (float *)(bars + 5);
	int *tb_lo = (int *)(boxs + 8), *tb_hi = tb_lo + 256;
	const int tid = threadIdx.x, lane = tid & 31;
	constexpr unsigned FULL = 0xffffffffu;
	constexpr int WARPS = 128 / 32;

	for (int i = tid; i < 2 * BUFB / 16; i += blockDim.x) ((uint4 *)bufs)[i] = make_uint4(0u, 0u, 0u, 0u);
	for (int i = tid; i < 256; i += blockDim.x) { tb_lo[i] = p.T; tb_hi[i] = -1; }
	if (tid == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(stg_smem_u32(bars)), "r"(RC) : "memory");
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(stg_smem_u32(bars + 1)), "r"(RC) : "memory");
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(stg_smem_u32(bars + 2)), "r"(WARPS) : "memory");
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(stg_smem_u32(bars + 3)), "r"(WARPS) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		*stop = 0;
		boxs[0] = box_in.qc[0]; boxs[1] = box_in.qc[1]; boxs[2] = box_in.qc[2];
		boxs[3] = box_in.rq; boxs[4] = box_in.dtx_lo; boxs[5] = box_in.dtx_hi;
	}
	/* the zero fill (generic proxy) before any bulk copy (async proxy) into it */
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	__syncthreads();

	const float pitch_fix = p.rx_cols ? p.px : p.py, pitch_var = p.rx_cols ? p.py : p.px;
	const float q_fix = v[0].q_fix, q_var = v[0].q_var;
	float lim2 = v[0].lim2;
	#pragma unroll
	for (int k = 1; k < NV; k++) lim2 = fmaxf(lim2, v[k].lim2);
	/* lateral offset of receive channel r, squared, as the term loop forms it */
	auto fixed2 = [&](int r) -> float {
		if (H) {
			const float df = fmaf(-(float)r, pitch_fix, q_fix);
			return df * df;
		}
		const float df = __fsub_rn(q_fix, __fmul_rn((float)r, pitch_fix));
		return __fmul_rn(df, df);
	};
	/* the block's transmit interval per receive channel (union of its voxels') */
	for (int r = u_begin; r < u_end; r += p.rx_step) {
		int lo = p.T, hi = -1;
		if (inside) aperture_interval(q_var, pitch_var, lim2 - fixed2(r), p.T, lo, hi);
		if (lo > hi) { lo = p.T; hi = -1; }
		lo = __reduce_min_sync(FULL, lo);
		hi = __reduce_max_sync(FULL, hi);
		if ((tid & 31) == 0 && lo <= hi) {
			atomicMin(tb_lo + r, lo);
			atomicMax(tb_hi + r, hi);
		}
	}
	__syncthreads();

	auto next_r = [&](int r) {
		for (; r < u_end; r += p.rx_step)
			if (tb_lo[r] <= tb_hi[r]) return r;
		return u_end;
	};
	/* rows t0 .. of receive channel r into buffer b: one bulk copy per row */
	auto issue = [&](int r, int t0, int b) {
		if (tid < RC) {
			const uint32_t bar = stg_smem_u32(bars + b);
			const int t = t0 + tid;
			if (t <= tb_hi[r]) {
				StgBox bx;
				bx.qc[0] = boxs[0]; bx.qc[1] = boxs[1]; bx.qc[2] = boxs[2];
				bx.rq = boxs[3]; bx.dtx_lo = boxs[4]; bx.dtx_hi = boxs[5];
				int lo, len;
				stg_window<SEGB, WM>(p, bx, r, t, lo, len);
				win_lo[b * RC + tid] = lo;
				const uint32_t bytes = (uint32_t)(len * SEGB);
				const uint32_t dst = stg_smem_u32(bufs + b * BUFB + tid * WM * SEGB);
				const uint8_t *src = (const uint8_t *)tab + ((size_t)(r * p.T + t) * p.S + lo) * SEGB;
				asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
				asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
				             :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
			} else {
				asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
			}
		}
	};

	int cr = next_r(u_begin);
	if (cr >= u_end) return;
	int ct0 = tb_lo[cr];
	issue(cr, ct0, 0);
	/* Chunk c sits in buffer c % 2. Its copies complete full[c % 2]; every warp
	 * arrives on empty[c % 2] when it has summed the chunk, and the copies of
	 * chunk c + 2 wait for that, so a warp can run a chunk ahead of the slowest
	 * instead of meeting it at a block barrier after every chunk. */
	uint32_t c = 0;
	int last_issued = 0;                /* the last chunk this thread's copies went to (chunk 0 above) */
	int buf = 0, prev_r = -1;
	int w_lo = 0, w_hi = -1;
	float f2 = 0.0f;
	float ax[NV], ay[NV];
	#pragma unroll
	for (int k = 0; k < NV; k++) ax[k] = ay[k] = 0.0f;
	while (true) {
		int nr = cr, nt0 = ct0 + RC;
		if (nt0 > tb_hi[cr]) {
			nr = next_r(cr + p.rx_step);
			nt0 = nr < u_end ? tb_lo[nr] : 0;
		}
		const bool has_next = nr < u_end;
		if (has_next && tid < RC) {
			/* buffer buf ^ 1 last held chunk c - 1: wait until every warp summed it */
			if (c == 0 || stg_wait_or_stop(stg_smem_u32(bars + 2 + (buf ^ 1)), ((c - 1) >> 1) & 1u, stop, p.wait_error)) {
				issue(nr, nt0, buf ^ 1);
				last_issued = (int)c + 1;
			}
		}
		if (cr != prev_r) {
			prev_r = cr;
			f2 = fixed2(cr);
			int lo = p.T, hi = -1;
			if (inside) aperture_interval(q_var, pitch_var, lim2 - f2, p.T, lo, hi);
			if (lo > hi) { lo = p.T; hi = -1; }
			w_lo = __reduce_min_sync(FULL, lo);
			w_hi = __reduce_max_sync(FULL, hi);
		}
		int ok = stg_wait_or_stop(stg_smem_u32(bars + buf), (c >> 1) & 1u, stop, p.wait_error) && !*stop;
		if (!__shfl_sync(FULL, ok, 0)) break;
		const int last = min(ct0 + RC - 1, tb_hi[cr]);
		int t = max(ct0, w_lo);
		const int te = min(last, w_hi);
		const uint8_t *base = bufs + buf * BUFB;
		if (H && NV == 2) {
			float2 hx = make_float2(ax[0], ax[NV - 1]), hy = make_float2(ay[0], ay[NV - 1]);
			const float2 dz2h = make_float2(v[0].dz2, v[NV - 1].dz2), ka2h = make_float2(v[0].ka2, v[NV - 1].ka2);
			const float2 ioh = make_float2(v[0].io, v[NV - 1].io);
			if (t == 0 && t <= te) {
				/* t == 0 >= ct0: the chunk's first row, with the 1 / sqrt(T) weight */
				stg_term_h2<INTERP, DEMOD, ROT, WM>(p, base, win_lo[buf * RC], fmaf(q_var, q_var, f2), dz2h, ka2h, ioh,
				                                    p.inv_sqrt_T, hx, hy);
				t = 1;
			}
			const int *wl = win_lo + buf * RC + (t - ct0);
			const uint8_t *wrow = base + (t - ct0) * WM * SEGB;
			float tf = (float)t;
			#pragma unroll 2
			for (; t <= te; t++, wl++, wrow += WM * SEGB, tf += 1.0f) {
				const float dv = fmaf(-tf, pitch_var, q_var);
				stg_term_h2<INTERP, DEMOD, ROT, WM>(p, wrow, *wl, fmaf(dv, dv, f2), dz2h, ka2h, ioh, 1.0f, hx, hy);
			}
			ax[0] = hx.x; ax[NV - 1] = hx.y; ay[0] = hy.x; ay[NV - 1] = hy.y;
		} else if (NV == 2) {
			float2 acc[2] = {make_float2(ax[0], ay[0]), make_float2(ax[NV - 1], ay[NV - 1])};
			const float2 dz2p = make_float2(v[0].dz2, v[NV - 1].dz2), ka2p = make_float2(v[0].ka2, v[NV - 1].ka2);
			const float2 dtxp = make_float2(v[0].dtx, v[NV - 1].dtx);
			if (t == 0 && t <= te) {
				/* transmit 0 carries the 1 / sqrt(T) weight: peeled, so the loop below
				 * has no per-term scale */
				const float dv = __fsub_rn(q_var, __fmul_rn(0.0f, pitch_var));
				const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
				/* t == 0 >= ct0: the chunk's first row */
				stg_term2<INTERP, DEMOD, ROT, WM>(p, (const float4 *)base, win_lo[buf * RC], lat2, dz2p, ka2p, dtxp,
				                                  p.inv_sqrt_T, acc);
				t = 1;
			}
			/* per term: the row's window through pointers stepped by one row, and t as
			 * a float counter (exact: t < 2^24, so the products are the ones (float)t gives) */
			const int *wl = win_lo + buf * RC + (t - ct0);
			const float4 *wrow = (const float4 *)(base + (t - ct0) * WM * SEGB);
			float tf = (float)t;
			#pragma unroll 2
			for (; t <= te; t++, wl++, wrow += WM * SEGB / 16, tf += 1.0f) {
				const float dv = __fsub_rn(q_var, __fmul_rn(tf, pitch_var));
				const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
				stg_term2<INTERP, DEMOD, ROT, WM>(p, wrow, *wl, lat2, dz2p, ka2p, dtxp, 1.0f, acc);
			}
			ax[0] = acc[0].x; ay[0] = acc[0].y; ax[NV - 1] = acc[1].x; ay[NV - 1] = acc[1].y;
		} else {
			if (t == 0 && t <= te) {
				const int lo = win_lo[buf * RC];
				const float dv = __fsub_rn(q_var, __fmul_rn(0.0f, pitch_var));
				const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
				#pragma unroll
				for (int k = 0; k < NV; k++)
					stg_term<INTERP, DEMOD, ROT, WM>(p, (const float4 *)base, lo, lat2, v[k].dz2, v[k].ka2, v[k].dtx,
					                                 p.inv_sqrt_T, ax[k], ay[k]);
				t = 1;
			}
			/* as the packed loop: row pointers stepped, t as an exact float counter */
			const int *wl = win_lo + buf * RC + (t - ct0);
			const float4 *wrow = (const float4 *)(base + (t - ct0) * WM * SEGB);
			float tf = (float)t;
			#pragma unroll 2
			for (; t <= te; t++, wl++, wrow += WM * SEGB / 16, tf += 1.0f) {
				const int lo = *wl;
				const float dv = __fsub_rn(q_var, __fmul_rn(tf, pitch_var));
				const float lat2 = __fadd_rn(f2, __fmul_rn(dv, dv));
				#pragma unroll
				for (int k = 0; k < NV; k++)
					stg_term<INTERP, DEMOD, ROT, WM>(p, wrow, lo, lat2, v[k].dz2, v[k].ka2, v[k].dtx, 1.0f, ax[k], ay[k]);
			}
		}
		if (!has_next || nr != cr) {
			#pragma unroll
			for (int k = 0; k < NV; k++) { sx[k] += ax[k]; sy[k] += ay[k]; ax[k] = ay[k] = 0.0f; }
		}
		__syncwarp();
		if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(stg_smem_u32(bars + 2 + buf)) : "memory");
		if (!has_next) break;
		cr = nr;
		ct0 = nt0;
		buf ^= 1;
		c++;
	}
	/* every warp is out of its loop (each wait is bounded), so the stop word is final */
	__syncthreads();
	if (*stop) {
		/* a wait ran out in this block: the copy threads drain what they issued
		 * (bounded), every voxel of the block reports NaN */
		if (tid < RC)
			for (int k = max(0, last_issued - 1); k <= last_issued; k++)   /* chunk k sits in buffer k % 2 */
				stg_wait(stg_smem_u32(bars + (k & 1)), ((uint32_t)k >> 1) & 1u);
		#pragma unroll
		for (int k = 0; k < NV; k++) sx[k] = sy[k] = __int_as_float(0x7fc00000);
	}
}

/* Thread threadIdx.x of voxel tile (bx, yt, bz) of HercTile<TY> (volumes: TY 4
 * or 8), outer-loop group grp, with the table staged in shared memory (smem:
 * stg_smem_bytes<INTERP, TY, H>()); blocks that cannot stage run hercules_tile
 * on the same tile. */
template <int INTERP, int TY, bool H>
__device__ __forceinline__ void hercules_tile_staged(const DasParams &p, const float4 *__restrict__ tab, int bx, int yt,
                                                     int bz, int grp, uint8_t *smem)
{
	using Tile = HercTile<TY, 128>;
	constexpr int NV = Tile::NV;
	constexpr int WM = stg_wm<TY>();
	const int tid = threadIdx.x;
	const int vx = bx * Tile::X + (tid % Tile::X);
	const int vy = yt * Tile::Y + ((tid / Tile::X) % Tile::Y);
	const int vz0 = (bz * Tile::Z + tid / (Tile::X * Tile::Y)) * NV;
	const bool inside = vx < p.dims[0] && vy < p.dims[1] && vz0 < p.dims[2];
	const bool demod = p.fc > 0.0f;
	const int rot = p.rot_table;
	HercVoxel v[NV] = {};
	/* 8-byte segments are copied in pairs: rows of an even sample count only */
	bool ok = (INTERP == INTERP_CUBIC || INTERP == INTERP_LINEAR) && (!demod || rot != 0) && p.T <= 256 &&
	          p.loop_end <= 256 && (!H || NV == 2) && (stg_seg_bytes<INTERP, H>() != 8 || p.S % 2 == 0);
	if (inside) {
		#pragma unroll
		for (int k = 0; k < NV; k++) {
			if (vz0 + k < p.dims[2]) {
				v[k] = hercules_setup(p, vx, vy, vz0 + k);
				ok = ok && v[k].fast && v[k].inrange && v[k].q_fix == v[0].q_fix && v[k].q_var == v[0].q_var;
			} else {
				ok = false;
			}
		}
	}
	const int x0 = bx * Tile::X, y0 = yt * Tile::Y, z0 = bz * Tile::Z * NV;
	const int x1 = min(x0 + Tile::X, p.dims[0]) - 1, y1 = min(y0 + Tile::Y, p.dims[1]) - 1;
	const int z1 = min(z0 + Tile::Z * NV, p.dims[2]) - 1;
	const StgBox box = stg_box(p, x0, x1, y0, y1, z0, z1);
	ok = ok && stg_box_fits<WM>(p, box);
	if (!__syncthreads_and(ok)) {
		if (p.stage_only) {
			/* test mode: mark the block's voxels instead of running hercules_tile */
			if (inside) {
				const int64_t nvox = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
				#pragma unroll
				for (int k = 0; k < NV; k++) {
					if (vz0 + k >= p.dims[2]) break;
					const int64_t o = ((int64_t)(vz0 + k) * p.dims[1] + vy) * p.dims[0] + vx;
					const float2 nan2 = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
					if (p.groups > 1) p.partial[grp * nvox + o] = nan2;
					else              p.frame[o] = nan2;
				}
			}
			return;
		}
		hercules_tile<INTERP, TY, 128, H>(p, tab, bx, yt, bz, grp);
		return;
	}
	const int u_begin = grp * p.per_group;
	const int u_end   = min(p.loop_end, u_begin + p.per_group);
	float sx[NV], sy[NV];
	#pragma unroll
	for (int k = 0; k < NV; k++) sx[k] = sy[k] = 0.0f;
	if (demod && rot == 1)
		hercules_staged_body<INTERP, TY, H, true, 1>(p, tab, smem, box, v, inside, u_begin, u_end, sx, sy);
	else if (demod)
		hercules_staged_body<INTERP, TY, H, true, 2>(p, tab, smem, box, v, inside, u_begin, u_end, sx, sy);
	else
		hercules_staged_body<INTERP, TY, H, false, 0>(p, tab, smem, box, v, inside, u_begin, u_end, sx, sy);
	if (!inside) return;
	if (H) {
		const float us = pow2f(-half_table_shift(__ldg(p.absmax)));
		#pragma unroll
		for (int k = 0; k < NV; k++) { sx[k] *= us; sy[k] *= us; }
	}
	const int64_t nvox = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	#pragma unroll
	for (int k = 0; k < NV; k++) {
		const int64_t o = ((int64_t)(vz0 + k) * p.dims[1] + vy) * p.dims[0] + vx;
		if (p.groups > 1) p.partial[grp * nvox + o] = make_float2(sx[k], sy[k]);
		else              p.frame[o] = make_float2(sx[k], sy[k]);
	}
}

} /* namespace bf */
