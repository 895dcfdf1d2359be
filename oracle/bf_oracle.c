/*
 * bf_oracle.c -- CPU oracle for the beamforming hot path. TEST INFRASTRUCTURE ONLY:
 * imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker; never linked into or called by the product library.
 *
 * Restates, in plain C, the reference's compute path:
 *   math.c:33-181                 Hadamard matrices, Kaiser and matched filters
 *   external/cephes.c:24-103      modified Bessel I0
 *   beamformer.c:303-481          pipeline planning (variants, strides, time offset)
 *   beamformer.c:483-518          DAS voxel transform
 *   shaders/decode.glsl:57-105    Hadamard decode (both passes)
 *   shaders/filter.glsl:29-91     demodulation / FIR filter
 *   shaders/das.glsl:23-341       delay-and-sum (FORCES, HERCULES, RCA, fast and full)
 *   shaders/sum.glsl + beamformer.c:218-235   frame averaging
 *   shaders/min_max.glsl + beamformer.c:595-607  min/max pyramid
 *
 * FP32 expressions are written one IEEE operation at a time in the reference's
 * left-to-right order; the file is compiled with -ffp-contract=off so no FMA is
 * formed. GLSL's implementation-defined round() is taken as round-half-away.
 */
#include "bf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BFO_PI_F      3.14159265358979323846f
#define BFO_DEG2RAD_F 0.017453292519943295f
#define BFO_PI_D      3.14159265358979323846

static int nthreads(int32_t t) { return t > 0 ? t : 1; }

/* ============================== host math ================================== */

/* Chebyshev series evaluation (cephes chbevl), used by I0. */
static double chbevl(double x, const double *c, int n)
{
	double b0 = c[0], b1 = 0.0, b2 = 0.0;
	for (int i = 1; i < n; i++) {
		b2 = b1;
		b1 = b0;
		b0 = x * b1 - b2 + c[i];
	}
	return 0.5 * (b0 - b2);
}

/* Modified Bessel function of order zero. Same published Chebyshev expansion as
 * the reference's vendored cephes_i0 (external/cephes.c:24-103): exp(-x) I0(x) on
 * [0, 8] and exp(-x) sqrt(x) I0(x) on (8, inf). Coefficients are Cephes 2.8's. */
double bfo_i0(double x)
{
	static const double A[30] = {
		-4.41534164647933937950E-18, 3.33079451882223809783E-17, -2.43127984654795469359E-16,
		1.71539128555513303061E-15, -1.16853328779934516808E-14, 7.67618549860493561688E-14,
		-4.85644678311192946090E-13, 2.95505266312963983461E-12, -1.72682629144155570723E-11,
		9.67580903537323691224E-11, -5.18979560163526290666E-10, 2.65982372468238665035E-9,
		-1.30002500998624804212E-8, 6.04699502254191894932E-8, -2.67079385394061173391E-7,
		1.11738753912010371815E-6, -4.41673835845875056359E-6, 1.64484480707288970893E-5,
		-5.75419501008210370398E-5, 1.88502885095841655729E-4, -5.76375574538582365885E-4,
		1.63947561694133579842E-3, -4.32430999505057594430E-3, 1.05464603945949983183E-2,
		-2.37374148058994688156E-2, 4.93052842396707084878E-2, -9.49010970480476444210E-2,
		1.71620901522208775349E-1, -3.04682672343198398683E-1, 6.76795274409476084995E-1,
	};
	static const double B[25] = {
		-7.23318048787475395456E-18, -4.83050448594418207126E-18, 4.46562142029675999901E-17,
		3.46122286769746109310E-17, -2.82762398051658348494E-16, -3.42548561967721913462E-16,
		1.77256013305652638360E-15, 3.81168066935262242075E-15, -9.55484669882830764870E-15,
		-4.15056934728722208663E-14, 1.54008621752140982691E-14, 3.85277838274214270114E-13,
		7.18012445138366623367E-13, -1.79417853150680611778E-12, -1.32158118404477131188E-11,
		-3.14991652796324136454E-11, 1.18891471078464383424E-11, 4.94060238822496958910E-10,
		3.39623202570838634515E-9, 2.26666899049817806459E-8, 2.04891858946906374183E-7,
		2.89137052083475648297E-6, 6.88975834691682398426E-5, 3.36911647825569408990E-3,
		8.04490411014108831608E-1,
	};
	if (x < 0) x = -x;
	if (x <= 8.0) return exp(x) * chbevl(x / 2.0 - 2.0, A, 30);
	return exp(x) * chbevl(32.0 / x - 2.0, B, 25) / sqrt(x);
}

static int is_pow2(int32_t a) { return (a & (a - 1)) == 0; }

/* Legendre symbol of k modulo the odd prime q (quadratic character). */
static int quadratic_character(int k, int q)
{
	k %= q;
	if (k < 0) k += q;
	if (k == 0) return 0;
	for (int x = 1; x < q; x++)
		if ((x * x) % q == k) return 1;
	return -1;
}

/* Bordered Paley-type Hadamard matrices of order 12 (q = 11) and 20 (q = 19) in
 * the orientation the reference tabulates (math.c:36-72): first row and column
 * all +1, core entry c[k] = -chi_q(k) for k != 0 and -1 on k = 0, with the core
 * rows cyclically shifted right by one per row for q = 11 and left for q = 19.
 * The tests check the result against the reference's own tables. */
static void paley_bordered(int q, int32_t *out)
{
	int n = q + 1;
	for (int j = 0; j < n; j++) out[j] = 1;
	for (int i = 1; i < n; i++) {
		out[i * n] = 1;
		for (int j = 1; j < n; j++) {
			int r = i - 1, c = j - 1;
			int k = (q == 11) ? (c - r) : (c + r);
			k %= q;
			if (k < 0) k += q;
			out[i * n + j] = (k == 0) ? -1 : -quadratic_character(k, q);
		}
	}
}

/* make_hadamard_transpose (math.c:33-122): Sylvester 2^k, or S_{2^k} (x) H_12 /
 * S_{2^k} (x) H_20 by Kronecker product, row-major [row][col]. */
int32_t bfo_hadamard_transpose(int32_t dim, int32_t *out)
{
	int32_t base = 0, order = dim;
	if (dim <= 0) return 0;
	if (is_pow2(dim)) {
		base = dim;
	} else if (dim % 20 == 0 && is_pow2(dim / 20)) {
		base = 20; order = dim / 20;
	} else if (dim % 12 == 0 && is_pow2(dim / 12)) {
		base = 12; order = dim / 12;
	}
	if (!base || !is_pow2(order)) return 0;

	const int kron = order != dim;   /* a 12 or 20 Paley factor is present */
	int32_t *m = !kron ? out : (int32_t *)malloc(sizeof(int32_t) * (size_t)order * (size_t)order);
	m[0] = 1;
	for (int32_t k = 1; k < order; k *= 2) {
		for (int32_t i = 0; i < k; i++) {
			for (int32_t j = 0; j < k; j++) {
				int32_t v = m[i * order + j];
				m[(i + k) * order + j]       = v;
				m[i * order + j + k]         = v;
				m[(i + k) * order + j + k]   = -v;
			}
		}
	}
	if (kron) {
		int32_t small[400];
		paley_bordered(base - 1, small);
		for (int32_t bi = 0; bi < order; bi++)
			for (int32_t bj = 0; bj < order; bj++)
				for (int32_t i = 0; i < base; i++)
					for (int32_t j = 0; j < base; j++)
						out[(bi * base + i) * dim + bj * base + j] = m[bi * order + bj] * small[i * base + j];
		free(m);
	}
	return 1;
}

/* kaiser_low_pass_filter (math.c:125-142), FP32 with FP64 Bessel. */
void bfo_kaiser_low_pass(float cutoff_frequency, float sampling_frequency, float beta,
                         int32_t length, float *out)
{
	float wc      = 2 * BFO_PI_F * cutoff_frequency / sampling_frequency;
	float a       = (float)length / 2.0f;
	float pi_i0_b = BFO_PI_F * (float)bfo_i0(beta);
	for (int32_t n = 0; n < length; n++) {
		float t = (float)n - a;
		/* f32_cmp(t, 0) of util.h:87 with F32_EPSILON 1e-6 */
		float at = t < 0 ? -t : t;
		int   eq = at <= 1e-6f * (at > 1.0f ? at : 1.0f);
		float impulse = !eq ? sinf(wc * t) / t : wc;
		t = t / a;
		float window = (float)bfo_i0(beta * sqrtf(1 - t * t)) / pi_i0_b;
		out[n] = impulse * window;
	}
}

void bfo_kaiser_low_pass_f64(double cutoff_frequency, double sampling_frequency, double beta,
                             int32_t length, double *out)
{
	double wc = 2 * BFO_PI_D * cutoff_frequency / sampling_frequency;
	double a  = (double)length / 2.0;
	double pi_i0_b = BFO_PI_D * bfo_i0(beta);
	for (int32_t n = 0; n < length; n++) {
		double t = (double)n - a;
		double impulse = (t != 0) ? sin(wc * t) / t : wc;
		t = t / a;
		out[n] = impulse * bfo_i0(beta * sqrt(1 - t * t)) / pi_i0_b;
	}
}

/* matched_filter (math.c:144-181): time-reversed (Hann-windowed one-cycle sine
 * convolved with the transmit sine) / length. */
void bfo_matched_filter(float xdc_center_frequency, float transmit_frequency,
                        float sampling_frequency, int32_t length, float *out)
{
	float *impulse  = (float *)calloc((size_t)length, sizeof(float));
	float *transmit = (float *)calloc((size_t)length, sizeof(float));
	for (int32_t i = 0; i < length; i++) out[i] = 0;
	{
		float wc = 2 * BFO_PI_F * xdc_center_frequency / sampling_frequency;
		int32_t impulse_length = (int32_t)ceilf(sampling_frequency / xdc_center_frequency);
		float ha = 2 * BFO_PI_F / (float)(impulse_length - 1);
		for (int32_t i = 0; i < impulse_length && i < length; i++) {
			float value  = sinf(wc * (float)i);
			float window = 0.5f - 0.5f * cosf(ha * (float)i);
			impulse[i] = value * window;
		}
	}
	{
		float wc = 2 * BFO_PI_F * transmit_frequency / sampling_frequency;
		for (int32_t i = 0; i < length; i++) transmit[i] = sinf(wc * (float)i);
	}
	for (int32_t i = 0; i < length; i++)
		for (int32_t j = 0; j < length; j++)
			if (i - j >= 0)
				out[length - 1 - i] += impulse[j] * transmit[i - j] / (float)length;
	free(impulse);
	free(transmit);
}

/* --------------------------- 4x4 column-major ------------------------------ */
typedef struct { float c[4][4]; } m4f;

static m4f m4_ident(void) { m4f r; memset(&r, 0, sizeof r); for (int i = 0; i < 4; i++) r.c[i][i] = 1; return r; }
static m4f m4_translate(float x, float y, float z) { m4f r = m4_ident(); r.c[3][0] = x; r.c[3][1] = y; r.c[3][2] = z; return r; }
static m4f m4_scale3(float x, float y, float z) { m4f r = m4_ident(); r.c[0][0] = x; r.c[1][1] = y; r.c[2][2] = z; return r; }
/* m4_mul (math.c:444-453): r.c[i][j] = dot(row_j(a), b.c[i]), dot left to right. */
static m4f m4_mul(m4f a, m4f b)
{
	m4f r;
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++)
			r.c[i][j] = a.c[0][j] * b.c[i][0] + a.c[1][j] * b.c[i][1] + a.c[2][j] * b.c[i][2] + a.c[3][j] * b.c[i][3];
	return r;
}
/* m4_rotation_about_z (math.c:510-521). */
static m4f m4_rot_z(float turns)
{
	float sa = sinf(turns * 2 * BFO_PI_F);
	float ca = cosf(turns * 2 * BFO_PI_F);
	m4f r = m4_ident();
	r.c[0][0] = ca; r.c[0][1] = -sa;
	r.c[1][0] = sa; r.c[1][1] = ca;
	return r;
}

/* das_voxel_transform_matrix (beamformer.c:483-518). */
void bfo_voxel_transform(const BeamformerParameters *bp, float out[16])
{
	float mn[3], ext[3], pts[3];
	for (int i = 0; i < 3; i++) {
		mn[i]  = bp->output_min_coordinate[i];
		float d = bp->output_max_coordinate[i] - bp->output_min_coordinate[i];
		ext[i] = d < 0 ? -d : d;
		pts[i] = (float)bp->output_points[i];
	}
	m4f T1 = m4_translate((pts[0] - 1.0f) * -0.5f, (pts[1] - 1.0f) * -0.5f, (pts[2] - 1.0f) * -0.5f);
	m4f T2 = m4_translate(mn[0] + ext[0] * 0.5f, mn[1] + ext[1] * 0.5f, mn[2] + ext[2] * 0.5f);
	m4f S  = m4_scale3(ext[0] / pts[0], ext[1] / pts[1], ext[2] / pts[2]);
	m4f R;
	switch (bp->das_shader_id) {
	case DASShaderKind_FORCES: case DASShaderKind_UFORCES: case DASShaderKind_FLASH:
		R = m4_ident();
		S.c[1][1]  = 0;
		T2.c[3][1] = 0;
		break;
	case DASShaderKind_HERCULES: case DASShaderKind_UHERCULES:
	case DASShaderKind_RCA_TPW: case DASShaderKind_RCA_VLS:
		R = m4_rot_z(bp->beamform_plane ? 0.0f : 0.25f);
		if (!(pts[0] > 1 && pts[1] > 1 && pts[2] > 1)) T2.c[3][1] = bp->off_axis_pos;
		break;
	default:
		R = m4_ident();
		break;
	}
	m4f M = m4_mul(R, m4_mul(T2, m4_mul(S, T1)));
	memcpy(out, M.c, sizeof(M.c));
}

void bfo_voxel_transform_f64(const BeamformerParameters *bp, double out[16])
{
	float f[16];
	bfo_voxel_transform(bp, f);
	for (int i = 0; i < 16; i++) out[i] = (double)f[i];
}

static uint32_t round_up_pow2(uint32_t a)
{
	uint32_t r = 1;
	while (r < a) r <<= 1;
	return r;
}

/* alloc_beamform_frame (beamformer.c:134-135). */
int32_t bfo_frame_mips(const int32_t dims[3])
{
	uint32_t m = (uint32_t)dims[0];
	if ((uint32_t)dims[1] > m) m = (uint32_t)dims[1];
	if ((uint32_t)dims[2] > m) m = (uint32_t)dims[2];
	uint32_t p = round_up_pow2(m);
	int32_t c = 0;
	while (!(p & 1u)) { p >>= 1; c++; }
	return c + 1;
}

/* ================================ planning ================================== */
static uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

/* plan_compute_pipeline (beamformer.c:303-481). The one intentional difference:
 * the Int16 halving of the decode dispatch width (beamformer.c:420) is applied
 * only when the data kind really is Int16 (the reference tests a field that is
 * never assigned, so it always halves). */
void bfo_plan(const BeamformerParameters *in, const int32_t *shaders, const uint8_t *slots,
              int32_t shader_count, int32_t data_kind, const BfoFilterSpec filters[4], BfoPlan *cp)
{
	memset(cp, 0, sizeof(*cp));
	BeamformerParameters *bp = &cp->das;
	*bp = *in;

	int decode_first = shader_count > 0 &&
	                   (shaders[0] == BeamformerShaderKind_Decode || shaders[0] == BeamformerShaderKind_CudaDecode);
	int cuda_hilbert = 0, demodulate = 0;
	for (int i = 0; i < shader_count; i++) {
		if (shaders[i] == BeamformerShaderKind_CudaHilbert) cuda_hilbert = 1;
		if (shaders[i] == BeamformerShaderKind_Demodulate)  demodulate = 1;
	}
	if (demodulate) cuda_hilbert = 0;

	for (int i = 0; i < shader_count; i++) {
		int32_t shader = shaders[i];
		int commit = 0;
		uint8_t slot = slots ? slots[i] : 0;
		switch (shader) {
		case BeamformerShaderKind_CudaHilbert: commit = cuda_hilbert; break;
		case BeamformerShaderKind_CudaDecode:
		case BeamformerShaderKind_Decode: {
			if (decode_first && demodulate) {
				shader = BeamformerShaderKind_DecodeInt16ToFloat;
			} else if (decode_first) {
				static const int32_t table[4] = {
					BeamformerShaderKind_Decode, BeamformerShaderKind_DecodeInt16Complex,
					BeamformerShaderKind_DecodeFloat, BeamformerShaderKind_DecodeFloatComplex,
				};
				int32_t k = data_kind < 0 ? 0 : data_kind > 3 ? 3 : data_kind;
				shader = table[k];
			} else {
				shader = data_kind == BeamformerDataKind_Int16 ? BeamformerShaderKind_DecodeInt16Complex
				                                               : BeamformerShaderKind_DecodeFloatComplex;
			}
			commit = 1;
		} break;
		case BeamformerShaderKind_Demodulate:
			if (decode_first || data_kind == BeamformerDataKind_Float32)
				shader = BeamformerShaderKind_DemodulateFloat;
			/* fall through */
		case BeamformerShaderKind_Filter: {
			const BfoFilterSpec *f = filters + (slot % BEAMFORMER_FILTER_SLOTS);
			if (f->length > 0)
				bp->time_offset += (float)f->length / 2.0f / f->sampling_frequency;
			commit = 1;
		} break;
		case BeamformerShaderKind_DAS:
			if (!bp->coherency_weighting) shader = BeamformerShaderKind_DASFast;
			commit = 1;
			break;
		default: commit = 1; break;
		}
		if (commit) {
			int idx = cp->shader_count++;
			cp->shaders[idx] = shader;
			cp->filter_slots[idx] = slot;
		}
	}

	uint32_t das_sample_stride   = 1;
	uint32_t das_transmit_stride = bp->dec_data_dim[0];
	uint32_t das_channel_stride  = bp->dec_data_dim[2] * bp->dec_data_dim[0];

	bp->decimation_rate = bp->decimation_rate > 1 ? bp->decimation_rate : 1;
	if (demodulate) {
		das_channel_stride  /= (2 * bp->decimation_rate);
		das_transmit_stride /= (2 * bp->decimation_rate);
	}

	uint32_t input_sample_stride   = 1;
	uint32_t input_transmit_stride = bp->dec_data_dim[0];
	uint32_t input_channel_stride  = bp->rf_raw_dim[0];

	BfoDecodeUBO *dp = &cp->decode;
	dp->decode_mode    = bp->decode;
	dp->transmit_count = bp->dec_data_dim[2];
	dp->input_sample_stride    = decode_first ? input_sample_stride   : bp->dec_data_dim[2];
	dp->input_channel_stride   = decode_first ? input_channel_stride  : das_channel_stride;
	dp->input_transmit_stride  = decode_first ? input_transmit_stride : 1;
	dp->output_sample_stride   = das_sample_stride;
	dp->output_channel_stride  = das_channel_stride;
	dp->output_transmit_stride = das_transmit_stride;
	if (decode_first) {
		dp->output_channel_stride  *= bp->decimation_rate;
		dp->output_transmit_stride *= bp->decimation_rate;
	}

	if (!demodulate) bp->center_frequency = 0;

	cp->decode_dispatch[0] = ceil_div(bp->dec_data_dim[0], 4);
	cp->decode_dispatch[1] = bp->dec_data_dim[1];
	cp->decode_dispatch[2] = ceil_div(bp->dec_data_dim[2], 16);
	if (decode_first && data_kind == BeamformerDataKind_Int16)
		cp->decode_dispatch[0] = ceil_div(cp->decode_dispatch[0], 2);

	if (demodulate) {
		BfoFilterUBO *mp = &cp->demod;
		mp->demodulation_frequency = bp->center_frequency;
		mp->sampling_frequency     = bp->sampling_frequency / 2;
		mp->decimation_rate        = bp->decimation_rate;
		mp->map_channels           = !decode_first;

		uint32_t dec0_in = bp->dec_data_dim[0];
		bp->sampling_frequency /= 2 * (float)mp->decimation_rate;
		bp->dec_data_dim[0]    /= 2 * mp->decimation_rate;

		if (decode_first) {
			mp->input_channel_stride   = dp->output_channel_stride;
			mp->input_sample_stride    = dp->output_sample_stride;
			mp->input_transmit_stride  = dp->output_transmit_stride;
			mp->output_channel_stride  = das_channel_stride;
			mp->output_sample_stride   = das_sample_stride;
			mp->output_transmit_stride = das_transmit_stride;
		} else {
			mp->input_channel_stride   = input_channel_stride / 2;
			mp->input_sample_stride    = input_sample_stride;
			mp->input_transmit_stride  = dec0_in / 2;
			mp->output_channel_stride  = dp->input_channel_stride;
			mp->output_sample_stride   = dp->input_sample_stride;
			mp->output_transmit_stride = dp->input_transmit_stride;
			cp->decode_dispatch[0] = ceil_div(bp->dec_data_dim[0], 4);
		}
		cp->demod_dispatch[0] = ceil_div(bp->dec_data_dim[0], 64);
		cp->demod_dispatch[1] = bp->dec_data_dim[1];
		cp->demod_dispatch[2] = bp->dec_data_dim[2];
	} else {
		cp->demod_dispatch[0] = ceil_div(bp->dec_data_dim[0], 64);
		cp->demod_dispatch[1] = bp->dec_data_dim[1];
		cp->demod_dispatch[2] = bp->dec_data_dim[2];
	}
	cp->rf_size = bp->dec_data_dim[0] * bp->dec_data_dim[1] * bp->dec_data_dim[2] * 8;

	BfoFilterUBO *flt = &cp->filter;
	flt->demodulation_frequency = bp->center_frequency;
	flt->sampling_frequency     = bp->sampling_frequency;
	flt->decimation_rate        = 1;
	flt->map_channels           = 0;
	flt->output_channel_stride  = bp->dec_data_dim[0] * bp->dec_data_dim[2];
	flt->output_sample_stride   = 1;
	flt->output_transmit_stride = bp->dec_data_dim[0];
	flt->input_channel_stride   = bp->dec_data_dim[0] * bp->dec_data_dim[2];
	flt->input_sample_stride    = 1;
	flt->input_transmit_stride  = bp->dec_data_dim[0];
}

/* ================================= decode =================================== */

/* decode.glsl:57-105. Sums of +-1 times int16 are exact integers, accumulated in
 * float as the shader does (exact below 2^24), divided once by the order. */
void bfo_decode(const BfoDecodeUBO *u, int32_t variant, int32_t first_stage, int32_t data_kind,
                const void *in, uint64_t in_bytes, void *out, uint64_t out_bytes,
                const int32_t *H, int32_t N, const int16_t *chmap, const uint32_t dispatch[3],
                int32_t threads)
{
	(void)data_kind;
	int rspi = 1;           /* RF samples per index */
	int in_kind;            /* 0 int32-packed int16 pair, 1 int16 complex pair, 2 float, 3 float2 */
	switch (variant) {
	case BeamformerShaderKind_DecodeFloat:        in_kind = 2; break;
	case BeamformerShaderKind_DecodeFloatComplex: in_kind = 3; break;
	case BeamformerShaderKind_DecodeInt16Complex: in_kind = 1; break;
	default:                                      in_kind = 0; rspi = 2; break;
	}
	int to_float = variant == BeamformerShaderKind_DecodeInt16ToFloat;
	uint32_t T = u->transmit_count;
	uint64_t elem_bytes = (in_kind == 3) ? 8 : 4;
	uint64_t in_elems   = in_bytes / elem_bytes;
	uint64_t out_vec2   = out_bytes / 8;
	float   *outf       = (float *)out;
	uint32_t xs = dispatch[0] * 4, cs = dispatch[1];
	uint32_t ts = dispatch[2] * 16;
	if (ts > T) ts = T; /* transmits beyond the Hadamard order are not decoded */

	/* pass 1: gather the raw data into [channel][sample index][transmit] */
	uint64_t scratch_elems = 0;
	void *scratch = 0;
	const void *src = in;
	if (first_stage) {
		scratch_elems = ((uint64_t)u->input_channel_stride * cs + (uint64_t)T * xs * rspi) / (uint64_t)rspi + T;
		scratch = calloc(scratch_elems, elem_bytes);
		#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
		for (int64_t c = 0; c < (int64_t)cs; c++) {
			for (uint32_t t = 0; t < ts; t++) {
				for (uint32_t x = 0; x < xs; x++) {
					uint32_t s = x * rspi;
					if (s >= u->input_transmit_stride) continue;
					uint64_t rf_offset = ((uint64_t)u->input_channel_stride * c + (uint64_t)T * s) / rspi;
					int32_t mc = chmap ? chmap[c] : (int32_t)c;
					uint64_t in_off = (uint64_t)u->input_channel_stride * (uint64_t)mc +
					                  (uint64_t)u->input_transmit_stride * t + (uint64_t)u->input_sample_stride * s;
					uint64_t si = in_off / rspi, di = rf_offset + t;
					if (di >= scratch_elems) continue;
					if (si < in_elems)
						memcpy((char *)scratch + di * elem_bytes, (const char *)in + si * elem_bytes, elem_bytes);
				}
			}
		}
		src = scratch;
	}
	uint64_t src_elems = first_stage ? scratch_elems : in_elems;

	/* pass 2: dot product with Hadamard row t */
	#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int64_t c = 0; c < (int64_t)cs; c++) {
		for (uint32_t t = 0; t < ts; t++) {
			for (uint32_t x = 0; x < xs; x++) {
				uint32_t s = x * rspi;
				uint64_t rf_offset = ((uint64_t)u->input_channel_stride * c + (uint64_t)T * s) / rspi;
				uint32_t ts_out = to_float ? x : s;
				if (ts_out >= u->output_transmit_stride) continue;
				uint64_t out_off = (uint64_t)u->output_channel_stride * c + (uint64_t)u->output_transmit_stride * t +
				                   (uint64_t)u->output_sample_stride * ts_out;
				float r[4] = {0, 0, 0, 0};
				uint32_t n_terms = u->decode_mode == DECODE_MODE_HADAMARD ? (uint32_t)N : 1;
				for (uint32_t i = 0; i < n_terms; i++) {
					uint64_t idx = u->decode_mode == DECODE_MODE_HADAMARD ? rf_offset + i : rf_offset + t;
					float v[4] = {0, 0, 0, 0};
					if (idx < src_elems) {
						const char *p = (const char *)src + idx * elem_bytes;
						if (in_kind == 0) {
							int32_t w; memcpy(&w, p, 4);
							int16_t lo = (int16_t)(w & 0xFFFF), hi = (int16_t)((uint32_t)w >> 16);
							v[0] = lo; v[1] = hi;
						} else if (in_kind == 1) {
							int32_t w; memcpy(&w, p, 4);
							int16_t lo = (int16_t)(w & 0xFFFF), hi = (int16_t)((uint32_t)w >> 16);
							v[0] = lo; v[1] = hi;
						} else if (in_kind == 2) {
							memcpy(&v[0], p, 4);
						} else {
							memcpy(&v[0], p, 8);
						}
					}
					if (u->decode_mode == DECODE_MODE_HADAMARD) {
						float h = (float)H[(uint64_t)t * (uint64_t)N + i];
						r[0] += h * v[0];
						r[1] += h * v[1];
					} else {
						r[0] = v[0];
						r[1] = v[1];
					}
				}
				if (u->decode_mode == DECODE_MODE_HADAMARD) {
					r[0] = r[0] / (float)N;
					r[1] = r[1] / (float)N;
				}
				if (in_kind == 0 && !to_float) {
					/* two complex outputs (y_s, 0), (y_s+1, 0) */
					if (out_off < out_vec2)     { outf[2 * out_off] = r[0];     outf[2 * out_off + 1] = 0; }
					if (out_off + 1 < out_vec2) { outf[2 * out_off + 2] = r[1]; outf[2 * out_off + 3] = 0; }
				} else if (in_kind == 2) {
					if (out_off < out_vec2) { outf[2 * out_off] = r[0]; outf[2 * out_off + 1] = 0; }
				} else {
					if (out_off < out_vec2) { outf[2 * out_off] = r[0]; outf[2 * out_off + 1] = r[1]; }
				}
			}
		}
	}
	free(scratch);
}

/* ================================= filter =================================== */
static float snorm_unpack(int16_t v)
{
	float f = (float)v / 32767.0f;
	return f < -1.0f ? -1.0f : f > 1.0f ? 1.0f : f;
}
static int16_t snorm_pack(float v)
{
	float c = v < -1.0f ? -1.0f : v > 1.0f ? 1.0f : v;
	return (int16_t)roundf(c * 32767.0f);
}

/* filter.glsl:29-91. Demodulate variants multiply (I, -Q) by sqrt(2) and the
 * phasor of -index; Filter rotates each input by +out_sample and the result
 * back, exactly as written (the rotations cancel up to rounding). */
void bfo_filter(const BfoFilterUBO *u, int32_t variant, const void *in, uint64_t in_bytes,
                void *out, uint64_t out_bytes, const float *taps, int32_t L,
                const int16_t *chmap, const uint32_t dispatch[3], int32_t threads)
{
	int int16_io = variant == BeamformerShaderKind_Demodulate;
	int demod    = variant != BeamformerShaderKind_Filter;
	uint64_t in_elems  = in_bytes / (int16_io ? 4 : 8);
	uint64_t out_elems = out_bytes / (int16_io ? 4 : 8);
	const float r360 = 360.0f * BFO_DEG2RAD_F;
	const float rt2  = sqrtf(2.0f);
	uint32_t xs = dispatch[0] * 64, cs = dispatch[1], ts = dispatch[2];

	#pragma omp parallel for collapse(2) num_threads(nthreads(threads)) schedule(static)
	for (int64_t c = 0; c < (int64_t)cs; c++) {
		for (int64_t t = 0; t < (int64_t)ts; t++) {
			uint32_t in_channel = u->map_channels ? (uint32_t)(int32_t)chmap[c] : (uint32_t)c;
			uint64_t in_offset  = (uint64_t)u->input_channel_stride * in_channel + (uint64_t)u->input_transmit_stride * t;
			int32_t target = u->map_channels ? (int32_t)(u->output_channel_stride / u->output_sample_stride)
			                                 : (int32_t)u->output_transmit_stride;
			for (uint32_t x = 0; x < xs; x++) {
				uint32_t in_sample = x * u->decimation_rate, out_sample = x;
				if ((int32_t)out_sample >= target) continue;
				uint64_t out_offset = (uint64_t)u->output_channel_stride * c + (uint64_t)u->output_transmit_stride * t +
				                      (uint64_t)u->output_sample_stride * out_sample;
				int32_t index = (int32_t)in_sample - L;
				int32_t start = index < 0 ? -index : 0;
				index += start;
				int32_t limit = target * (int32_t)u->decimation_rate;
				float rx = 0, ry = 0;
				for (int32_t i = start; i < L && index < limit; i++, index++) {
					uint64_t si = in_offset + (uint64_t)index;
					float vx = 0, vy = 0;
					if (si < in_elems) {
						if (int16_io) {
							uint32_t w; memcpy(&w, (const char *)in + si * 4, 4);
							vx = snorm_unpack((int16_t)(w & 0xFFFF));
							vy = snorm_unpack((int16_t)(w >> 16));
						} else {
							memcpy(&vx, (const char *)in + si * 8, 4);
							memcpy(&vy, (const char *)in + si * 8 + 4, 4);
						}
					}
					float h = taps[L - i - 1];
					if (demod) {
						/* rotate_iq(v * (1,-1), -index), mat2(cos,-sin,sin,cos) column-major */
						float arg = r360 * u->demodulation_frequency * (float)(-index) / u->sampling_frequency;
						float ca = cosf(arg), sa = sinf(arg);
						float x0 = vx, y0 = -vy;
						float qx = ca * x0 + sa * y0;
						float qy = -sa * x0 + ca * y0;
						qx = rt2 * qx; qy = rt2 * qy;
						rx += qx * h; ry += qy * h;
					} else {
						float arg = r360 * u->demodulation_frequency * (float)(int32_t)out_sample / u->sampling_frequency;
						float ca = cosf(arg), sa = sinf(arg);
						float qx = ca * vx + sa * vy;
						float qy = -sa * vx + ca * vy;
						rx += qx * h; ry += qy * h;
					}
				}
				if (!demod) {
					float arg = r360 * u->demodulation_frequency * (float)(-(int32_t)out_sample) / u->sampling_frequency;
					float ca = cosf(arg), sa = sinf(arg);
					float qx = ca * rx + sa * ry;
					float qy = -sa * rx + ca * ry;
					rx = qx; ry = qy;
				}
				if (out_offset < out_elems) {
					if (int16_io) {
						uint32_t w = (uint32_t)(uint16_t)snorm_pack(rx) | ((uint32_t)(uint16_t)snorm_pack(ry) << 16);
						memcpy((char *)out + out_offset * 4, &w, 4);
					} else {
						((float *)out)[2 * out_offset]     = rx;
						((float *)out)[2 * out_offset + 1] = ry;
					}
				}
			}
		}
	}
}

/* FP64 demodulate/filter on float2 data (error reference). */
void bfo_filter_f64(const BfoFilterUBO *u, int32_t variant, const double *in, uint64_t in_count,
                    double *out, uint64_t out_count, const double *taps, int32_t L,
                    const uint32_t dispatch[3], int32_t threads)
{
	int demod = variant != BeamformerShaderKind_Filter;
	const double r360 = 2.0 * BFO_PI_D;
	const double rt2  = sqrt(2.0);
	uint32_t xs = dispatch[0] * 64, cs = dispatch[1], ts = dispatch[2];
	#pragma omp parallel for collapse(2) num_threads(nthreads(threads)) schedule(static)
	for (int64_t c = 0; c < (int64_t)cs; c++) {
		for (int64_t t = 0; t < (int64_t)ts; t++) {
			uint64_t in_offset = (uint64_t)u->input_channel_stride * c + (uint64_t)u->input_transmit_stride * t;
			int32_t target = (int32_t)u->output_transmit_stride;
			for (uint32_t x = 0; x < xs; x++) {
				uint32_t in_sample = x * u->decimation_rate, out_sample = x;
				if ((int32_t)out_sample >= target) continue;
				uint64_t out_offset = (uint64_t)u->output_channel_stride * c + (uint64_t)u->output_transmit_stride * t +
				                      (uint64_t)u->output_sample_stride * out_sample;
				int32_t index = (int32_t)in_sample - L;
				int32_t start = index < 0 ? -index : 0;
				index += start;
				int32_t limit = target * (int32_t)u->decimation_rate;
				double rx = 0, ry = 0;
				for (int32_t i = start; i < L && index < limit; i++, index++) {
					uint64_t si = in_offset + (uint64_t)index;
					double vx = 0, vy = 0;
					if (si < in_count) { vx = in[2 * si]; vy = in[2 * si + 1]; }
					double h = taps[L - i - 1];
					if (demod) {
						double arg = r360 * (double)u->demodulation_frequency * (double)(-index) / (double)u->sampling_frequency;
						double ca = cos(arg), sa = sin(arg);
						double qx = ca * vx - sa * vy, qy = -sa * vx - ca * vy;
						rx += rt2 * qx * h; ry += rt2 * qy * h;
					} else {
						rx += vx * h; ry += vy * h;
					}
				}
				if (out_offset < out_count) { out[2 * out_offset] = rx; out[2 * out_offset + 1] = ry; }
			}
		}
	}
}

/* =================================== DAS ==================================== */
/* FP32 and FP64 instantiations of the same das.glsl restatement. */
#define BFO_REAL      float
#define BFO_SFX(n)    n
#define BFO_SQRT      sqrtf
#define BFO_COS       cosf
#define BFO_SIN       sinf
#define BFO_FABS      fabsf
#define BFO_ROUND     roundf
#define BFO_FLOOR     floorf
#define BFO_DEG2RAD   BFO_DEG2RAD_F
#include "bf_oracle_das.inc"
#undef BFO_REAL
#undef BFO_SFX
#undef BFO_SQRT
#undef BFO_COS
#undef BFO_SIN
#undef BFO_FABS
#undef BFO_ROUND
#undef BFO_FLOOR
#undef BFO_DEG2RAD

#define BFO_REAL      double
#define BFO_SFX(n)    n##_f64
#define BFO_SQRT      sqrt
#define BFO_COS       cos
#define BFO_SIN       sin
#define BFO_FABS      fabs
#define BFO_ROUND     round
#define BFO_FLOOR     floor
#define BFO_DEG2RAD   (BFO_PI_D / 180.0)
#include "bf_oracle_das.inc"

/* ================================ sum / min_max ============================= */
static uint32_t orone(uint32_t x) { return x ? x : 1; }

void bfo_sum(float *out, const float *const *ins, int32_t count, float prescale, const int32_t dims[3],
             int32_t threads)
{
	uint64_t X = (uint64_t)dims[0], Y = (uint64_t)dims[1], Z = (uint64_t)dims[2];
	uint64_t cx = 32ull * orone((uint32_t)X / 32u), cy = orone((uint32_t)Y), cz = 32ull * orone((uint32_t)Z / 32u);
	memset(out, 0, sizeof(float) * 2 * X * Y * Z);
	#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
	for (int64_t z = 0; z < (int64_t)Z; z++) {
		if ((uint64_t)z >= cz) continue;
		for (uint64_t y = 0; y < Y && y < cy; y++) {
			for (uint64_t x = 0; x < X && x < cx; x++) {
				uint64_t v = ((uint64_t)z * Y + y) * X + x;
				for (int32_t i = 0; i < count; i++) {
					float a = prescale * ins[i][2 * v];
					float b = prescale * ins[i][2 * v + 1];
					out[2 * v]     = out[2 * v] + a;
					out[2 * v + 1] = out[2 * v + 1] + b;
				}
			}
		}
	}
}

uint64_t bfo_min_max_levels_floats(const int32_t dims[3])
{
	int32_t mips = bfo_frame_mips(dims);
	uint64_t total = 0;
	for (int32_t l = 1; l < mips; l++) {
		uint64_t x = (uint64_t)dims[0] >> l, y = (uint64_t)dims[1] >> l, z = (uint64_t)dims[2] >> l;
		total += 2 * (x ? x : 1) * (y ? y : 1) * (z ? z : 1);
	}
	return total;
}

void bfo_min_max(const float *frame, const int32_t dims[3], float *levels_out, int32_t threads)
{
	int32_t mips = bfo_frame_mips(dims);
	const float *prev = frame;
	uint64_t pX = (uint64_t)dims[0], pY = (uint64_t)dims[1], pZ = (uint64_t)dims[2];
	float *cur = levels_out;
	for (int32_t l = 1; l < mips; l++) {
		uint32_t w = (uint32_t)dims[0] >> l, h = (uint32_t)dims[1] >> l, d = (uint32_t)dims[2] >> l;
		uint64_t X = w ? w : 1, Y = h ? h : 1, Z = d ? d : 1;
		uint64_t cx = 32ull * orone(w / 32), cy = orone(h), cz = 32ull * orone(d / 32);
		#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
		for (int64_t z = 0; z < (int64_t)Z; z++) {
			for (uint64_t y = 0; y < Y; y++) {
				for (uint64_t x = 0; x < X; x++) {
					uint64_t o = ((uint64_t)z * Y + y) * X + x;
					if (!(x < cx && y < cy && (uint64_t)z < cz)) { cur[2 * o] = NAN; cur[2 * o + 1] = NAN; continue; }
					float mn = 1000000000.0f, mx = 0.0f;
					for (int i = 0; i < 2; i++) {
						for (int j = 0; j < 2; j++) {
							for (int k = 0; k < 2; k++) {
								uint64_t ix = 2 * x + i, iy = 2 * y + j, iz = 2 * (uint64_t)z + k;
								float vx = 0, vy = 0;
								if (ix < pX && iy < pY && iz < pZ) {
									uint64_t pi = (iz * pY + iy) * pX + ix;
									vx = prev[2 * pi]; vy = prev[2 * pi + 1];
								}
								mn = fminf(mn, vx);
								mx = fmaxf(mx, vy);
							}
						}
					}
					cur[2 * o] = mn; cur[2 * o + 1] = mx;
				}
			}
		}
		prev = cur;
		pX = X; pY = Y; pZ = Z;
		cur += 2 * X * Y * Z;
	}
}
