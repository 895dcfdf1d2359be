/*
 * bf_host.cpp -- host math and pipeline planning of the library.
 *
 *   plan_pipeline    restates plan_compute_pipeline (beamformer.c:303-481)
 *   hadamard_matrix  make_hadamard_transpose (math.c:33-122)
 *   kaiser_low_pass  kaiser_low_pass_filter (math.c:125-142)
 *   matched_filter   matched_filter (math.c:144-181)
 *   bessel_i0        cephes_i0 (external/cephes.c:24-103; Cephes 2.8 expansion)
 *   voxel_transform  das_voxel_transform_matrix (beamformer.c:483-518)
 *   frame_mips       alloc_beamform_frame mip count (beamformer.c:134-135)
 *
 * Compiled with -ffp-contract=off: the voxel transform and the constants derived
 * on the host feed the DAS delay chain and must round exactly as the reference's
 * expressions do.
 */
#include "bf_host.h"

#include <cmath>
#include <cstring>

namespace bf {

static constexpr float PI_F = 3.14159265358979323846f;

/* ------------------------------ Hadamard --------------------------------- */
static int legendre(int k, int q)
{
	k %= q;
	if (k < 0) k += q;
	if (k == 0) return 0;
	for (int x = 1; x < q; x++)
		if ((x * x) % q == k) return 1;
	return -1;
}

/* Bordered Paley matrix of order q + 1 (q = 11 or 19) in the orientation of the
 * reference's tables: first row/column +1, core -chi_q(k) off the diagonal and
 * -1 on it, rows cyclically shifted right (q = 11) or left (q = 19). */
static void paley(int q, std::vector<int8_t> &m)
{
	const int n = q + 1;
	m.assign((size_t)n * n, 1);
	for (int i = 1; i < n; i++) {
		for (int j = 1; j < n; j++) {
			int k = (q == 11) ? (j - i) : (j + i - 2);
			k %= q;
			if (k < 0) k += q;
			m[(size_t)i * n + j] = (int8_t)(k == 0 ? -1 : -legendre(k, q));
		}
	}
}

static bool pow2(int32_t a) { return a > 0 && (a & (a - 1)) == 0; }

bool hadamard_matrix(int32_t order, std::vector<int8_t> &out, int32_t &sylvester, int32_t &base)
{
	sylvester = 0; base = 0;
	if (order <= 0) return false;
	if (pow2(order))                               { base = 1;  sylvester = order; }
	else if (order % 20 == 0 && pow2(order / 20))  { base = 20; sylvester = order / 20; }
	else if (order % 12 == 0 && pow2(order / 12))  { base = 12; sylvester = order / 12; }
	else return false;

	/* Sylvester: S_2k = [[S, S], [S, -S]] */
	std::vector<int8_t> s((size_t)sylvester * sylvester);
	s[0] = 1;
	for (int32_t k = 1; k < sylvester; k *= 2)
		for (int32_t i = 0; i < k; i++)
			for (int32_t j = 0; j < k; j++) {
				int8_t v = s[(size_t)i * sylvester + j];
				s[(size_t)(i + k) * sylvester + j] = v;
				s[(size_t)i * sylvester + j + k] = v;
				s[(size_t)(i + k) * sylvester + j + k] = (int8_t)-v;
			}
	if (base == 1) { out = s; return true; }

	std::vector<int8_t> b;
	paley(base - 1, b);
	out.assign((size_t)order * order, 0);
	for (int32_t bi = 0; bi < sylvester; bi++)
		for (int32_t bj = 0; bj < sylvester; bj++)
			for (int32_t i = 0; i < base; i++)
				for (int32_t j = 0; j < base; j++)
					out[(size_t)(bi * base + i) * order + bj * base + j] =
						(int8_t)(s[(size_t)bi * sylvester + bj] * b[(size_t)i * base + j]);
	return true;
}

/* --------------------------- filters and I0 ------------------------------ */
static double cheb(double x, const double *c, int n)
{
	double b0 = c[0], b1 = 0.0, b2 = 0.0;
	for (int i = 1; i < n; i++) { b2 = b1; b1 = b0; b0 = x * b1 - b2 + c[i]; }
	return 0.5 * (b0 - b2);
}

double bessel_i0(double x)
{
	/* Cephes 2.8 Chebyshev coefficients: exp(-x) I0(x) on [0, 8] ... */
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
	/* ... and exp(-x) sqrt(x) I0(x) on (8, inf) in 32/x - 2 */
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
	x = std::fabs(x);
	if (x <= 8.0) return std::exp(x) * cheb(x / 2.0 - 2.0, A, 30);
	return std::exp(x) * cheb(32.0 / x - 2.0, B, 25) / std::sqrt(x);
}

void kaiser_low_pass(float cutoff, float fs, float beta, int32_t length, float *out)
{
	const float wc = 2 * PI_F * cutoff / fs;
	const float a = (float)length / 2.0f;
	const float norm = PI_F * (float)bessel_i0(beta);
	for (int32_t n = 0; n < length; n++) {
		float t = (float)n - a;
		float at = std::fabs(t);
		bool zero = at <= 1e-6f * (at > 1.0f ? at : 1.0f);   /* util.h f32_cmp(t, 0) */
		float impulse = zero ? wc : sinf(wc * t) / t;
		t = t / a;
		out[n] = impulse * ((float)bessel_i0(beta * sqrtf(1 - t * t)) / norm);
	}
}

void matched_filter(float xdc_fc, float tx_f, float fs, int32_t length, float *out)
{
	std::vector<float> impulse((size_t)length, 0.0f), tx((size_t)length, 0.0f);
	for (int32_t i = 0; i < length; i++) out[i] = 0;
	const float wc = 2 * PI_F * xdc_fc / fs;
	const int32_t ilen = (int32_t)ceilf(fs / xdc_fc);
	const float ha = 2 * PI_F / (float)(ilen - 1);
	for (int32_t i = 0; i < ilen && i < length; i++)
		impulse[(size_t)i] = sinf(wc * (float)i) * (0.5f - 0.5f * cosf(ha * (float)i));
	const float wt = 2 * PI_F * tx_f / fs;
	for (int32_t i = 0; i < length; i++) tx[(size_t)i] = sinf(wt * (float)i);
	for (int32_t i = 0; i < length; i++)
		for (int32_t j = 0; j <= i; j++)
			out[length - 1 - i] += impulse[(size_t)j] * tx[(size_t)(i - j)] / (float)length;
}

/* ---------------------------- voxel transform ---------------------------- */
struct M4 { float c[4][4]; };

static M4 identity() { M4 m{}; for (int i = 0; i < 4; i++) m.c[i][i] = 1; return m; }
static M4 mul(const M4 &a, const M4 &b)
{
	M4 r;
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) {
			float s = a.c[0][j] * b.c[i][0];
			s = s + a.c[1][j] * b.c[i][1];
			s = s + a.c[2][j] * b.c[i][2];
			s = s + a.c[3][j] * b.c[i][3];
			r.c[i][j] = s;
		}
	return r;
}

void voxel_transform(const BeamformerParameters &bp, float out[16])
{
	float lo[3], ext[3], pts[3];
	for (int i = 0; i < 3; i++) {
		lo[i] = bp.output_min_coordinate[i];
		ext[i] = std::fabs(bp.output_max_coordinate[i] - bp.output_min_coordinate[i]);
		pts[i] = (float)bp.output_points[i];
	}
	M4 T1 = identity(), T2 = identity(), S = identity(), R = identity();
	for (int i = 0; i < 3; i++) {
		T1.c[3][i] = (pts[i] - 1.0f) * -0.5f;
		T2.c[3][i] = lo[i] + ext[i] * 0.5f;
		S.c[i][i]  = ext[i] / pts[i];
	}
	switch (bp.das_shader_id) {
	case DASShaderKind_FORCES: case DASShaderKind_UFORCES: case DASShaderKind_FLASH:
		S.c[1][1] = 0;
		T2.c[3][1] = 0;
		break;
	case DASShaderKind_HERCULES: case DASShaderKind_UHERCULES:
	case DASShaderKind_RCA_TPW: case DASShaderKind_RCA_VLS: {
		float turns = bp.beamform_plane ? 0.0f : 0.25f;
		float sa = sinf(turns * 2 * PI_F), ca = cosf(turns * 2 * PI_F);
		R.c[0][0] = ca; R.c[0][1] = -sa;
		R.c[1][0] = sa; R.c[1][1] = ca;
		if (!(pts[0] > 1 && pts[1] > 1 && pts[2] > 1)) T2.c[3][1] = bp.off_axis_pos;
	} break;
	default: break;
	}
	M4 m = mul(R, mul(T2, mul(S, T1)));
	std::memcpy(out, m.c, sizeof(m.c));
}

int32_t frame_mips(const int32_t dims[3])
{
	uint32_t m = 1;
	for (int i = 0; i < 3; i++) m = (uint32_t)dims[i] > m ? (uint32_t)dims[i] : m;
	uint32_t p = 1;
	int32_t levels = 1;
	while (p < m) { p <<= 1; levels++; }
	return levels;
}

/* -------------------------------- planning ------------------------------- */
static uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

void plan_pipeline(const BeamformerParameters &in, const int32_t *shaders, const uint8_t *slots, int32_t count,
                   int32_t data_kind, const FilterSpec filters[BEAMFORMER_FILTER_SLOTS], Plan &pl)
{
	pl = Plan{};
	BeamformerParameters &bp = pl.das;
	bp = in;

	const bool decode_first = count > 0 && (shaders[0] == BeamformerShaderKind_Decode ||
	                                        shaders[0] == BeamformerShaderKind_CudaDecode);
	bool hilbert = false, demod = false;
	for (int32_t i = 0; i < count; i++) {
		hilbert |= shaders[i] == BeamformerShaderKind_CudaHilbert;
		demod   |= shaders[i] == BeamformerShaderKind_Demodulate;
	}
	if (demod) hilbert = false;
	pl.decode_first = decode_first;
	pl.demodulate = demod;

	for (int32_t i = 0; i < count; i++) {
		int32_t kind = shaders[i];
		uint8_t slot = slots[i];
		bool keep = true;
		switch (kind) {
		case BeamformerShaderKind_CudaHilbert: keep = hilbert; break;
		case BeamformerShaderKind_CudaDecode:
		case BeamformerShaderKind_Decode:
			if (decode_first && demod) kind = BeamformerShaderKind_DecodeInt16ToFloat;
			else if (decode_first) {
				switch (data_kind) {
				case BeamformerDataKind_Int16Complex:   kind = BeamformerShaderKind_DecodeInt16Complex; break;
				case BeamformerDataKind_Float32:        kind = BeamformerShaderKind_DecodeFloat; break;
				case BeamformerDataKind_Float32Complex: kind = BeamformerShaderKind_DecodeFloatComplex; break;
				default:                                kind = BeamformerShaderKind_Decode; break;
				}
			} else {
				kind = data_kind == BeamformerDataKind_Int16 ? BeamformerShaderKind_DecodeInt16Complex
				                                             : BeamformerShaderKind_DecodeFloatComplex;
			}
			break;
		case BeamformerShaderKind_Demodulate:
			if (decode_first || data_kind == BeamformerDataKind_Float32) kind = BeamformerShaderKind_DemodulateFloat;
			[[fallthrough]];
		case BeamformerShaderKind_Filter: {
			const FilterSpec &f = filters[slot % BEAMFORMER_FILTER_SLOTS];
			if (f.kind >= 0 && f.length > 0) bp.time_offset += (float)f.length / 2.0f / f.sampling_frequency;
		} break;
		case BeamformerShaderKind_DAS:
			if (!bp.coherency_weighting) kind = BeamformerShaderKind_DASFast;
			break;
		default: break;
		}
		if (keep) {
			pl.shaders[pl.count] = kind;
			pl.slots[pl.count] = slot;
			pl.count++;
		}
	}

	uint32_t das_ts = bp.dec_data_dim[0];
	uint32_t das_cs = bp.dec_data_dim[2] * bp.dec_data_dim[0];
	bp.decimation_rate = bp.decimation_rate > 1 ? bp.decimation_rate : 1;
	const uint32_t D = bp.decimation_rate;
	if (demod) { das_cs /= 2 * D; das_ts /= 2 * D; }

	Strides &ds = pl.decode_st;
	pl.decode_mode = bp.decode;
	pl.transmit_count = bp.dec_data_dim[2];
	ds.in_sample   = decode_first ? 1 : bp.dec_data_dim[2];
	ds.in_channel  = decode_first ? bp.rf_raw_dim[0] : das_cs;
	ds.in_transmit = decode_first ? bp.dec_data_dim[0] : 1;
	ds.out_sample = 1;
	ds.out_channel = das_cs;
	ds.out_transmit = das_ts;
	if (decode_first) { ds.out_channel *= D; ds.out_transmit *= D; }

	if (!demod) bp.center_frequency = 0;

	/* decode dispatch width (beamformer.c:415-421): groups of 4 invocations, halved
	 * for int16 data decoded first (two samples per invocation) */
	uint32_t dispatch_x = div_up(bp.dec_data_dim[0], 4);
	if (decode_first && data_kind == BeamformerDataKind_Int16) dispatch_x = div_up(dispatch_x, 2);
	if (demod) {
		pl.demod_frequency  = bp.center_frequency;
		pl.demod_fs         = bp.sampling_frequency / 2;
		pl.demod_decimation = D;
		pl.demod_map        = !decode_first;
		const uint32_t dec0_in = bp.dec_data_dim[0];
		bp.sampling_frequency /= 2 * (float)D;
		bp.dec_data_dim[0]    /= 2 * D;
		Strides &ms = pl.demod_st;
		if (decode_first) {
			ms.in_channel = ds.out_channel; ms.in_sample = ds.out_sample; ms.in_transmit = ds.out_transmit;
			ms.out_channel = das_cs; ms.out_sample = 1; ms.out_transmit = das_ts;
		} else {
			ms.in_channel = bp.rf_raw_dim[0] / 2; ms.in_sample = 1; ms.in_transmit = dec0_in / 2;
			ms.out_channel = ds.in_channel; ms.out_sample = ds.in_sample; ms.out_transmit = ds.in_transmit;
			dispatch_x = div_up(bp.dec_data_dim[0], 4);
		}
	}
	pl.decode_invocations_x = dispatch_x * 4;
	pl.demod_rows_x = bp.dec_data_dim[0];
	pl.rf_size = bp.dec_data_dim[0] * bp.dec_data_dim[1] * bp.dec_data_dim[2] * 8;

	pl.filter_frequency = bp.center_frequency;
	pl.filter_fs = bp.sampling_frequency;
	Strides &fs = pl.filter_st;
	fs.out_channel = bp.dec_data_dim[0] * bp.dec_data_dim[2];
	fs.out_sample = 1;
	fs.out_transmit = bp.dec_data_dim[0];
	fs.in_channel = fs.out_channel;
	fs.in_sample = 1;
	fs.in_transmit = bp.dec_data_dim[0];
}

} /* namespace bf */
