/*
 * ref_shader_driver.cpp -- runs the reference's compute shaders, compiled as C++
 * through glsl_shim.hpp, over the dispatch grids the reference issues for them.
 * TEST INFRASTRUCTURE ONLY: it is the reference side of the parity checks.
 *
 * The generated include (oracle/_ref/ref_shaders_gen.inc, written by
 * build_ref.py from the reference checkout) holds one C++ namespace per shader
 * variant. This file binds buffers/images/uniforms and loops over
 * gl_GlobalInvocationID the way do_compute_shader (beamformer.c:521-709) and
 * do_sum_shader (beamformer.c:218-235) dispatch them.
 */
#include "glsl_shim.hpp"
#include "ref_shaders_gen.inc"

#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

using namespace glsl;

template <class S> static void bind(S &s, const void *p, uint64_t bytes)
{
	using T = std::remove_reference_t<decltype(*s.p)>;
	s.p = (T *)const_cast<void *>(p);
	s.n = (int64_t)(bytes / sizeof(T));
}

/* invocation loop, parallel over the y (decode/filter) or z extent */
template <class F> static void dispatch(uint32_t nx, uint32_t ny, uint32_t nz, F body)
{
	#pragma omp parallel for collapse(2) schedule(static)
	for (int64_t z = 0; z < (int64_t)nz; z++) {
		for (int64_t y = 0; y < (int64_t)ny; y++) {
			for (uint32_t x = 0; x < nx; x++) {
				gl_GlobalInvocationID = uvec3{x, (uint)y, (uint)z};
				body();
			}
		}
	}
}

struct RefDecodeUBO {
	uint32_t input_channel_stride, input_sample_stride, input_transmit_stride;
	uint32_t output_channel_stride, output_sample_stride, output_transmit_stride;
	uint32_t transmit_count, decode_mode;
};
struct RefFilterUBO {
	uint32_t input_channel_stride, input_sample_stride, input_transmit_stride;
	uint32_t output_channel_stride, output_sample_stride, output_transmit_stride;
	uint32_t decimation_rate, map_channels;
	float demodulation_frequency, sampling_frequency;
};

#define SET_STRIDES(ns, u) do { \
	ns::input_channel_stride = u->input_channel_stride; ns::input_sample_stride = u->input_sample_stride; \
	ns::input_transmit_stride = u->input_transmit_stride; ns::output_channel_stride = u->output_channel_stride; \
	ns::output_sample_stride = u->output_sample_stride; ns::output_transmit_stride = u->output_transmit_stride; \
} while (0)

/* decode.glsl: both passes for the first stage (beamformer.c:534-561). */
template <int Which> static void run_decode(const RefDecodeUBO *u, int first_stage, const void *in, uint64_t in_bytes,
                                            void *scratch, uint64_t scratch_bytes, void *out, uint64_t out_bytes,
                                            const int8_t *hadamard, int n, const int16_t *chmap, const uint32_t d[3])
{
#define DECODE_BODY(ns) do { \
	SET_STRIDES(ns, u); ns::transmit_count = u->transmit_count; ns::decode_mode = u->decode_mode; \
	ns::hadamard = iimage2D{hadamard, n, n}; ns::channel_mapping = iimage1D{chmap, 256}; \
	uint32_t X = d[0] * 4, Y = d[1], Z = d[2] * 16; \
	if (first_stage) { \
		bind(ns::rf_data, in, in_bytes); bind(ns::out_rf_data, scratch, scratch_bytes); \
		ns::u_first_pass = true; dispatch(X, Y, Z, [] { ns::shader_main(); }); \
		bind(ns::rf_data, scratch, scratch_bytes); \
	} else { \
		bind(ns::rf_data, in, in_bytes); \
	} \
	bind(ns::out_data, out, out_bytes); ns::u_first_pass = false; \
	dispatch(X, Y, Z, [] { ns::shader_main(); }); \
} while (0)
	if constexpr (Which == 0) DECODE_BODY(decode_i16);
	if constexpr (Which == 1) DECODE_BODY(decode_i16c);
	if constexpr (Which == 2) DECODE_BODY(decode_f32);
	if constexpr (Which == 3) DECODE_BODY(decode_f32c);
	if constexpr (Which == 4) DECODE_BODY(decode_i16_to_f32);
#undef DECODE_BODY
}

template <int Which> static void run_filter(const RefFilterUBO *u, const void *in, uint64_t in_bytes, void *out,
                                            uint64_t out_bytes, const float *taps, int length, const int16_t *chmap,
                                            const uint32_t d[3])
{
#define FILTER_BODY(ns) do { \
	SET_STRIDES(ns, u); ns::decimation_rate = u->decimation_rate; ns::map_channels = u->map_channels != 0; \
	ns::demodulation_frequency = u->demodulation_frequency; ns::sampling_frequency = u->sampling_frequency; \
	ns::filter_coefficients = image1D{taps, length, 1}; ns::channel_mapping = iimage1D{chmap, 256}; \
	bind(ns::in_data, in, in_bytes); bind(ns::out_data, out, out_bytes); \
	dispatch(d[0] * 64, d[1], d[2], [] { ns::shader_main(); }); \
} while (0)
	if constexpr (Which == 0) FILTER_BODY(filter_f32c);
	if constexpr (Which == 1) FILTER_BODY(demod_i16);
	if constexpr (Which == 2) FILTER_BODY(demod_f32);
#undef FILTER_BODY
}

template <class NS> struct das_binder;

#define DAS_SET_UBO(ns, p) do { \
	for (int c = 0; c < 4; c++) ns::xdc_transform.c[c] = vec4(p->xdc_transform[4 * c], p->xdc_transform[4 * c + 1], \
	                                                          p->xdc_transform[4 * c + 2], p->xdc_transform[4 * c + 3]); \
	ns::dec_data_dim = ivec4{(int)p->dec_data_dim[0], (int)p->dec_data_dim[1], (int)p->dec_data_dim[2], (int)p->dec_data_dim[3]}; \
	ns::xdc_element_pitch = vec2(p->xdc_element_pitch[0], p->xdc_element_pitch[1]); \
	ns::rf_raw_dim = ivec2((int)p->rf_raw_dim[0], (int)p->rf_raw_dim[1]); \
	ns::transmit_mode = p->transmit_mode; ns::decode = p->decode; ns::das_shader_id = p->das_shader_id; \
	ns::time_offset = p->time_offset; \
	ns::output_min_coordinate = vec4(p->output_min_coordinate[0], p->output_min_coordinate[1], p->output_min_coordinate[2], p->output_min_coordinate[3]); \
	ns::output_max_coordinate = vec4(p->output_max_coordinate[0], p->output_max_coordinate[1], p->output_max_coordinate[2], p->output_max_coordinate[3]); \
	ns::output_points = uvec4{(uint)p->output_points[0], (uint)p->output_points[1], (uint)p->output_points[2], (uint)p->output_points[3]}; \
	ns::sampling_frequency = p->sampling_frequency; ns::center_frequency = p->center_frequency; \
	ns::speed_of_sound = p->speed_of_sound; ns::off_axis_pos = p->off_axis_pos; ns::beamform_plane = p->beamform_plane; \
	ns::f_number = p->f_number; ns::interpolate = p->interpolate != 0; ns::coherency_weighting = p->coherency_weighting != 0; \
	ns::decimation_rate = p->decimation_rate; ns::readi_group_id = p->readi_group_id; ns::readi_group_size = p->readi_group_size; \
} while (0)

extern "C" {

void ref_decode(const RefDecodeUBO *u, int variant, int first_stage, const void *in, uint64_t in_bytes,
                void *scratch, uint64_t scratch_bytes, void *out, uint64_t out_bytes, const int8_t *hadamard, int n,
                const int16_t *chmap, const uint32_t d[3])
{
	switch (variant) {
	case 3:  run_decode<0>(u, first_stage, in, in_bytes, scratch, scratch_bytes, out, out_bytes, hadamard, n, chmap, d); break;
	case 8:  run_decode<1>(u, first_stage, in, in_bytes, scratch, scratch_bytes, out, out_bytes, hadamard, n, chmap, d); break;
	case 9:  run_decode<2>(u, first_stage, in, in_bytes, scratch, scratch_bytes, out, out_bytes, hadamard, n, chmap, d); break;
	case 10: run_decode<3>(u, first_stage, in, in_bytes, scratch, scratch_bytes, out, out_bytes, hadamard, n, chmap, d); break;
	case 11: run_decode<4>(u, first_stage, in, in_bytes, scratch, scratch_bytes, out, out_bytes, hadamard, n, chmap, d); break;
	}
}

void ref_filter(const RefFilterUBO *u, int variant, const void *in, uint64_t in_bytes, void *out, uint64_t out_bytes,
                const float *taps, int length, const int16_t *chmap, const uint32_t d[3])
{
	switch (variant) {
	case 4:  run_filter<0>(u, in, in_bytes, out, out_bytes, taps, length, chmap, d); break;
	case 5:  run_filter<1>(u, in, in_bytes, out, out_bytes, taps, length, chmap, d); break;
	case 12: run_filter<2>(u, in, in_bytes, out, out_bytes, taps, length, chmap, d); break;
	}
}

/* das.glsl over the frame (beamformer.c:608-681). fast = 1: clear, then one
 * pass per receive channel (per transmit for VLS/TPW) with u_channel set. */
void ref_das(const BeamformerParameters *p, int fast, const float *rf, uint64_t rf_bytes, const int16_t *sparse,
             const float *focal, const float M[16], float *frame, const int32_t dims[3])
{
	image3D img{frame, dims[0], dims[1], dims[2]};
	uint32_t gx = ((uint32_t)dims[0] + 15) / 16 * 16, gy = (uint32_t)dims[1], gz = ((uint32_t)dims[2] + 15) / 16 * 16;
	if (fast) {
		std::memset(frame, 0, sizeof(float) * 2 * (size_t)dims[0] * dims[1] * dims[2]);
		DAS_SET_UBO(das_fast, p);
		bind(das_fast::rf_data, rf, rf_bytes);
		das_fast::u_out_data_tex = img;
		das_fast::sparse_elements = iimage1D{sparse, 256};
		das_fast::focal_vectors = image1D{focal, 256, 2};
		for (int c = 0; c < 4; c++) das_fast::u_voxel_transform.c[c] = vec4(M[4 * c], M[4 * c + 1], M[4 * c + 2], M[4 * c + 3]);
		int loop_end = (p->das_shader_id == 3 || p->das_shader_id == 4) ? (int)p->dec_data_dim[2] : (int)p->dec_data_dim[1];
		for (int index = 0; index < loop_end; index++) {
			das_fast::u_channel = index;
			dispatch(gx, gy, gz, [] { das_fast::shader_main(); });
		}
	} else {
		DAS_SET_UBO(das_full, p);
		bind(das_full::rf_data, rf, rf_bytes);
		das_full::u_out_data_tex = img;
		das_full::sparse_elements = iimage1D{sparse, 256};
		das_full::focal_vectors = image1D{focal, 256, 2};
		for (int c = 0; c < 4; c++) das_full::u_voxel_transform.c[c] = vec4(M[4 * c], M[4 * c + 1], M[4 * c + 2], M[4 * c + 3]);
		das_full::u_voxel_offset = ivec3(0, 0, 0);
		dispatch(gx, gy, gz, [] { das_full::shader_main(); });
	}
}

static uint32_t orone(uint32_t x) { return x ? x : 1; }

/* do_sum_shader (beamformer.c:218-235) */
void ref_sum(float *out, const float *const *ins, int count, float prescale, const int32_t dims[3])
{
	std::memset(out, 0, sizeof(float) * 2 * (size_t)dims[0] * dims[1] * dims[2]);
	sum::u_out_img = image3D{out, dims[0], dims[1], dims[2]};
	sum::u_sum_prescale = prescale;
	for (int i = 0; i < count; i++) {
		sum::u_in_img = image3D{const_cast<float *>(ins[i]), dims[0], dims[1], dims[2]};
		dispatch(32 * orone((uint32_t)dims[0] / 32), orone((uint32_t)dims[1]), 32 * orone((uint32_t)dims[2] / 32),
		         [] { sum::shader_main(); });
	}
}

/* MinMax stage (beamformer.c:595-607): levels_out holds levels 1..mips-1, NaN
 * where the dispatch writes nothing. */
void ref_min_max(const float *frame, const int32_t dims[3], int mips, float *levels_out, uint64_t levels_floats)
{
	for (uint64_t i = 0; i < levels_floats; i++) levels_out[i] = __builtin_nanf("");
	const float *prev = frame;
	int pw = dims[0], ph = dims[1], pd = dims[2];
	float *cur = levels_out;
	for (int l = 1; l < mips; l++) {
		uint32_t w = (uint32_t)dims[0] >> l, h = (uint32_t)dims[1] >> l, d = (uint32_t)dims[2] >> l;
		int W = w ? (int)w : 1, H = h ? (int)h : 1, D = d ? (int)d : 1;
		min_max::u_out_data_tex = image3D{const_cast<float *>(prev), pw, ph, pd};
		min_max::u_mip_view_tex = image3D{cur, W, H, D};
		min_max::u_mip_map = l;
		dispatch(32 * orone(w / 32), orone(h), 32 * orone(d / 32), [] { min_max::shader_main(); });
		prev = cur;
		pw = W; ph = H; pd = D;
		cur += 2 * (size_t)W * H * D;
	}
}

} /* extern "C" */
