/*
 * c_driver.c -- a C11 caller of the library, written the way the reference's own
 * drivers call its client library (tests/throughput.c:336-378 of the reference):
 * push parameters, tables, a Kaiser filter and the pipeline Decode -> Demodulate ->
 * DAS, then beamform_data_synchronized and compute_timings. It includes only
 * include/ogl_beamformer_lib.h and links libogl_beamformer_lib.so.
 *
 * The RF is a seeded int16 pattern (32 channels x 32 transmits x 512 samples, a
 * Hadamard-encoded echo plus noise). Exit status 0 when every call succeeds and
 * the volume is finite and not zero; it prints the volume energy and the DAS time.
 */
#include "ogl_beamformer_lib.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define S 512u
#define C 32u
#define T 32u
#define PX 32
#define PZ 32

static uint32_t lcg(uint32_t *s) { *s = *s * 1664525u + 1013904223u; return *s >> 8; }

static int fail(const char *what)
{
	printf("%s failed: %s\n", what, beamformer_get_last_error_string());
	return 1;
}

int main(void)
{
	BeamformerParameters bp;
	memset(&bp, 0, sizeof(bp));
	const float pitch = 1e-4f;
	for (int i = 0; i < 4; i++) bp.xdc_transform[i * 5] = 1.0f;
	bp.xdc_transform[12] = (C - 1) / 2.0f * pitch;          /* centre the array on the origin */
	bp.xdc_transform[13] = (T - 1) / 2.0f * pitch;
	bp.dec_data_dim[0] = S; bp.dec_data_dim[1] = C; bp.dec_data_dim[2] = T; bp.dec_data_dim[3] = 1;
	bp.xdc_element_pitch[0] = bp.xdc_element_pitch[1] = pitch;
	bp.rf_raw_dim[0] = S * T; bp.rf_raw_dim[1] = C;
	bp.transmit_mode = 1;
	bp.decode = 1;
	bp.das_shader_id = DASShaderKind_HERCULES;
	bp.output_min_coordinate[0] = -1.5e-3f; bp.output_min_coordinate[2] = 1.0e-3f;
	bp.output_max_coordinate[0] = 1.5e-3f;  bp.output_max_coordinate[2] = 3.5e-3f;
	bp.output_points[0] = PX; bp.output_points[1] = 1; bp.output_points[2] = PZ; bp.output_points[3] = 1;
	bp.sampling_frequency = 50e6f;
	bp.center_frequency = 12.5e6f;
	bp.speed_of_sound = 1540.0f;
	bp.f_number = 1.0f;
	bp.interpolate = 1;
	bp.decimation_rate = 2;

	/* RF: an echo at sample 100 + 3 t on every channel, Hadamard-encoded across
	 * transmits (Sylvester order 32), plus noise */
	int16_t *rf = malloc(sizeof(int16_t) * S * T * C);
	uint32_t seed = 12345u;
	for (uint32_t c = 0; c < C; c++)
		for (uint32_t i = 0; i < T; i++)
			for (uint32_t s = 0; s < S; s++) {
				float v = 0.0f;
				for (uint32_t t = 0; t < T; t++) {
					const int h = (__builtin_popcount(i & t) & 1) ? -1 : 1;
					const float d = (float)s - (100.0f + 3.0f * (float)t);
					v += (float)h * 200.0f * expf(-d * d / 18.0f) * sinf(0.5f * 3.14159265f * d);
				}
				v += (float)((int)(lcg(&seed) % 201) - 100);
				rf[((size_t)c * T + i) * S + s] = (int16_t)lrintf(v);
			}

	int16_t map[256], sparse[256];
	float focal[512];
	for (int i = 0; i < 256; i++) { map[i] = (int16_t)i; sparse[i] = (int16_t)i; focal[2 * i] = 0.0f; focal[2 * i + 1] = INFINITY; }

	if (!beamformer_set_global_timeout(-1)) return fail("set_global_timeout");
	if (!beamformer_push_channel_mapping(map, 256)) return fail("push_channel_mapping");
	if (!beamformer_push_sparse_elements(sparse, 256)) return fail("push_sparse_elements");
	if (!beamformer_push_focal_vectors(focal, 256)) return fail("push_focal_vectors");
	if (!beamformer_create_kaiser_low_pass_filter(5.65f, 5e6f, 25e6f, 32, 0)) return fail("create_kaiser_low_pass_filter");
	if (!beamformer_push_parameters(&bp)) return fail("push_parameters");
	int32_t stages[3] = {BeamformerShaderKind_Decode, BeamformerShaderKind_Demodulate, BeamformerShaderKind_DAS};
	if (!beamformer_push_pipeline(stages, 3, BeamformerDataKind_Int16)) return fail("push_pipeline");

	int32_t pts[3] = {PX, 1, PZ};
	float *out = calloc((size_t)2 * PX * PZ, sizeof(float));
	if (!beamform_data_synchronized(rf, S * T * C * (uint32_t)sizeof(int16_t), pts, out, -1))
		return fail("beamform_data_synchronized");

	double energy = 0.0;
	for (int i = 0; i < 2 * PX * PZ; i++) {
		if (!isfinite(out[i])) { printf("non-finite output at %d\n", i); return 1; }
		energy += (double)out[i] * out[i];
	}
	if (!(energy > 0.0)) { printf("all-zero volume\n"); return 1; }

	BeamformerComputeStatsTable stats;
	memset(&stats, 0, sizeof(stats));
	if (!beamformer_compute_timings(&stats, -1)) return fail("compute_timings");
	float das = 0.0f;
	for (int r = 0; r < 32; r++) das = fmaxf(das, stats.times[r][BeamformerShaderKind_DASFast]);
	printf("ok: volume energy %.6g, DAS %.3f ms\n", energy, das * 1e3f);
	free(out);
	free(rf);
	return 0;
}
