/*
 * bf_host.h -- host-side planning and filter/matrix generation of the library.
 */
#pragma once
#include <cstdint>
#include <vector>
#include "ogl_beamformer_lib.h"
#include "bf_kernels.h"

namespace bf {

struct FilterSpec {
	int32_t kind = -1;            /* BeamformerFilterKind, -1 = empty slot */
	int32_t length = 0;
	float   sampling_frequency = 0;
	float   param0 = 0, param1 = 0;
};

/* Result of planning a pushed pipeline (reference beamformer.c:303-481). */
struct Plan {
	int32_t  shaders[MAX_COMPUTE_SHADER_STAGES];
	uint8_t  slots[MAX_COMPUTE_SHADER_STAGES];
	int32_t  count = 0;
	bool     decode_first = false, demodulate = false;
	uint32_t rf_size = 0;                    /* bytes of channel data the DAS stage may read */

	Strides  decode_st{};
	uint32_t decode_mode = 0, transmit_count = 0;
	uint32_t decode_invocations_x = 0;       /* decode dispatch width in invocations (reference grid) */

	Strides  demod_st{};
	uint32_t demod_decimation = 1, demod_map = 0;
	float    demod_frequency = 0, demod_fs = 0;
	uint32_t demod_rows_x = 0;               /* outputs per row (dispatch width) */

	Strides  filter_st{};
	float    filter_frequency = 0, filter_fs = 0;

	BeamformerParameters das{};              /* parameters as the DAS stage sees them */
};

void     plan_pipeline(const BeamformerParameters &in, const int32_t *shaders, const uint8_t *slots, int32_t count,
                       int32_t data_kind, const FilterSpec filters[BEAMFORMER_FILTER_SLOTS], Plan &out);

/* Hadamard matrix of the reference's construction (math.c:33-122), row-major
 * int8. Returns false for orders the reference does not build. */
bool     hadamard_matrix(int32_t order, std::vector<int8_t> &out, int32_t &sylvester, int32_t &base);
double   bessel_i0(double x);
void     kaiser_low_pass(float cutoff, float fs, float beta, int32_t length, float *out);
void     matched_filter(float xdc_fc, float tx_f, float fs, int32_t length, float *out);
void     voxel_transform(const BeamformerParameters &bp, float out[16]);
int32_t  frame_mips(const int32_t dims[3]);

constexpr float DEG2RAD_F = 0.017453292519943295f;

} /* namespace bf */
