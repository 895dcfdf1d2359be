/*
 * bf_oracle.h -- CPU oracle for the beamforming hot path. TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's compute path (decode.glsl, filter.glsl,
 * das.glsl, sum.glsl, min_max.glsl and the host glue in beamformer.c / math.c),
 * used by the tests as the parity checker and by bench.py as the timed CPU
 * baseline. Nothing in the product library links, loads or calls this code.
 *
 * Two numeric modes:
 *   - *_f32: FP32 "reference semantics". Every floating-point expression is
 *     evaluated in the order the reference writes it, one IEEE operation at a
 *     time (compiled with -ffp-contract=off), so that sample delays and phases
 *     are reproducible bit for bit by the CUDA kernels.
 *   - *_f64: the same algorithm in FP64, the error reference for the
 *     mixed-precision variants.
 */
#ifndef BF_ORACLE_H
#define BF_ORACLE_H

#include <stdint.h>
#include "../include/ogl_beamformer_lib.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Decode stage uniform block (reference beamformer.h:123-139). */
typedef struct {
	uint32_t input_channel_stride, input_sample_stride, input_transmit_stride;
	uint32_t output_channel_stride, output_sample_stride, output_transmit_stride;
	uint32_t transmit_count, decode_mode;
} BfoDecodeUBO;

/* Filter/demodulate uniform block (reference beamformer.h:112-147). */
typedef struct {
	uint32_t input_channel_stride, input_sample_stride, input_transmit_stride;
	uint32_t output_channel_stride, output_sample_stride, output_transmit_stride;
	uint32_t decimation_rate, map_channels;
	float    demodulation_frequency, sampling_frequency;
} BfoFilterUBO;

typedef struct {
	int32_t kind;                /* BeamformerFilterKind */
	int32_t length;
	float   sampling_frequency;  /* creation-time sampling frequency */
	float   param0, param1;      /* (beta, cutoff) or (xdc_center_frequency, tx_frequency) */
} BfoFilterSpec;

/* Planned pipeline (reference beamformer.c:303-481). */
typedef struct {
	int32_t  shaders[MAX_COMPUTE_SHADER_STAGES];
	uint8_t  filter_slots[MAX_COMPUTE_SHADER_STAGES];
	int32_t  shader_count;
	uint32_t decode_dispatch[3];
	uint32_t demod_dispatch[3];
	uint32_t rf_size;
	BfoDecodeUBO decode;
	BfoFilterUBO demod;
	BfoFilterUBO filter;
	BeamformerParameters das;
} BfoPlan;

/* ---- host math (reference math.c, external/cephes.c) ---- */
double   bfo_i0(double x);
int32_t  bfo_hadamard_transpose(int32_t dim, int32_t *out);  /* returns 1 if built */
void     bfo_kaiser_low_pass(float cutoff_frequency, float sampling_frequency, float beta,
                             int32_t length, float *out);
void     bfo_matched_filter(float xdc_center_frequency, float transmit_frequency,
                            float sampling_frequency, int32_t length, float *out);
void     bfo_kaiser_low_pass_f64(double cutoff_frequency, double sampling_frequency, double beta,
                                 int32_t length, double *out);
void     bfo_voxel_transform(const BeamformerParameters *bp, float out[16]);
void     bfo_voxel_transform_f64(const BeamformerParameters *bp, double out[16]);
int32_t  bfo_frame_mips(const int32_t dims[3]);

/* ---- planning ---- */
void     bfo_plan(const BeamformerParameters *bp, const int32_t *shaders, const uint8_t *slots,
                  int32_t shader_count, int32_t data_kind, const BfoFilterSpec filters[4],
                  BfoPlan *out);

/* ---- stages ---- */
/* decode.glsl: `variant` is the planned shader kind (Decode, DecodeInt16Complex,
 * DecodeFloat, DecodeFloatComplex, DecodeInt16ToFloat). first_stage selects the
 * raw-input reshuffle pass. `in` is the raw RF (first stage) or the previous
 * stage's output; `out` receives float2 data. */
void bfo_decode(const BfoDecodeUBO *u, int32_t variant, int32_t first_stage, int32_t data_kind,
                const void *in, uint64_t in_bytes, void *out, uint64_t out_bytes,
                const int32_t *hadamard, int32_t hadamard_dim, const int16_t *channel_mapping,
                const uint32_t dispatch[3], int32_t threads);

/* filter.glsl: variant is Demodulate (packed snorm int16 in/out), DemodulateFloat
 * or Filter. taps has `length` entries. */
void bfo_filter(const BfoFilterUBO *u, int32_t variant, const void *in, uint64_t in_bytes,
                void *out, uint64_t out_bytes, const float *taps, int32_t length,
                const int16_t *channel_mapping, const uint32_t dispatch[3], int32_t threads);
void bfo_filter_f64(const BfoFilterUBO *u, int32_t variant, const double *in, uint64_t in_count,
                    double *out, uint64_t out_count, const double *taps, int32_t length,
                    const uint32_t dispatch[3], int32_t threads);

/* das.glsl: fast = 1 accumulates one receive channel (or transmit) per pass in
 * the order of the reference's DAS_FAST dispatch loop; fast = 0 is the
 * full/coherency path. rf holds rf_floats floats (float2 samples). frame is
 * dims[0]*dims[1]*dims[2] float2 in x-fastest order and is overwritten. The
 * voxel subset [voxel_begin, voxel_end) (linear index) is computed; others are
 * left untouched, which lets a caller sample the volume. */
void bfo_das(const BeamformerParameters *p, int32_t fast, const float *rf, uint64_t rf_floats,
             const int16_t *sparse_elements, const float *focal_vectors, const float M[16],
             float *frame, const int32_t dims[3], int64_t voxel_begin, int64_t voxel_end,
             int32_t interpolation_override, int32_t threads);
void bfo_das_f64(const BeamformerParameters *p, int32_t fast, const double *rf, uint64_t rf_count,
                 const int16_t *sparse_elements, const float *focal_vectors, const double M[16],
                 double *frame, const int32_t dims[3], int64_t voxel_begin, int64_t voxel_end,
                 int32_t interpolation_override, int32_t threads);

/* sum.glsl + do_sum_shader: out = sum_i prescale * in_i, over the reference's
 * ORONE(x/32) x ORONE(y) x ORONE(z/32) dispatch of 32x1x32 groups. */
void bfo_sum(float *out, const float *const *ins, int32_t count, float prescale, const int32_t dims[3],
             int32_t threads);

/* min_max.glsl over all mip levels. levels_out receives levels 1..mips-1
 * concatenated, each max(1, d >> l) sized, float2 per texel. Texels the
 * reference's dispatch never writes are set to NaN. */
void bfo_min_max(const float *frame, const int32_t dims[3], float *levels_out, int32_t threads);
uint64_t bfo_min_max_levels_floats(const int32_t dims[3]);

/* DAS validity statistics: number of (voxel, transmit, receive) terms whose
 * apodization is not negligible (|arg| < pi/2) for the given parameters. */
uint64_t bfo_das_active_terms(const BeamformerParameters *p, const int16_t *sparse_elements,
                              const float *focal_vectors, const float M[16], const int32_t dims[3],
                              int64_t voxel_begin, int64_t voxel_end, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
