/*
 * ogl_beamformer_lib.h -- C ABI of the GB300 beamforming library.
 *
 * Drop-in for the client library of the reference beamformer
 * (helpers/ogl_beamformer_lib_base.h + beamformer_parameters.h, concatenated into
 * one header by build.c:659-671 in the reference). Every type, enum value and
 * function signature below keeps the reference's binary contract so that existing
 * callers (MATLAB loadlibrary, C test drivers) link against this library unchanged.
 *
 * Differences in *transport*: the reference library talks to a separate `ogl`
 * server process through a 2 GB POSIX shared-memory region and futex locks
 * (helpers/ogl_beamformer_lib.c:30-125). This library runs the whole pipeline
 * in-process on one GB300: pushes copy the caller's data to device memory, compute
 * is launched on a CUDA stream, and the `timeout_ms` arguments bound the waits on
 * that stream instead of waits on shared-memory locks.
 *
 * All functions are C ABI (`extern "C"`), take plain pointers and sizes, and are
 * not thread safe (one process-global context, as in the reference).
 */
#ifndef OGL_BEAMFORMER_LIB_H
#define OGL_BEAMFORMER_LIB_H

#include <stddef.h>
#include <stdint.h>

#ifndef LIB_FN
  #if defined(_WIN32)
    #define LIB_FN __declspec(dllexport)
  #else
    #define LIB_FN __attribute__((visibility("default")))
  #endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------
 * Shader (stage) kinds. Values are the reference's (beamformer_parameters.h:14-41).
 * Kinds 8..13 are internal variants chosen by pipeline planning; callers push
 * kinds 0..7.
 * ---------------------------------------------------------------------------- */
typedef enum {
	BeamformerShaderKind_CudaDecode         = 0,
	BeamformerShaderKind_CudaHilbert        = 1,
	BeamformerShaderKind_DAS                = 2,
	BeamformerShaderKind_Decode             = 3,
	BeamformerShaderKind_Filter             = 4,
	BeamformerShaderKind_Demodulate         = 5,
	BeamformerShaderKind_MinMax             = 6,
	BeamformerShaderKind_Sum                = 7,
	BeamformerShaderKind_DecodeInt16Complex = 8,
	BeamformerShaderKind_DecodeFloat        = 9,
	BeamformerShaderKind_DecodeFloatComplex = 10,
	BeamformerShaderKind_DecodeInt16ToFloat = 11,
	BeamformerShaderKind_DemodulateFloat    = 12,
	BeamformerShaderKind_DASFast            = 13,
	BeamformerShaderKind_Render3D           = 14,
	BeamformerShaderKind_Count              = 15,

	BeamformerShaderKind_ComputeCount = BeamformerShaderKind_Render3D,
} BeamformerShaderKind;

/* Per-frame stage timings in seconds, last 32 computes (beamformer_parameters.h:43-48). */
typedef struct {
	float times[32][BeamformerShaderKind_Count];
	float rf_time_deltas[32];
} BeamformerComputeStatsTable;

/* Decode modes (beamformer_parameters.h:51-53). */
enum { DECODE_MODE_NONE = 0, DECODE_MODE_HADAMARD = 1 };

/* Input data kinds (beamformer_parameters.h:55-63). */
typedef enum {
	BeamformerDataKind_Int16          = 0,
	BeamformerDataKind_Int16Complex   = 1,
	BeamformerDataKind_Float32        = 2,
	BeamformerDataKind_Float32Complex = 3,
} BeamformerDataKind;

/* Filter kinds (beamformer_parameters.h:65-71). */
typedef enum {
	BeamformerFilterKind_Kaiser  = 0,
	BeamformerFilterKind_Matched = 1,
} BeamformerFilterKind;

/* Image plane tags (beamformer_parameters.h:74-85). */
typedef enum {
	BeamformerViewPlaneTag_XZ        = 0,
	BeamformerViewPlaneTag_YZ        = 1,
	BeamformerViewPlaneTag_XY        = 2,
	BeamformerViewPlaneTag_Arbitrary = 3,
	BeamformerViewPlaneTag_Count,
} BeamformerViewPlaneTag;

/* Delay-and-sum kinds, stored in BeamformerParameters.das_shader_id
 * (beamformer_parameters.h:88-99). */
typedef enum {
	DASShaderKind_FORCES         = 0,
	DASShaderKind_UFORCES        = 1,
	DASShaderKind_HERCULES       = 2,
	DASShaderKind_RCA_VLS        = 3,
	DASShaderKind_RCA_TPW        = 4,
	DASShaderKind_UHERCULES      = 5,
	DASShaderKind_RACES          = 6,
	DASShaderKind_EPIC_FORCES    = 7,
	DASShaderKind_EPIC_UFORCES   = 8,
	DASShaderKind_EPIC_UHERCULES = 9,
	DASShaderKind_FLASH          = 10,
	DASShaderKind_Count,
} DASShaderKind;

#define MAX_BEAMFORMED_SAVED_FRAMES 16   /* beamformer_parameters.h:127 */
#define MAX_COMPUTE_SHADER_STAGES   16   /* beamformer_parameters.h:128 */
#define BEAMFORMER_FILTER_SLOTS      4   /* beamformer_parameters.h:130 */

/* ------------------------------------------------------------------------------
 * Parameter block. std140-compatible, 208 bytes, field order and offsets exactly
 * as the reference's X-macro expansion (beamformer_parameters.h:134-175):
 *   xdc_transform 0, dec_data_dim 64, xdc_element_pitch 80, rf_raw_dim 88,
 *   transmit_mode 96, decode 100, das_shader_id 104, time_offset 108,
 *   output_min_coordinate 112, output_max_coordinate 128, output_points 144,
 *   sampling_frequency 160, center_frequency 164, speed_of_sound 168,
 *   off_axis_pos 172, beamform_plane 176, f_number 180, interpolate 184,
 *   coherency_weighting 188, decimation_rate 192, readi_group_id 196,
 *   readi_group_size 200.
 * ---------------------------------------------------------------------------- */
#define BF_PARAMETERS_UI_FIELDS \
	float    output_min_coordinate[4]; /* [m] back-top-left corner of the output region */ \
	float    output_max_coordinate[4]; /* [m] front-bottom-right corner of the output region */ \
	int32_t  output_points[4];         /* width, height, depth, frames to average */ \
	float    sampling_frequency;       /* [Hz] */ \
	float    center_frequency;         /* [Hz] */ \
	float    speed_of_sound;           /* [m/s] */ \
	float    off_axis_pos;             /* [m] plane position normal to the beamformed plane */ \
	int32_t  beamform_plane;           /* plane to beamform in TPW/VLS/HERCULES */ \
	float    f_number;                 /* receive F# (0 disables apodization) */ \
	uint32_t interpolate;              /* cubic interpolation of RF samples */ \
	uint32_t coherency_weighting;      /* coherency-weighted output */

#define BF_PARAMETERS_HEAD_FIELDS \
	float    xdc_transform[16];        /* column-major array transform */ \
	uint32_t dec_data_dim[4];          /* samples, channels, transmits; last ignored */ \
	float    xdc_element_pitch[2];     /* [m] element pitch {row, col} */ \
	uint32_t rf_raw_dim[2];            /* raw data dimensions */ \
	int32_t  transmit_mode;            /* transmit/receive orientation bits */ \
	uint32_t decode;                   /* DECODE_MODE_* */ \
	uint32_t das_shader_id;            /* DASShaderKind */ \
	float    time_offset;              /* [s] pulse length correction */

#define BF_PARAMETERS_TAIL_FIELDS \
	uint32_t decimation_rate;          /* decimation of the demodulation stage */ \
	uint32_t readi_group_id;           /* READI group of this data */ \
	uint32_t readi_group_size;         /* READI transmit group size */

typedef struct { BF_PARAMETERS_UI_FIELDS   } BeamformerUIParameters;
typedef struct { BF_PARAMETERS_HEAD_FIELDS } BeamformerParametersHead;
typedef struct { BF_PARAMETERS_TAIL_FIELDS } BeamformerParametersTail;

typedef struct {
	BF_PARAMETERS_HEAD_FIELDS
	BF_PARAMETERS_UI_FIELDS
	BF_PARAMETERS_TAIL_FIELDS
	float _pad[1];
} BeamformerParameters;

#if defined(__cplusplus)
static_assert(sizeof(BeamformerParameters) == 208, "BeamformerParameters must be 208 bytes");
static_assert(offsetof(BeamformerParameters, output_min_coordinate) == 112, "UI block offset");
static_assert(offsetof(BeamformerParameters, decimation_rate) == 192, "tail block offset");
#elif defined(__STDC_VERSION__) && __STDC_VERSION__ >= 201112L
_Static_assert(sizeof(BeamformerParameters) == 208, "BeamformerParameters must be 208 bytes");
_Static_assert(offsetof(BeamformerParameters, output_min_coordinate) == 112, "UI block offset");
_Static_assert(offsetof(BeamformerParameters, decimation_rate) == 192, "tail block offset");
#endif

/* Live-imaging dirty flags and parameters (beamformer_parameters.h:184-202). */
typedef enum {
	BeamformerLiveImagingDirtyFlags_ImagePlaneOffsets = 1 << 0,
	BeamformerLiveImagingDirtyFlags_TransmitPower     = 1 << 1,
	BeamformerLiveImagingDirtyFlags_TGCControlPoints  = 1 << 2,
	BeamformerLiveImagingDirtyFlags_SaveData          = 1 << 3,
	BeamformerLiveImagingDirtyFlags_StopImaging       = 1 << 4,
} BeamformerLiveImagingDirtyFlags;

typedef struct {
	uint32_t active;
	uint32_t save_enabled;
	uint32_t save_active;
	float    transmit_power;
	float    image_plane_offsets[BeamformerViewPlaneTag_Count];
	float    tgc_control_points[8];
} BeamformerLiveImagingParameters;

/* ------------------------------------------------------------------------------
 * Errors. Kinds 0..13 keep the reference's values (ogl_beamformer_lib_base.h:10-28).
 * Kinds 14..16 are this library's additions for failures that only exist in an
 * in-process CUDA implementation.
 * ---------------------------------------------------------------------------- */
typedef enum {
	BF_LIB_ERR_KIND_NONE                    = 0,
	BF_LIB_ERR_KIND_VERSION_MISMATCH        = 1,
	BF_LIB_ERR_KIND_INVALID_ACCESS          = 2,
	BF_LIB_ERR_KIND_COMPUTE_STAGE_OVERFLOW  = 3,
	BF_LIB_ERR_KIND_INVALID_COMPUTE_STAGE   = 4,
	BF_LIB_ERR_KIND_INVALID_START_SHADER    = 5,
	BF_LIB_ERR_KIND_INVALID_DEMOD_DATA_KIND = 6,
	BF_LIB_ERR_KIND_INVALID_IMAGE_PLANE     = 7,
	BF_LIB_ERR_KIND_BUFFER_OVERFLOW         = 8,
	BF_LIB_ERR_KIND_WORK_QUEUE_FULL         = 9,
	BF_LIB_ERR_KIND_EXPORT_SPACE_OVERFLOW   = 10,
	BF_LIB_ERR_KIND_SHARED_MEMORY           = 11,
	BF_LIB_ERR_KIND_SYNC_VARIABLE           = 12,
	BF_LIB_ERR_KIND_INVALID_TIMEOUT         = 13,
	BF_LIB_ERR_KIND_CUDA_DEVICE             = 14, /* no usable CUDA device / context */
	BF_LIB_ERR_KIND_CUDA_RUNTIME            = 15, /* a CUDA call or kernel launch failed */
	BF_LIB_ERR_KIND_UNSUPPORTED             = 16, /* stage or DAS mode not implemented here */
} BeamformerLibErrorKind;

/* Interface version; same number as the reference's shared-memory layout
 * version (beamformer_work_queue.h:5) so version checks in callers still pass. */
#define BEAMFORMER_SHARED_MEMORY_VERSION 11u

/* Largest RF push accepted, bytes. The reference bounds pushes by its 2 GB
 * shared-memory scratch (beamformer_work_queue.h:106-110); the same bound is kept. */
#define BEAMFORMER_MAX_RF_DATA_SIZE (2147483648ull - 65536ull)

/* ---------------------------- reference interface --------------------------- */

/* ogl_beamformer_lib_base.h:30 / ogl_beamformer_lib.c:127-131 */
LIB_FN uint32_t beamformer_get_api_version(void);

/* ogl_beamformer_lib_base.h:32-34 / ogl_beamformer_lib.c:133-152 */
LIB_FN BeamformerLibErrorKind beamformer_get_last_error(void);
LIB_FN const char *beamformer_get_last_error_string(void);
LIB_FN const char *beamformer_error_string(BeamformerLibErrorKind kind);

/* Timeout for calls that wait but take no timeout argument. Range [-1, ...);
 * -1 waits forever, 0 tries once (default).
 * ogl_beamformer_lib_base.h:36-44 / ogl_beamformer_lib.c:154-164 */
LIB_FN uint32_t beamformer_set_global_timeout(int32_t timeout_ms);

/* Push RF, beamform, and copy the (complex, 2 floats per point) output volume
 * into out_data. output_points is clamped to >= 1 and written back.
 * ogl_beamformer_lib_base.h:46-49 / ogl_beamformer_lib.c:460-491 */
LIB_FN uint32_t beamform_data_synchronized(void *data, uint32_t data_size, int32_t output_points[3],
                                           float *out_data, int32_t timeout_ms);

/* Stage timings of the last 32 computes.
 * ogl_beamformer_lib_base.h:51-52 / ogl_beamformer_lib.c:493-506 */
LIB_FN uint32_t beamformer_compute_timings(BeamformerComputeStatsTable *output, int32_t timeout_ms);

/* Start a compute on the most recently pushed RF.
 * ogl_beamformer_lib_base.h:54-55 / ogl_beamformer_lib.c:285-290 */
LIB_FN uint32_t beamformer_start_compute(void);

/* Wait until previously queued compute has been dispatched.
 * ogl_beamformer_lib_base.h:57-58 / ogl_beamformer_lib.c:292-300 */
LIB_FN uint32_t beamformer_wait_for_compute_dispatch(int32_t timeout_ms);

/* ogl_beamformer_lib_base.h:60-65 / ogl_beamformer_lib.c:338-390 */
LIB_FN uint32_t beamformer_push_data_with_compute(void *data, uint32_t size, uint32_t image_plane_tag);
LIB_FN uint32_t beamformer_push_data(void *data, uint32_t size);
LIB_FN uint32_t beamformer_push_channel_mapping(int16_t *mapping,  uint32_t count);
LIB_FN uint32_t beamformer_push_sparse_elements(int16_t *elements, uint32_t count);
LIB_FN uint32_t beamformer_push_focal_vectors(float     *vectors,  uint32_t count);

/* ogl_beamformer_lib_base.h:67-71 / ogl_beamformer_lib.c:192-225, 392-429 */
LIB_FN uint32_t beamformer_set_pipeline_stage_parameters(int32_t stage_index, int32_t parameter);
LIB_FN uint32_t beamformer_push_pipeline(int32_t *shaders, int32_t shader_count, BeamformerDataKind data_kind);
LIB_FN uint32_t beamformer_push_parameters(BeamformerParameters *);
LIB_FN uint32_t beamformer_push_parameters_ui(BeamformerUIParameters *);
LIB_FN uint32_t beamformer_push_parameters_head(BeamformerParametersHead *);

/* Kaiser low-pass and matched filters into one of BEAMFORMER_FILTER_SLOTS slots.
 * ogl_beamformer_lib_base.h:73-97 / ogl_beamformer_lib.c:227-254, math.c:125-181 */
LIB_FN uint32_t beamformer_create_kaiser_low_pass_filter(float beta, float cutoff_frequency,
                                                         float sampling_frequency,
                                                         int16_t length, uint8_t slot);
LIB_FN uint32_t beamformer_create_matched_filter(float xdc_center_frequency, float transmit_frequency,
                                                 float sampling_frequency,
                                                 int16_t length, uint8_t slot);

/* ogl_beamformer_lib_base.h:99-103 / ogl_beamformer_lib.c:508-540 */
LIB_FN int32_t  beamformer_live_parameters_get_dirty_flag(void);
LIB_FN uint32_t beamformer_set_live_parameters(BeamformerLiveImagingParameters *);
LIB_FN BeamformerLiveImagingParameters *beamformer_get_live_parameters(void);

/* ------------------------------------------------------------------------------
 * Extensions of this library (no counterpart in the reference's exported API).
 * They expose what the reference keeps inside its server process, so that
 * device-resident callers and tests can reach it.
 * ---------------------------------------------------------------------------- */

/* Use RF that already lives in device memory for the next compute instead of a
 * host push: the pipeline reads `device_data` directly (no copy). The caller
 * keeps the buffer alive and unchanged until that compute has finished. The
 * compute waits for the work queued on the legacy default stream before it
 * starts (so data written there, e.g. by PyTorch's default stream, is complete);
 * data written on another stream needs that stream set with set_stream, or a
 * synchronisation, first.
 * Counterpart of beamformer_push_data (ogl_beamformer_lib.c:360-382) for a
 * caller whose data is already on the GPU. */
LIB_FN uint32_t beamformer_gb300_push_data_device(const void *device_data, uint64_t size);

/* Run computes on this CUDA stream (a cudaStream_t passed as a pointer; NULL
 * selects the library's own stream). Lets a caller order the pipeline with its
 * own work and time it with events on the same stream. */
LIB_FN uint32_t beamformer_gb300_set_stream(void *cuda_stream);
LIB_FN void    *beamformer_gb300_get_stream(void);

/* Block until every queued compute has finished (timeout_ms as above). */
LIB_FN uint32_t beamformer_gb300_synchronize(int32_t timeout_ms);

/* Copy a frame out of the device frame store: which = 0 latest beamformed
 * frame, 1 latest averaged frame (written by the Sum stage). mip_level selects
 * the Min/Max pyramid level (0 = the frame itself). Output is 2 floats per
 * point in x-fastest order; out_size is in bytes; out may be host or device
 * memory. The reference keeps these levels in GL textures (beamformer.c:119-151,
 * 595-607). */
LIB_FN uint32_t beamformer_gb300_export_frame(uint32_t which, uint32_t mip_level, float *out,
                                              uint64_t out_size, int32_t dims_out[3]);

/* Copy the output of the last intermediate (non-DAS) stage, i.e. the decoded
 * or filtered channel data the next stage would read (the reference's
 * rf_data_ssbos, beamformer.c:153-191). Returns the byte count in *size_out. */
LIB_FN uint32_t beamformer_gb300_export_channel_data(void *out, uint64_t out_size, uint64_t *size_out);

/* Copy the current filter taps of a slot (as generated on the host, float32). */
LIB_FN uint32_t beamformer_gb300_get_filter(uint8_t slot, float *taps, int32_t capacity, int32_t *length_out);

/* Interpolation used by the DAS stage: -1 follows BeamformerParameters.interpolate
 * (0 nearest, non-zero cubic, das.glsl:64-72); 0 nearest, 1 cubic, 2 linear.
 * Linear interpolation has no counterpart in the reference. */
LIB_FN uint32_t beamformer_gb300_set_interpolation(int32_t mode);

/* Arithmetic of the front end (no counterpart in the reference; the precision
 * variant): 0 = FP32 as the reference (default); 1 = FP16, 2 = BF16. With 1 or 2
 * a pipeline must start Decode (int16 data, Hadamard order a power of two <= 128)
 * -> Demodulate with decimation 1, 2 or 4 and at most 160 taps: the decoded
 * samples are rounded once to the 16-bit type, and the demodulating FIR runs as
 * a Toeplitz contraction on the tensor cores with FP32 accumulation. DAS and the
 * later stages stay FP32. Other pipelines fail with UNSUPPORTED at compute time
 * while a 16-bit precision is selected. Takes effect at the next compute. */
LIB_FN uint32_t beamformer_gb300_set_filter_precision(int32_t precision);

/* Arithmetic of HERCULES delay-and-sum (no counterpart in the reference; the
 * precision variant): 0 = FP32 with the reference's sample indices (default);
 * 1 = the per-frame interpolation table in FP16 (coefficients scaled by a power
 * of two from the frame's largest channel-data magnitude, evaluated in packed
 * FP16), the sample index from an approximate square root and one FMA, and a
 * degree-3 apodization polynomial, with FP32 sums. Applies where DAS runs on the
 * HERCULES fast path (DASFast; dense channel data, no sparse elements, no
 * coherency weighting; in beamformer_gb300_beamform_batch its HERCULES
 * acquisitions, each table with its own scale); other DAS stages stay FP32.
 * Takes effect at the next compute. */
LIB_FN uint32_t beamformer_gb300_set_das_precision(int32_t precision);

/* Receive-aperture subsampling of HERCULES delay-and-sum (no counterpart in the
 * reference; the input of the learned variant): DAS sums receive channels 0,
 * step, 2 step, ... only (step 1, the default, uses all). Other DAS modes fail
 * with UNSUPPORTED while step > 1. Takes effect at the next compute. */
LIB_FN uint32_t beamformer_gb300_set_receive_subsampling(int32_t step);

/* Serve the reference's shared-memory protocol (the `ogl` server side of
 * helpers/ogl_beamformer_lib.c: region "/ogl_beamformer_shared_memory", version
 * BEAMFORMER_SHARED_MEMORY_VERSION, beamformer.c:842-1111, 1230-1276) in the
 * calling thread, computing with this library, so unmodified clients of the
 * reference's client library beamform on this GPU. Runs until
 * beamformer_gb300_serve_stop() or, with idle_exit_ms >= 0, until that long
 * without work; returns 0, or -1 if the region cannot be created. No counterpart
 * in the reference's client library; the ogl_beamformer_server executable wraps it. */
LIB_FN int32_t beamformer_gb300_serve(int32_t idle_exit_ms);
LIB_FN void    beamformer_gb300_serve_stop(void);

/* Beamform `count` acquisitions in one go (the batched variant; no counterpart
 * in the reference, which beamforms one acquisition per compute). Acquisition i
 * has its own parameters[i] (transmit and sample counts, output grid, DAS mode),
 * its raw RF at the DEVICE pointer rf[i] (rf_size[i] bytes, the pushed data kind)
 * and its volume written to the DEVICE pointer out[i] (output_points x 2 floats,
 * x fastest). All share the pushed pipeline, filters, channel mapping, sparse
 * elements, focal vectors and interpolation; the pipeline's last stage must be DAS
 * without coherency weighting, the DAS modes HERCULES (not sparse) or FORCES, and
 * all acquisitions must use one interpolation mode. The front ends run per
 * acquisition and the DAS of all acquisitions runs as persistent launches that
 * take voxel tiles from cost-ordered work lists (one launch for the HERCULES
 * tiles, one for the FORCES tiles, per 64 acquisitions); on
 * the first call for a set of parameters and pointers the tile shape and grid
 * size are autotuned on the device and the whole batch is captured in a CUDA graph,
 * which later calls with the same set replay. As for push_data_device, the
 * batch first waits for the work queued on the legacy default stream. timeout_ms
 * as beamform_data_synchronized. Fails with UNSUPPORTED for other pipelines or a
 * 16-bit filter precision. */
LIB_FN uint32_t beamformer_gb300_beamform_batch(const BeamformerParameters *parameters, uint32_t count,
                                                const void *const *rf, const uint64_t *rf_size, float *const *out,
                                                int32_t timeout_ms);

/* The autotuner's choice for the current batch: *volume_tiles 1 when HERCULES
 * volumes use 4x4x16 voxel tiles (0: 8x1x16), *ctas the persistent grid size, and
 * the timed DAS milliseconds of every candidate (tile shape x {4, 5, 6} CTAs per
 * SM, in that order) when candidate_ms has room for *count_out values. */
LIB_FN uint32_t beamformer_gb300_batch_tuning(int32_t *volume_tiles, int32_t *ctas, float *candidate_ms,
                                              int32_t capacity, int32_t *count_out);

/* Delay-and-sum of one frame that allocates no device memory. Has no
 * counterpart in the reference. It is meant for callers that cannot let a
 * library allocate on the GPU while they run: for example an acquisition loop
 * that fixes its whole memory budget at start-up, or a host application whose
 * device memory belongs to its own allocator. Such callers cannot grant the
 * scratch buffer the regular pipeline allocates for small volumes.
 *   das_parameters  the parameters as the DAS stage sees them (for a
 *                   decode -> demodulate -> DAS pipeline: dec_data_dim[0],
 *                   sampling_frequency divided by 2 * decimation_rate,
 *                   time_offset including the filter delays);
 *   focal_vectors   host, 256 (angle, depth) pairs (NULL: all zero);
 *   sparse_elements host, 256 entries (NULL: 0..255);
 *   channel_data    device, float2 [channel][transmit][sample];
 *   frame           device, output_points[0..2] float2 in x-fastest order;
 *   cuda_stream     cudaStream_t as a pointer (NULL: the default stream).
 * The two host tables are read before the call returns; they travel to the GPU
 * as kernel parameters, so the caller may reuse them at once.
 * The call is self-contained: das_parameters->interpolate selects nearest (0)
 * or cubic (non-zero) interpolation, every receive channel is summed, and the
 * library-wide settings of set_interpolation, set_receive_subsampling and
 * set_das_precision do not apply to it.
 * Small volumes split the receive channels into groups whose partial sums are
 * kept in a static device array of 262144 float2 entries (2 MiB) that every GPU
 * loading this library holds until the process exits. The call uses as many
 * groups as that array holds for the volume, down to one group, which writes
 * the frame directly and needs no partial sums, so no volume is refused for
 * lack of room. The first call on a device looks up the array's device
 * address; make that first call before any stream capture. After a
 * cudaDeviceReset, call beamformer_gb300_shutdown() before the next call so
 * that the address is looked up again. All calls share the array and the
 * tables, which keep the last call's contents, so calls that overlap on the
 * GPU race. */
LIB_FN uint32_t beamformer_gb300_das_no_alloc(const BeamformerParameters *das_parameters, const float *focal_vectors,
                                              const int16_t *sparse_elements, const void *channel_data,
                                              uint64_t channel_data_bytes, float *frame, void *cuda_stream);

/* Measured bandwidth of the GPU's shared-memory (L1) data path in bytes per
 * second, the roofline denominator of delay-and-sum: a conflict-free 16-byte-per-
 * lane streaming kernel on every SM, timed with CUDA events (best of six after
 * two warm-ups, about 0.1 s). A measurement aid with no counterpart in the
 * reference; it changes no clock or power setting. */
LIB_FN uint32_t beamformer_gb300_measure_shared_bandwidth(double *bytes_per_second);

/* Number of kernel launches this library issued since load (all streams). */
LIB_FN uint64_t beamformer_gb300_kernel_launch_count(void);

/* Release all device state (the next call re-initialises it). */
LIB_FN void     beamformer_gb300_shutdown(void);

#ifdef __cplusplus
}
#endif

#endif /* OGL_BEAMFORMER_LIB_H */
