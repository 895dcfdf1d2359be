/*
 * bf_kernels.h -- launch interface between the host library (bf_library.cpp)
 * and the sm_103a kernels (bf_decode.cu, bf_filter.cu, bf_das.cu,
 * bf_reduce.cu, bf_hilbert.cu, ...). Plain structs passed by value to the kernels.
 */
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bf {

/* Strides in elements of the stage's storage type, as the reference's stage
 * uniform blocks define them (beamformer.h:112-147). */
struct Strides {
	uint32_t in_channel, in_sample, in_transmit;
	uint32_t out_channel, out_sample, out_transmit;
};

/* ------------------------------- decode ---------------------------------- */
enum DecodeInput  { DEC_IN_I16 = 0, DEC_IN_I16C = 1, DEC_IN_F32 = 2, DEC_IN_F32C = 3 };
/* REAL_F16 / REAL_BF16: the real pairs layout as 16-bit floats (the precision
 * variant's input to the tensor-core FIR) */
enum DecodeOutput { DEC_OUT_COMPLEX = 0, DEC_OUT_REAL_PAIRS = 1, DEC_OUT_REAL_F16 = 2, DEC_OUT_REAL_BF16 = 3 };

struct DecodeParams {
	const void    *in;             /* raw RF or previous stage output */
	uint64_t       in_elems;       /* element count of `in` (bounds) */
	float         *out;            /* float2 output */
	uint64_t       out_vec2;       /* float2 count of `out` (bounds) */
	const int16_t *channel_map;    /* device, 256 entries; null = identity */
	const int8_t  *hadamard;       /* device, T*T, row = transmit */
	Strides        st;
	uint32_t       samples;        /* samples per transmit row to produce */
	uint32_t       in_limit;       /* samples at or beyond this read as zero (the reference's gather guard) */
	uint32_t       channels;
	uint32_t       transmits;      /* Hadamard order */
	uint32_t       sylvester;      /* Sylvester factor (power of two) */
	uint32_t       base;           /* 1, 12 or 20: dense factor of the Kronecker product */
	uint32_t       hadamard_mode;  /* 0 none (reshape), 1 Hadamard */
	uint32_t       first_stage;    /* map channels and read raw layout */
	int            input;          /* DecodeInput */
	int            output;         /* DecodeOutput */
};

/* --------------------------- demodulate / filter ------------------------- */
enum FilterKind { FILT_DEMOD_F32 = 0, FILT_DEMOD_I16 = 1, FILT_COMPLEX = 2 };

struct FilterParams {
	const void    *in;
	uint64_t       in_elems;
	void          *out;
	uint64_t       out_elems;
	const float   *taps;           /* device, reversed per phase (see bf_filter.cu) */
	const float2  *phasor;         /* device, per input index: (cos, sin) of the demodulation angle */
	const int16_t *channel_map;
	Strides        st;
	uint32_t       out_samples;    /* outputs per row (target) */
	uint32_t       in_samples;     /* inputs per row usable (target * decimation) */
	uint32_t       channels, transmits;
	uint32_t       decimation;
	uint32_t       taps_len;
	uint32_t       map_channels;
	int            kind;
	const float   *host_taps;      /* host, h[0 .. taps_len): the launcher passes them by value */
};

/* ---------------------------------- DAS ---------------------------------- */
enum DasFamily { DAS_FORCES = 0, DAS_HERCULES = 1, DAS_RCA = 2, DAS_NONE = 3 };
enum DasInterp { INTERP_NEAREST = 0, INTERP_CUBIC = 1, INTERP_LINEAR = 2 };

struct DasParams {
	const float2  *rf;
	int64_t        rf_count;       /* float2 samples readable (bound range of the reference) */
	float2        *frame;
	int32_t        dims[3];
	float          M[16];          /* voxel -> world, column major */
	float          X[16];          /* world -> transducer (xdc_transform) */
	int32_t        S, C, T;        /* dec_data_dim */
	int32_t        family, das_id, interp, fast, coherency, sparse_mode;
	int32_t        tx_rows, rx_cols, rx_rows, loop_end;
	float          fs, fc, c, toff;
	float          r360_fc;        /* radians(360) * center_frequency */
	float          apod_scale;     /* f_number * radians(180) */
	float          apod_hi;        /* 0.25 * radians(360) */
	float          inv_sqrt_T;
	float          px, py;
	float          cy_forces;      /* pitch.y * floor(channels / 2) */
	const float4  *focal;          /* per focal vector: sin(angle), cos(angle), depth, isinf(depth) */
	const int16_t *sparse;
	/* division by the constants c and fs: x * (1/b) corrected by one FMA, used only
	 * where a device-side exhaustive check proved it equal to IEEE division */
	float          rc, rfs;
	float          c_lo, c_hi, fs_lo, fs_hi;   /* verified ranges of x (empty: always IEEE) */
	/* split of the outer (receive channel / transmit) loop over groups of blocks;
	 * groups > 1 writes partial sums to `partial` (groups x voxels) */
	int32_t        groups, per_group;
	float2        *partial;
	/* receive-distance square root: 1 = rsqrt + one Newton step (checked equal to
	 * IEEE sqrt over [sqrt_lo, sqrt_hi]), 0 = IEEE sqrt */
	int32_t        fast_sqrt;
	int32_t        dense_rows;   /* rf holds exactly C*T*S samples (< 2^31), S >= 4: branch-free HERCULES path */
	int32_t        rx_step;      /* HERCULES: receive channels 0, rx_step, 2 rx_step, ... (1 = all) */
	float          sqrt_lo, sqrt_hi;
	/* HERCULES table interpolation with demodulation: rot_table = 1 stores the
	 * table segment of sample s rotated by exp(i theta (s + 1/2)), its phase in
	 * turns being (s * rot_step + rot_half) / 2^32 (0.32 fixed point of theta / 2 pi
	 * and theta / 4 pi, modulo 1), so a term at sample index s + f rotates only by
	 * exp(i theta (f - 1/2)); theta = r360_fc / fs. rot_table = 2: that angle is
	 * reduced to [-pi, pi] per term (|theta| > 2 pi) */
	int32_t        rot_table;
	uint32_t       rot_step, rot_half;
	float          theta, theta_half;
	/* DAS precision 1 (HERCULES fast path only): the table holds FP16 pairs of the
	 * coefficients times 2^k, k chosen per frame from the largest channel-data
	 * magnitude (*absmax, float bits, written by launch_das_table); the segment is
	 * evaluated in packed FP16, the sample index is sqrt(x) * fs_c + io with io =
	 * dtx * fs_c + toff_fs per voxel, and the voxel sums are multiplied by 2^-k */
	int32_t        half_table;
	unsigned      *absmax;
	float          fs_c, toff_fs;
	/* set to 1 by a kernel whose bounded wait ran out (the staged HERCULES path);
	 * beamformer_gb300_synchronize reports it */
	unsigned      *wait_error;
	/* tests only (OGL_BF_DAS_STAGED=require): blocks of the staged HERCULES kernel
	 * that cannot stage write NaN instead of running the unstaged code */
	int32_t        stage_only;
};

/* Exhaustively compare x * rb + correction with IEEE x / b for every float x in
 * [lo, hi]; *mismatch receives the count of differing x. */
cudaError_t launch_verify_sqrt(float lo, float hi, unsigned long long *mismatch, cudaStream_t s);
cudaError_t launch_verify_division(float b, float rb, float lo, float hi, unsigned long long *mismatch, cudaStream_t s);

/* launchers: return cudaSuccess or the launch error */
cudaError_t launch_decode(const DecodeParams &p, cudaStream_t s);
cudaError_t launch_filter(const FilterParams &p, cudaStream_t s);
cudaError_t launch_das(const DasParams &p, cudaStream_t s);
/* Precision variant of DemodulateFloat after a 16-bit Decode (bf_fir_tc.cu):
 * Toeplitz contraction on tcgen05 tensor cores, fp16/bf16 operands, f32
 * accumulate. `table` (fir_tc_table_bytes, device) holds the tap matrix and the
 * per-output rotations written by fir_tc_tables. */
bool        fir_tc_supported(uint32_t decimation, uint32_t taps);
/* the driver's cuTensorMapEncodeTiled (PFN_cuTensorMapEncodeTiled_v12000), or null */
void       *tensor_map_encoder();
int64_t     fir_tc_table_bytes(uint32_t decimation, uint32_t taps, uint32_t n_out);
bool        fir_tc_tables(uint32_t decimation, const float *h, uint32_t taps, double demod_frequency,
                          double demod_fs, uint32_t n_out, bool bf16, void *table);
cudaError_t launch_fir_tc(const void *x, uint32_t rows, uint32_t row_samples, uint32_t valid_samples,
                          uint32_t decimation, uint32_t taps, uint32_t n_out, bool bf16, const void *table,
                          float2 *out, unsigned *error, cudaStream_t s);
cudaError_t launch_das_reduce(const float2 *partial, float2 *frame, int64_t n, int groups, cudaStream_t s);
/* HERCULES fast path (bf_das_hercules.cu): for parameters das_hercules_supported
 * accepts; `table` holds das_hercules_table_bytes bytes (none: nearest FP32
 * interpolation of data that is not rotated) */
bool        das_hercules_supported(const DasParams &p);
/* blocks of one channel group of the HERCULES launch, and resident blocks per SM */
int64_t     das_hercules_tiles(const DasParams &p);
int         das_hercules_blocks_per_sm(const DasParams &p);
/* the HERCULES fast path of p reads its FP32 table staged in shared memory
 * (blocks whose windows do not fit still run the unstaged tile code) */
bool        das_hercules_use_staged(const DasParams &p);
int64_t     das_hercules_table_bytes(const DasParams &p);
cudaError_t launch_das_hercules(const DasParams &p, float4 *table, cudaStream_t s);
/* FORCES fast path (bf_das_forces.cu): the same per-frame table (das_hercules_table_bytes
 * bytes, built by the launch), for parameters das_forces_supported accepts */
bool        das_forces_supported(const DasParams &p);
cudaError_t launch_das_forces(const DasParams &p, float4 *table, cudaStream_t s);
cudaError_t launch_sum(float2 *out, const float2 *const *ins, int count, float prescale, const int32_t dims[3],
                       cudaStream_t s);
cudaError_t launch_min_max(const float2 *level0, const int32_t dims[3], int mips, float2 *levels, cudaStream_t s);

/* Batched DAS (bf_das_batch.cu): many acquisitions' voxel tiles in one
 * persistent launch. Each acquisition's DasParams has groups = 1. */
enum DasBatchPath { DAS_BATCH_HERC_VOLUME = 0, DAS_BATCH_HERC_PLANE = 1, DAS_BATCH_GENERIC = 2 };
struct DasBatchAcq {
	DasParams     p;
	const float4 *table;       /* HERCULES interpolation table (das_hercules_table_bytes) */
	int32_t       path;        /* DasBatchPath */
	int32_t       staged;      /* HERCULES tiles read the FP32 table staged in shared memory */
};
/* up to DAS_BATCH_MAX acquisitions per launch, passed by value in the kernel's
 * parameter space (read through the constant cache, like a single launch's) */
constexpr int DAS_BATCH_MAX = 64;
struct DasBatchArgs {
	DasBatchAcq acq[DAS_BATCH_MAX];
};
/* tile grid of an acquisition on a path; work items are int4 (acquisition, tile x, y, z) */
void        das_batch_tiles(const DasParams &p, int path, int tiles[3]);
cudaError_t launch_das_batch(const DasBatchArgs &args, const int4 *items, int n_items, int *counter, int interp,
                             bool general, bool half, int ctas, cudaStream_t s);
/* the per-frame HERCULES interpolation table alone (cubic / linear; nothing for nearest) */
cudaError_t launch_das_table(const DasParams &p, float4 *table, cudaStream_t s);

/* DAS with its partial sums and tables in static device arrays (no allocation);
 * capacity in float2 partial-sum entries (groups x voxels) */
cudaError_t launch_das_no_alloc(DasParams p, const float4 *focal4, const int16_t *sparse, cudaStream_t s);
int64_t     das_no_alloc_capacity();
void        das_no_alloc_forget_devices();

/* CudaHilbert stage (bf_hilbert.cu): analytic signal of each of `rows` rows of
 * `samples` complex values (real parts used), in -> out; samples a power of two
 * in [2, 16384]; twiddles = samples / 2 values from analytic_twiddles, on the
 * device */
bool        analytic_supported(uint32_t samples);
void        analytic_twiddles(uint32_t samples, float2 *host_out);
cudaError_t launch_analytic(const float2 *in, float2 *out, int64_t rows, uint32_t samples, const float2 *twiddles,
                            cudaStream_t s);

/* kernel launches issued since load (all launchers count here) */
extern uint64_t g_kernel_launches;

/* Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
 * looked up once per device); 1 if the query fails. Grid sizes follow it. */
int device_sm_count();

/* Measured bandwidth of the shared-memory data path (conflict-free LDS.128 from
 * every SM, best of six event-timed launches after two warm-ups). */
cudaError_t measure_shared_bandwidth(double *bytes_per_second, cudaStream_t s);

} /* namespace bf */
