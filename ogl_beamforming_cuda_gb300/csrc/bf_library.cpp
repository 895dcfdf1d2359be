/*
 * bf_library.cpp -- the C ABI of include/ogl_beamformer_lib.h.
 *
 * In-process replacement of the reference's client library
 * (helpers/ogl_beamformer_lib.c) together with the compute side of its server
 * (beamformer.c: complete_queue :842-1111, do_compute_shader :521-709,
 * beamformer_rf_upload :1230-1276, coalesce_timing_table :1113-1173).
 *
 * Data flow of one compute on the GPU:
 *   RF push (host -> device, upload stream, 3-slot ring as the reference's
 *   MAX_RAW_DATA_FRAMES_IN_FLIGHT) -> compute stream waits on the upload event
 *   -> planned stages (decode, demodulate/filter, DAS, sum, min/max) on two
 *   ping-pong channel buffers and a 16-frame ring -> events per stage feed the
 *   timing table.
 *
 * Error behaviour follows the reference: every entry point returns 1/0 (or a
 * pointer/-1) and sets a process-global last error. Validation that needs no
 * device (pipeline, sizes, timeouts) runs before any CUDA call, as the
 * reference validates before touching shared memory.
 */
#include "ogl_beamformer_lib.h"
#include "bf_host.h"

#include <algorithm>
#include <chrono>
#include <cmath>

#include <nvtx3/nvToolsExt.h>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

using namespace bf;

namespace {

constexpr int RF_SLOTS = 3;                 /* MAX_RAW_DATA_FRAMES_IN_FLIGHT (beamformer.h:180) */
constexpr int TIMING_SLOTS = 8;
constexpr uint64_t SCRATCH_SIZE = BEAMFORMER_MAX_RF_DATA_SIZE;

struct DeviceFrame {
	float2  *data = nullptr;
	float2  *levels = nullptr;
	int32_t  dims[3] = {0, 0, 0};
	int32_t  mips = 0;
	uint64_t level_texels = 0;
	bool     written = false;
};

struct PendingTiming {
	cudaEvent_t ev[MAX_COMPUTE_SHADER_STAGES + 1] = {};
	int32_t     shaders[MAX_COMPUTE_SHADER_STAGES] = {};
	int32_t     count = 0;
	bool        active = false;
};

struct StageTables {
	float   *taps = nullptr;     /* polyphase-arranged taps */
	size_t   taps_cap = 0;
	float2  *phasor = nullptr;   /* demodulation phasor per input index */
	size_t   phasor_cap = 0;
};

struct Context {
	/* ---- state pushed by the caller ---- */
	BeamformerParameters params{};
	int32_t  shaders[MAX_COMPUTE_SHADER_STAGES] = {};
	uint8_t  slots[MAX_COMPUTE_SHADER_STAGES] = {};
	int32_t  shader_count = 0;
	int32_t  data_kind = BeamformerDataKind_Int16;
	int16_t  channel_mapping[256];
	int16_t  sparse_elements[256];
	float    focal_vectors[512] = {};
	FilterSpec filters[BEAMFORMER_FILTER_SLOTS];
	std::vector<float> taps[BEAMFORMER_FILTER_SLOTS];
	BeamformerLiveImagingParameters live{};
	uint32_t live_dirty = 0;
	int32_t  timeout_ms = 0;
	BeamformerLibErrorKind last_error = BF_LIB_ERR_KIND_NONE;
	bool     dirty = true;

	/* ---- device ---- */
	bool         ready = false;
	cudaStream_t own_stream = nullptr, stream = nullptr, upload_stream = nullptr;
	void        *raw[RF_SLOTS] = {};
	uint64_t     raw_cap = 0, raw_size[RF_SLOTS] = {};
	cudaEvent_t  upload_done[RF_SLOTS] = {}, compute_done[RF_SLOTS] = {};
	bool         slot_used[RF_SLOTS] = {};
	uint32_t     insert_index = 0;
	int          latest_slot = -1;
	const void  *ext_rf = nullptr;
	uint64_t     ext_size = 0;
	bool         use_ext = false;
	cudaEvent_t  ext_done = nullptr, last_done = nullptr;
	cudaEvent_t  caller_ready = nullptr;     /* recorded on the legacy default stream */

	float2      *chan[2] = {};
	uint64_t     chan_bytes = 0;         /* allocated */
	uint64_t     chan_used = 0;          /* size the current plan uses */
	int          last_chan = -1;

	int8_t      *hadamard = nullptr;
	int32_t      hadamard_order = 0, hadamard_sylvester = 0, hadamard_base = 0;
	bool         hadamard_ok = false;
	int16_t     *d_chmap = nullptr, *d_sparse = nullptr;
	float4      *d_focal = nullptr;
	StageTables  stage_tables[MAX_COMPUTE_SHADER_STAGES];

	Plan         plan{};
	bool         plan_ok = false;
	float        M[16] = {};

	DeviceFrame  frames[MAX_BEAMFORMED_SAVED_FRAMES];
	DeviceFrame  averaged[2];
	uint32_t     frame_counter = 0, averaged_counter = 0;
	int          latest_kind = -1, latest_index = -1;   /* 0 frame ring, 1 averaged */
	int          latest_das_index = -1;

	PendingTiming timing[TIMING_SLOTS];
	uint32_t     timing_next = 0;
	BeamformerComputeStatsTable stats{};
	uint32_t     stats_index = 0, rf_delta_index = 0;
	std::chrono::steady_clock::time_point last_upload{};
	bool         have_last_upload = false;
	int32_t      interpolation_override = -1;
	/* precision variant: 0 FP32 (reference arithmetic), 1 FP16, 2 BF16 Decode output
	 * and tensor-core Demodulate FIR */
	int32_t      precision = 0;
	/* DAS precision: 0 FP32 (reference arithmetic), 1 FP16 interpolation table
	 * (HERCULES fast path; other DAS paths stay FP32) */
	int32_t      das_precision = 0;
	unsigned    *d_absmax = nullptr;      /* per-frame channel-data magnitude of the FP16 table */
	int32_t      rx_step = 1;             /* receive subsampling of HERCULES DAS (learned variant input) */
	bool         tc_active = false;
	void        *tc_table = nullptr;
	size_t       tc_table_cap = 0;
	unsigned    *d_tc_error = nullptr;

	/* DAS: partial sums of channel groups, and verified division ranges per divisor */
	float2      *das_partial = nullptr;
	uint64_t     das_partial_bytes = 0;
	float4      *das_table = nullptr;         /* HERCULES interpolation table */
	uint64_t     das_table_bytes = 0;
	float2      *d_hilbert_tw = nullptr;      /* CudaHilbert FFT twiddles for hilbert_n samples */
	uint32_t     hilbert_n = 0;
	unsigned long long *d_mismatch = nullptr;
	struct DivCheck { float b, lo, hi; };
	std::vector<DivCheck> div_checks;
	int          sqrt_checked = -1;      /* -1 unknown, 0 IEEE only, 1 Newton sqrt verified */

	Context()
	{
		for (int i = 0; i < 256; i++) { channel_mapping[i] = (int16_t)i; sparse_elements[i] = (int16_t)i; }
	}
};

Context g;

uint32_t fail(BeamformerLibErrorKind k)
{
	g.last_error = k;
	return 0;
}

bool cuda_ok(cudaError_t e)
{
	if (e != cudaSuccess) {
		g.last_error = BF_LIB_ERR_KIND_CUDA_RUNTIME;
		cudaGetLastError();
		return false;
	}
	return true;
}

/* Wait for an event with the reference's timeout convention: -1 forever,
 * 0 one try, N milliseconds. */
bool wait_event(cudaEvent_t ev, int32_t timeout_ms)
{
	if (!ev) return true;
	if (timeout_ms < 0) return cudaEventSynchronize(ev) == cudaSuccess;
	auto start = std::chrono::steady_clock::now();
	for (;;) {
		cudaError_t e = cudaEventQuery(ev);
		if (e == cudaSuccess) return true;
		if (e != cudaErrorNotReady) { cudaGetLastError(); return false; }
		auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - start).count();
		if (ms >= timeout_ms) return false;
		std::this_thread::sleep_for(std::chrono::microseconds(50));
	}
}

bool ensure_cuda()
{
	if (g.ready) return true;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
		cudaGetLastError();
		return fail(BF_LIB_ERR_KIND_CUDA_DEVICE), false;
	}
	if (!cuda_ok(cudaStreamCreateWithFlags(&g.own_stream, cudaStreamNonBlocking))) return false;
	if (!cuda_ok(cudaStreamCreateWithFlags(&g.upload_stream, cudaStreamNonBlocking))) return false;
	for (int i = 0; i < RF_SLOTS; i++) {
		if (!cuda_ok(cudaEventCreateWithFlags(&g.upload_done[i], cudaEventDisableTiming))) return false;
		if (!cuda_ok(cudaEventCreateWithFlags(&g.compute_done[i], cudaEventDisableTiming))) return false;
	}
	if (!cuda_ok(cudaEventCreateWithFlags(&g.ext_done, cudaEventDisableTiming))) return false;
	if (!cuda_ok(cudaEventCreateWithFlags(&g.caller_ready, cudaEventDisableTiming))) return false;
	for (auto &t : g.timing)
		for (auto &e : t.ev)
			if (!cuda_ok(cudaEventCreate(&e))) return false;
	if (!cuda_ok(cudaMalloc(&g.d_chmap, 256 * sizeof(int16_t)))) return false;
	if (!cuda_ok(cudaMalloc(&g.d_sparse, 256 * sizeof(int16_t)))) return false;
	if (!cuda_ok(cudaMalloc(&g.d_focal, 256 * sizeof(float4)))) return false;
	if (!g.stream) g.stream = g.own_stream;
	g.ready = true;
	g.dirty = true;
	return true;
}

void free_frame(DeviceFrame &f)
{
	cudaFree(f.data);
	cudaFree(f.levels);
	f = DeviceFrame{};
}

bool ensure_frame(DeviceFrame &f, const int32_t dims[3])
{
	if (f.data && f.dims[0] == dims[0] && f.dims[1] == dims[1] && f.dims[2] == dims[2]) return true;
	free_frame(f);
	uint64_t n = (uint64_t)dims[0] * dims[1] * dims[2];
	f.mips = frame_mips(dims);
	f.level_texels = 0;
	for (int l = 1; l < f.mips; l++) {
		uint64_t x = (uint64_t)dims[0] >> l, y = (uint64_t)dims[1] >> l, z = (uint64_t)dims[2] >> l;
		f.level_texels += (x ? x : 1) * (y ? y : 1) * (z ? z : 1);
	}
	if (!cuda_ok(cudaMalloc(&f.data, n * sizeof(float2)))) return false;
	if (f.level_texels && !cuda_ok(cudaMalloc(&f.levels, f.level_texels * sizeof(float2)))) return false;
	cudaMemsetAsync(f.data, 0, n * sizeof(float2), g.stream);
	std::memcpy(f.dims, dims, sizeof(f.dims));
	f.written = false;
	return true;
}

/* (Re)build everything derived from the pushed state. */
/* Channel mapping, sparse elements and focal vectors (sin/cos of the angle on
 * the host) to the device. */
bool upload_element_tables()
{
	float4 focal[256];
	for (int i = 0; i < 256; i++) {
		float angle = g.focal_vectors[2 * i] * DEG2RAD_F;
		float depth = g.focal_vectors[2 * i + 1];
		focal[i] = make_float4(sinf(angle), cosf(angle), depth, std::isinf(depth) ? 1.0f : 0.0f);
	}
	if (!cuda_ok(cudaMemcpy(g.d_chmap, g.channel_mapping, sizeof(g.channel_mapping), cudaMemcpyHostToDevice))) return false;
	if (!cuda_ok(cudaMemcpy(g.d_sparse, g.sparse_elements, sizeof(g.sparse_elements), cudaMemcpyHostToDevice))) return false;
	if (!cuda_ok(cudaMemcpy(g.d_focal, focal, sizeof(focal), cudaMemcpyHostToDevice))) return false;
	return true;
}

/* Per-stage filter taps (polyphase arranged) and demodulation phasors of a plan. */
bool build_stage_tables(const Plan &pl, StageTables *tables)
{
	for (int i = 0; i < pl.count; i++) {
		int k = pl.shaders[i];
		if (k != BeamformerShaderKind_Demodulate && k != BeamformerShaderKind_DemodulateFloat &&
		    k != BeamformerShaderKind_Filter)
			continue;
		const bool is_filter = k == BeamformerShaderKind_Filter;
		const std::vector<float> &h = g.taps[pl.slots[i] % BEAMFORMER_FILTER_SLOTS];
		const uint32_t L = (uint32_t)h.size();
		const uint32_t D = is_filter ? 1 : pl.demod_decimation;
		const uint32_t Lp = (L + D - 1) / D, Lpad = Lp * D;
		std::vector<float> hp((size_t)D * Lp, 0.0f);
		for (uint32_t kp = Lpad - L; kp < Lpad; kp++) hp[(size_t)(kp % D) * Lp + kp / D] = h[Lpad - 1 - kp];
		StageTables &st = tables[i];
		if (hp.size() > st.taps_cap) {
			cudaFree(st.taps);
			st.taps = nullptr;
			if (!cuda_ok(cudaMalloc(&st.taps, hp.size() * sizeof(float)))) return false;
			st.taps_cap = hp.size();
		}
		if (!cuda_ok(cudaMemcpyAsync(st.taps, hp.data(), hp.size() * sizeof(float), cudaMemcpyHostToDevice, g.stream)))
			return false;
		cudaStreamSynchronize(g.stream);
		if (!is_filter) {
			const bool map = pl.demod_map != 0;
			const uint32_t target = map ? pl.demod_st.out_channel / pl.demod_st.out_sample : pl.demod_st.out_transmit;
			const uint32_t n_in = target * D;
			std::vector<float2> ph(n_in);
			const float r360 = 360.0f * DEG2RAD_F;
			for (uint32_t j = 0; j < n_in; j++) {
				/* filter.glsl rotate_iq(v, -j): radians(360) * f * index / fs */
				float arg = r360 * pl.demod_frequency * (float)(-(int32_t)j) / pl.demod_fs;
				ph[j] = make_float2(cosf(arg), sinf(arg));
			}
			if (n_in > st.phasor_cap) {
				cudaFree(st.phasor);
				st.phasor = nullptr;
				if (!cuda_ok(cudaMalloc(&st.phasor, n_in * sizeof(float2)))) return false;
				st.phasor_cap = n_in;
			}
			if (n_in && !cuda_ok(cudaMemcpy(st.phasor, ph.data(), n_in * sizeof(float2), cudaMemcpyHostToDevice)))
				return false;
		}
	}
	return true;
}

/* Precision variant: a first-stage int16 Hadamard Decode (fast Walsh-Hadamard
 * orders) writing fp16/bf16, followed by DemodulateFloat on the tensor cores, with
 * dense [channel][transmit][sample] layouts. Other pipelines fail UNSUPPORTED
 * while a 16-bit precision is selected. */
bool prepare_precision()
{
	g.tc_active = false;
	if (g.precision == 0) return true;
	const Plan &pl = g.plan;
	const uint32_t T = pl.das.dec_data_dim[2], C = pl.das.dec_data_dim[1];
	bool ok = pl.count >= 2 && pl.shaders[0] == BeamformerShaderKind_DecodeInt16ToFloat &&
	          pl.shaders[1] == BeamformerShaderKind_DemodulateFloat && g.data_kind == BeamformerDataKind_Int16 &&
	          pl.decode_mode == DECODE_MODE_HADAMARD && g.hadamard_ok && g.hadamard_base == 1 &&
	          (uint32_t)g.hadamard_sylvester == pl.transmit_count && pl.transmit_count <= 128;
	const Strides &ds = pl.decode_st, &ms = pl.demod_st;
	const std::vector<float> &h = g.taps[pl.slots[1] % BEAMFORMER_FILTER_SLOTS];
	const uint32_t L = (uint32_t)h.size(), D = pl.demod_decimation, n_out = ms.out_transmit;
	ok = ok && ds.out_sample == 1 && ds.out_channel == (uint64_t)ds.out_transmit * T && ms.in_sample == 1 &&
	     ms.in_transmit == ds.out_transmit && ms.in_channel == ds.out_channel && ms.out_sample == 1 &&
	     ms.out_channel == (uint64_t)n_out * T && (2 * ds.out_transmit) % 8 == 0 && n_out > 0 &&
	     (uint64_t)C * T * n_out * 8 <= g.chan_bytes && fir_tc_supported(D, L);
	if (!ok) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
	const size_t need = (size_t)fir_tc_table_bytes(D, L, n_out);
	if (need > g.tc_table_cap) {
		cudaStreamSynchronize(g.stream);
		cudaFree(g.tc_table);
		g.tc_table = nullptr;
		g.tc_table_cap = 0;
		if (!cuda_ok(cudaMalloc(&g.tc_table, need))) return false;
		g.tc_table_cap = need;
	}
	if (!g.d_tc_error) {
		if (!cuda_ok(cudaMalloc(&g.d_tc_error, sizeof(unsigned)))) return false;
		if (!cuda_ok(cudaMemset(g.d_tc_error, 0, sizeof(unsigned)))) return false;
	}
	cudaStreamSynchronize(g.stream);
	if (!fir_tc_tables(D, h.data(), L, pl.demod_frequency, pl.demod_fs, n_out, g.precision == 2, g.tc_table))
		return fail(BF_LIB_ERR_KIND_CUDA_RUNTIME), false;
	g.tc_active = true;
	return true;
}

bool prepare()
{
	if (!g.dirty && g.plan_ok) return true;
	g.plan_ok = false;
	plan_pipeline(g.params, g.shaders, g.slots, g.shader_count, g.data_kind, g.filters, g.plan);
	const Plan &pl = g.plan;

	for (int i = 0; i < pl.count; i++) {
		int k = pl.shaders[i];
		if (k == BeamformerShaderKind_Render3D) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
		if (k == BeamformerShaderKind_CudaHilbert) {
			/* analytic signal by a power-of-two FFT per row */
			const uint32_t n = pl.das.dec_data_dim[0];
			if (!analytic_supported(n)) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
			if (n != g.hilbert_n) {
				std::vector<float2> tw(n / 2);
				analytic_twiddles(n, tw.data());
				cudaStreamSynchronize(g.stream);
				cudaFree(g.d_hilbert_tw);
				g.d_hilbert_tw = nullptr;
				g.hilbert_n = 0;
				if (!cuda_ok(cudaMalloc(&g.d_hilbert_tw, tw.size() * sizeof(float2)))) return false;
				if (!cuda_ok(cudaMemcpy(g.d_hilbert_tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice)))
					return false;
				g.hilbert_n = n;
			}
		}
		if (k == BeamformerShaderKind_Demodulate || k == BeamformerShaderKind_DemodulateFloat ||
		    k == BeamformerShaderKind_Filter) {
			const FilterSpec &f = g.filters[pl.slots[i] % BEAMFORMER_FILTER_SLOTS];
			if (f.kind < 0 || f.length <= 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS), false;
		}
	}

	/* channel buffers: 2 * 4 * samples * channels * transmits (beamformer.c:165) */
	uint64_t need = 8ull * g.params.dec_data_dim[0] * g.params.dec_data_dim[1] * g.params.dec_data_dim[2];
	if (need > g.chan_bytes) {
		cudaStreamSynchronize(g.stream);
		cudaFree(g.chan[0]); cudaFree(g.chan[1]);
		g.chan[0] = g.chan[1] = nullptr;
		g.chan_bytes = 0;
		if (!cuda_ok(cudaMalloc(&g.chan[0], need)) || !cuda_ok(cudaMalloc(&g.chan[1], need))) return false;
		cudaMemsetAsync(g.chan[0], 0, need, g.stream);
		cudaMemsetAsync(g.chan[1], 0, need, g.stream);
		g.chan_bytes = need;
	}
	g.chan_used = need;
	/* a new plan may write only part of a channel buffer (the reference's dispatch
	 * grid decides); start it from zeros rather than the previous plan's data */
	cudaMemsetAsync(g.chan[0], 0, g.chan_bytes, g.stream);
	cudaMemsetAsync(g.chan[1], 0, g.chan_bytes, g.stream);

	/* Hadamard matrix for the transmit count (uploaded as the reference does when dims change) */
	int32_t order = (int32_t)g.params.dec_data_dim[2];
	if (order != g.hadamard_order) {
		std::vector<int8_t> h;
		g.hadamard_ok = hadamard_matrix(order, h, g.hadamard_sylvester, g.hadamard_base);
		cudaStreamSynchronize(g.stream);
		cudaFree(g.hadamard);
		g.hadamard = nullptr;
		if (g.hadamard_ok) {
			if (!cuda_ok(cudaMalloc(&g.hadamard, h.size()))) return false;
			if (!cuda_ok(cudaMemcpy(g.hadamard, h.data(), h.size(), cudaMemcpyHostToDevice))) return false;
		}
		g.hadamard_order = order;
	}
	if (!prepare_precision()) return false;

	bool uses_decode = false;
	for (int i = 0; i < pl.count; i++)
		if (pl.shaders[i] == BeamformerShaderKind_Decode || pl.shaders[i] == BeamformerShaderKind_DecodeInt16Complex ||
		    pl.shaders[i] == BeamformerShaderKind_DecodeFloat || pl.shaders[i] == BeamformerShaderKind_DecodeFloatComplex ||
		    pl.shaders[i] == BeamformerShaderKind_DecodeInt16ToFloat || pl.shaders[i] == BeamformerShaderKind_CudaDecode)
			uses_decode = true;
	if (uses_decode && pl.decode_mode == DECODE_MODE_HADAMARD && !g.hadamard_ok)
		return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;

	if (!build_stage_tables(pl, g.stage_tables)) return false;

	if (!upload_element_tables()) return false;

	voxel_transform(pl.das, g.M);
	g.plan_ok = true;
	g.dirty = false;
	return true;
}


/* Range of dividends for which the reciprocal division by b is exact (checked
 * once per divisor on the device); an empty range (lo > hi) means IEEE division. */
bool division_range(float b, float lo, float hi, float &out_lo, float &out_hi)
{
	for (const auto &d : g.div_checks)
		if (d.b == b && d.lo <= lo) { out_lo = d.lo; out_hi = d.hi; return true; }
	out_lo = INFINITY; out_hi = 0.0f;
	if (!(b > 0.0f) || !std::isfinite(b)) return true;
	if (!g.d_mismatch && !cuda_ok(cudaMalloc(&g.d_mismatch, sizeof(unsigned long long)))) return false;
	unsigned long long bad = 0;
	if (!cuda_ok(cudaMemsetAsync(g.d_mismatch, 0, sizeof(bad), g.stream))) return false;
	if (!cuda_ok(launch_verify_division(b, 1.0f / b, lo, hi, g.d_mismatch, g.stream))) return false;
	if (!cuda_ok(cudaMemcpyAsync(&bad, g.d_mismatch, sizeof(bad), cudaMemcpyDeviceToHost, g.stream))) return false;
	if (!cuda_ok(cudaStreamSynchronize(g.stream))) return false;
	if (bad == 0) { out_lo = lo; out_hi = hi; }
	g.div_checks.push_back({b, out_lo, out_hi});
	return true;
}

/* Check once whether the rsqrt + Newton square root equals IEEE sqrt on every
 * float in [2^-40, 2^24] (squared receive distances in m^2 lie far inside). */
bool sqrt_verified()
{
	if (g.sqrt_checked >= 0) return g.sqrt_checked == 1;
	if (!g.d_mismatch && !cuda_ok(cudaMalloc(&g.d_mismatch, sizeof(unsigned long long)))) return false;
	unsigned long long bad = 1;
	if (cudaMemsetAsync(g.d_mismatch, 0, sizeof(bad), g.stream) == cudaSuccess &&
	    launch_verify_sqrt(0x1p-40f, 0x1p24f, g.d_mismatch, g.stream) == cudaSuccess &&
	    cudaMemcpyAsync(&bad, g.d_mismatch, sizeof(bad), cudaMemcpyDeviceToHost, g.stream) == cudaSuccess &&
	    cudaStreamSynchronize(g.stream) == cudaSuccess) {
		g.sqrt_checked = bad == 0 ? 1 : 0;
	} else {
		cudaGetLastError();
		g.sqrt_checked = 0;
	}
	return g.sqrt_checked == 1;
}

bool ensure_raw_capacity(uint64_t size)
{
	if (size <= g.raw_cap) return true;
	for (int i = 0; i < RF_SLOTS; i++)
		if (g.slot_used[i]) cudaEventSynchronize(g.compute_done[i]);
	cudaStreamSynchronize(g.upload_stream);
	uint64_t cap = (size + (2ull << 20) - 1) & ~((2ull << 20) - 1);
	for (int i = 0; i < RF_SLOTS; i++) {
		cudaFree(g.raw[i]);
		g.raw[i] = nullptr;
	}
	g.raw_cap = 0;
	for (int i = 0; i < RF_SLOTS; i++)
		if (!cuda_ok(cudaMalloc(&g.raw[i], cap))) return false;
	g.raw_cap = cap;
	return true;
}

void note_upload()
{
	auto now = std::chrono::steady_clock::now();
	if (g.have_last_upload) {
		float dt = std::chrono::duration<float>(now - g.last_upload).count();
		g.rf_delta_index = (g.rf_delta_index + 1) % 32;
		g.stats.rf_time_deltas[g.rf_delta_index] = dt;
	}
	g.last_upload = now;
	g.have_last_upload = true;
}

uint32_t push_data_base(const void *data, uint64_t size, int32_t timeout_ms)
{
	if (size > BEAMFORMER_MAX_RF_DATA_SIZE) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	if (!data && size) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!ensure_cuda()) return 0;
	int slot = (int)(g.insert_index % RF_SLOTS);
	/* the slot may still be read by an in-flight compute (the reference's upload
	 * thread waits on the slot's compute fence, beamformer.c:1243-1256) */
	if (g.slot_used[slot] && !wait_event(g.compute_done[slot], timeout_ms)) return fail(BF_LIB_ERR_KIND_SYNC_VARIABLE);
	if (!ensure_raw_capacity(size)) return 0;
	if (size && !cuda_ok(cudaMemcpyAsync(g.raw[slot], data, size, cudaMemcpyHostToDevice, g.upload_stream))) return 0;
	if (!cuda_ok(cudaEventRecord(g.upload_done[slot], g.upload_stream))) return 0;
	/* the caller may reuse its buffer as soon as this returns */
	if (!cuda_ok(cudaEventSynchronize(g.upload_done[slot]))) return 0;
	g.raw_size[slot] = size;
	g.latest_slot = slot;
	g.insert_index++;
	g.use_ext = false;
	note_upload();
	return 1;
}

void collect_timings(bool block)
{
	for (int n = 0; n < TIMING_SLOTS; n++) {
		PendingTiming &t = g.timing[(g.timing_next + n) % TIMING_SLOTS];
		if (!t.active) continue;
		if (!block && cudaEventQuery(t.ev[t.count]) != cudaSuccess) { cudaGetLastError(); continue; }
		if (block) cudaEventSynchronize(t.ev[t.count]);
		float *row = g.stats.times[g.stats_index % 32];
		std::memset(row, 0, sizeof(g.stats.times[0]));
		for (int i = 0; i < t.count; i++) {
			float ms = 0;
			if (cudaEventElapsedTime(&ms, t.ev[i], t.ev[i + 1]) == cudaSuccess && t.shaders[i] >= 0 &&
			    t.shaders[i] < BeamformerShaderKind_Count)
				row[t.shaders[i]] += ms * 1e-3f;
			cudaGetLastError();
		}
		g.stats_index++;
		t.active = false;
	}
}

/* Decode stage i of a plan: src = the pushed RF (first stage), in_buf / out_buf =
 * channel buffers of buf_bytes each. */
void fill_decode_params(const Plan &pl, int i, const void *src, uint64_t src_bytes, void *in_buf, void *out_buf,
                        uint64_t buf_bytes, const int8_t *hadamard, int sylvester, int base, DecodeParams &p)
{
	const int kind = pl.shaders[i];
	const bool first = i == 0;
	p.first_stage = first;
	if (first) {
		p.in = src;
		switch (g.data_kind) {
		case BeamformerDataKind_Int16Complex:   p.input = DEC_IN_I16C; p.in_elems = src_bytes / 4; break;
		case BeamformerDataKind_Float32:        p.input = DEC_IN_F32;  p.in_elems = src_bytes / 4; break;
		case BeamformerDataKind_Float32Complex: p.input = DEC_IN_F32C; p.in_elems = src_bytes / 8; break;
		default:                                p.input = DEC_IN_I16;  p.in_elems = src_bytes / 2; break;
		}
		p.channel_map = g.d_chmap;
	} else {
		p.in = in_buf;
		p.input = kind == BeamformerShaderKind_DecodeInt16Complex ? DEC_IN_I16C : DEC_IN_F32C;
		p.in_elems = buf_bytes / (p.input == DEC_IN_I16C ? 4 : 8);
		p.channel_map = nullptr;
	}
	p.out = (float *)out_buf;
	p.out_vec2 = buf_bytes / 8;
	p.hadamard = hadamard;
	p.st = pl.decode_st;
	p.output = kind == BeamformerShaderKind_DecodeInt16ToFloat ? DEC_OUT_REAL_PAIRS : DEC_OUT_COMPLEX;
	/* samples the reference's dispatch writes: pass-2 guard (time sample < output
	 * transmit stride) and grid width; int16 data decoded first packs two samples
	 * per invocation */
	const uint32_t ots = pl.decode_st.out_transmit, cov = pl.decode_invocations_x;
	const bool pairs = first && g.data_kind == BeamformerDataKind_Int16;
	if (p.output == DEC_OUT_REAL_PAIRS || p.output == DEC_OUT_REAL_F16 || p.output == DEC_OUT_REAL_BF16)
		p.samples = 2 * std::min(ots, cov);
	else if (pairs)
		p.samples = 2 * std::min((ots + 1) / 2, cov);
	else
		p.samples = std::min(ots, cov);
	/* pass-1 gather guard: time sample < input transmit stride */
	p.in_limit = first ? (pairs ? (pl.decode_st.in_transmit + 1) / 2 * 2 : pl.decode_st.in_transmit) : 0xFFFFFFFFu;
	p.channels = pl.das.dec_data_dim[1];
	p.transmits = pl.transmit_count;
	p.sylvester = (uint32_t)sylvester;
	p.base = (uint32_t)base;
	p.hadamard_mode = pl.decode_mode == DECODE_MODE_HADAMARD;
}

/* Demodulate / Filter stage i of a plan (see fill_decode_params). */
void fill_filter_params(const Plan &pl, int i, const void *src, uint64_t src_bytes, void *in_buf, void *out_buf,
                        uint64_t buf_bytes, const StageTables &st, FilterParams &p)
{
	const int kind = pl.shaders[i];
	const bool is_filter = kind == BeamformerShaderKind_Filter;
	const bool map = !is_filter && pl.demod_map;
	p.kind = is_filter ? FILT_COMPLEX : kind == BeamformerShaderKind_Demodulate ? FILT_DEMOD_I16 : FILT_DEMOD_F32;
	if (map) {
		p.in = src;
		p.in_elems = src_bytes / (p.kind == FILT_DEMOD_I16 ? 4 : 8);
	} else {
		p.in = in_buf;
		p.in_elems = buf_bytes / 8;
	}
	p.out = out_buf;
	p.out_elems = buf_bytes / (p.kind == FILT_DEMOD_I16 ? 4 : 8);
	p.st = is_filter ? pl.filter_st : pl.demod_st;
	p.decimation = is_filter ? 1 : pl.demod_decimation;
	p.map_channels = map;
	p.channel_map = g.d_chmap;
	p.out_samples = map ? p.st.out_channel / p.st.out_sample : p.st.out_transmit;
	p.in_samples = p.out_samples * p.decimation;
	p.channels = pl.das.dec_data_dim[1];
	p.transmits = pl.das.dec_data_dim[2];
	p.taps = st.taps;
	p.phasor = st.phasor;
	p.taps_len = (uint32_t)g.taps[pl.slots[i] % BEAMFORMER_FILTER_SLOTS].size();
	p.host_taps = g.taps[pl.slots[i] % BEAMFORMER_FILTER_SLOTS].data();
}

/* Phase rotation of the HERCULES interpolation table (DasParams::rot_table):
 * used for demodulated data. 1: the per-term angle theta (f - 1/2), f in
 * [0, 1) (nearest: theta (idx - round(idx))), stays within [-pi, pi], the range
 * of the fast sine and cosine; 2: |theta| up to 256, the angle reduced per term
 * first (decimation 4 gives theta = 4 pi). Nearest interpolation uses the rotated
 * samples only for voxels whose indices are proven in range. */
static uint32_t turns_q32(double turns)
{
	const double fr = turns - std::floor(turns);
	return (uint32_t)((uint64_t)std::llround(fr * 4294967296.0) & 0xffffffffu);
}

void set_das_rotation(DasParams &p)
{
	const double theta = (double)p.r360_fc / (double)p.fs;
	p.theta = (float)theta;
	p.theta_half = (float)(0.5 * theta);
	const bool table = p.fc > 0.0f && std::isfinite(theta) && std::fabs(theta) <= 256.0;
	p.rot_table = !table ? 0 : std::fabs(theta) <= 2.0 * M_PI * (1.0 + 1e-6) ? 1 : 2;
	p.rot_step = p.rot_table ? turns_q32(theta / (2.0 * M_PI)) : 0;
	/* segments are rotated at their middle (j + 1/2), nearest samples at j */
	p.rot_half = p.rot_table && p.interp != INTERP_NEAREST ? turns_q32(theta / (4.0 * M_PI)) : 0;
}

/* DAS stage of a plan reading channel data rf (rf_bytes readable) into frame
 * (dims, voxel transform M); the outer loop is not split (groups = 1). */
bool fill_das_params(const Plan &pl, int kind, const void *rf, uint64_t rf_bytes, float2 *frame,
                     const int32_t dims[3], const float M[16], DasParams &p)
{
	const BeamformerParameters &d = pl.das;
	p.rf = (const float2 *)rf;
	uint64_t readable = pl.rf_size / 8;
	p.rf_count = (int64_t)(readable < rf_bytes / 8 ? readable : rf_bytes / 8);
	p.frame = frame;
	std::memcpy(p.dims, dims, sizeof(p.dims));
	std::memcpy(p.M, M, sizeof(p.M));
	std::memcpy(p.X, d.xdc_transform, sizeof(p.X));
	p.S = (int32_t)d.dec_data_dim[0];
	p.C = (int32_t)d.dec_data_dim[1];
	p.T = (int32_t)d.dec_data_dim[2];
	p.das_id = (int32_t)d.das_shader_id;
	switch (d.das_shader_id) {
	case DASShaderKind_FORCES: case DASShaderKind_UFORCES:       p.family = DAS_FORCES; break;
	case DASShaderKind_HERCULES: case DASShaderKind_UHERCULES:   p.family = DAS_HERCULES; break;
	case DASShaderKind_RCA_VLS: case DASShaderKind_RCA_TPW:
	case DASShaderKind_FLASH:                                     p.family = DAS_RCA; break;
	default:                                                      p.family = DAS_NONE; break;
	}
	p.sparse_mode = d.das_shader_id == DASShaderKind_UFORCES || d.das_shader_id == DASShaderKind_UHERCULES;
	p.fast = kind == BeamformerShaderKind_DASFast;
	p.coherency = d.coherency_weighting != 0;
	p.interp = g.interpolation_override >= 0 ? g.interpolation_override : (d.interpolate ? INTERP_CUBIC : INTERP_NEAREST);
	p.tx_rows = !((d.transmit_mode & 2) != 0);
	p.rx_cols = (d.transmit_mode & 1) != 0;
	p.rx_rows = !p.rx_cols;
	p.loop_end = (d.das_shader_id == DASShaderKind_RCA_VLS || d.das_shader_id == DASShaderKind_RCA_TPW) ? p.T : p.C;
	p.fs = d.sampling_frequency;
	p.fc = d.center_frequency;
	p.c = d.speed_of_sound;
	p.toff = d.time_offset;
	const float r360 = 360.0f * DEG2RAD_F;
	p.r360_fc = r360 * d.center_frequency;
	p.apod_scale = d.f_number * (180.0f * DEG2RAD_F);
	p.apod_hi = 0.25f * r360;
	p.inv_sqrt_T = 1.0f / sqrtf((float)p.T);
	p.px = d.xdc_element_pitch[0];
	p.py = d.xdc_element_pitch[1];
	p.cy_forces = p.py * (float)(p.C / 2);
	p.focal = g.d_focal;
	p.sparse = g.d_sparse;
	p.rc = 1.0f / p.c;
	p.rfs = 1.0f / p.fs;
	/* distances and sample indices in [2^-100, 2^20] (below, the quotients by
	 * c and fs would be subnormal) */
	if (!division_range(p.c, 0x1p-100f, 0x1p20f, p.c_lo, p.c_hi)) return false;
	if (!division_range(p.fs, 0x1p-100f, 0x1p20f, p.fs_lo, p.fs_hi)) return false;
	p.fast_sqrt = sqrt_verified() ? 1 : 0;
	p.sqrt_lo = 0x1p-100f;
	p.sqrt_hi = 0x1p30f;
	{
		const int64_t dense = (int64_t)p.C * p.T * p.S;
		p.dense_rows = p.rf_count >= dense && dense < (1ll << 31) && p.S >= 4;
	}
	p.groups = 1;
	p.per_group = p.loop_end;
	set_das_rotation(p);
	p.rx_step = g.rx_step;
	if (p.rx_step > 1 && (p.family != DAS_HERCULES || !p.fast || p.sparse_mode)) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
	p.fs_c = (float)((double)p.fs / (double)p.c);
	p.toff_fs = (float)((double)p.toff * (double)p.fs);
	if (!g.d_tc_error) {
		if (!cuda_ok(cudaMalloc(&g.d_tc_error, sizeof(unsigned)))) return false;
		if (!cuda_ok(cudaMemset(g.d_tc_error, 0, sizeof(unsigned)))) return false;
	}
	p.wait_error = g.d_tc_error;
	p.half_table = g.das_precision == 1 && p.family == DAS_HERCULES ? 1 : 0;
	if (p.half_table) {
		if (!g.d_absmax && !cuda_ok(cudaMalloc(&g.d_absmax, sizeof(unsigned)))) return false;
		p.absmax = g.d_absmax;
	}
	return true;
}

/* Receive channels per block group of the HERCULES launch. The launch is tiles x
 * groups blocks on SMs x blocks-per-SM slots (the occupancy of the kernel that
 * runs). The group count minimises, as fractions of the launch:
 *   - the slots a part-full last wave leaves idle, (waves - w) / waves;
 *   - the uneven end of the blocks' durations, about half a wave: 0.5 / waves;
 *   - per group and voxel, the partial sum written and reduced and the voxel's
 *     set-up, about 12 terms' worth each: 12 G / terms per voxel.
 * Measured on one GB300: 8 groups for the 128 x 128 x 256 cubic volume (0.7 %
 * faster than 2, which only removes the part-full wave), 64 for a 128 x 128 plane
 * (2-7 % faster than 19). */
int32_t hercules_per_group(const DasParams &p)
{
	const int sms = device_sm_count();
	const double slots = (double)sms * das_hercules_blocks_per_sm(p);
	const int64_t tiles = das_hercules_tiles(p);
	const double terms = (double)p.T * p.loop_end / (p.rx_step > 0 ? p.rx_step : 1);
	double best = 1e30;
	int32_t best_per = p.loop_end;
	for (int g = 1; g <= p.loop_end && g <= 64; g++) {
		int32_t per = (p.loop_end + g - 1) / g;
		per = (per + p.rx_step - 1) / p.rx_step * p.rx_step;
		const int32_t G = (p.loop_end + per - 1) / per;
		const double w = (double)tiles * G / slots, waves = std::ceil(w);
		const double cost = (waves - w) / waves + 0.5 / waves + (G > 1 ? G * 12.0 / (terms > 1 ? terms : 1) : 0.0);
		if (cost < best - 1e-9) {
			best = cost;
			best_per = per;
		}
	}
	return best_per;
}

/* NVTX range names per shader kind (enum order of beamformer_parameters.h:14-41):
 * host ranges around each stage's launches and around a whole compute, which a
 * profiler lines up with the stage's kernels */
const char *stage_label(int kind)
{
	static const char *names[BeamformerShaderKind_Count] = {
		"CudaDecode", "CudaHilbert", "DAS", "Decode", "Filter", "Demodulate", "MinMax", "Sum",
		"DecodeInt16Complex", "DecodeFloat", "DecodeFloatComplex", "DecodeInt16ToFloat", "DemodulateFloat",
		"DASFast", "Render3D"};
	return kind >= 0 && kind < BeamformerShaderKind_Count ? names[kind] : "stage";
}

bool run_stage(int i, const void *src, uint64_t src_bytes, DeviceFrame &frame, bool &did_sum, int &sum_target)
{
	const Plan &pl = g.plan;
	const int kind = pl.shaders[i];
	const int out_idx = g.last_chan < 0 ? 0 : 1 - g.last_chan;
	const int in_idx = g.last_chan < 0 ? 0 : g.last_chan;
	cudaError_t err = cudaSuccess;

	switch (kind) {
	case BeamformerShaderKind_CudaDecode:
	case BeamformerShaderKind_Decode:
	case BeamformerShaderKind_DecodeInt16Complex:
	case BeamformerShaderKind_DecodeFloat:
	case BeamformerShaderKind_DecodeFloatComplex:
	case BeamformerShaderKind_DecodeInt16ToFloat: {
		DecodeParams p{};
		fill_decode_params(pl, i, src, src_bytes, g.chan[in_idx], g.chan[out_idx], g.chan_bytes, g.hadamard,
		                   g.hadamard_sylvester, g.hadamard_base, p);
		if (g.tc_active && i == 0) {
			p.output = g.precision == 2 ? DEC_OUT_REAL_BF16 : DEC_OUT_REAL_F16;
			p.samples = 2 * std::min(pl.decode_st.out_transmit, pl.decode_invocations_x);
		}
		err = launch_decode(p, g.stream);
		g.last_chan = out_idx;
	} break;
	case BeamformerShaderKind_Demodulate:
	case BeamformerShaderKind_DemodulateFloat:
	case BeamformerShaderKind_Filter: {
		if (g.tc_active && i == 1) {
			const Strides &ds = pl.decode_st;
			const uint32_t rows = pl.das.dec_data_dim[1] * pl.das.dec_data_dim[2];
			const uint32_t valid = 2 * std::min(ds.out_transmit, pl.decode_invocations_x);
			const uint32_t L = (uint32_t)g.taps[pl.slots[i] % BEAMFORMER_FILTER_SLOTS].size();
			err = launch_fir_tc(g.chan[in_idx], rows, 2 * ds.out_transmit, valid, pl.demod_decimation, L,
			                    pl.demod_st.out_transmit, g.precision == 2, g.tc_table, (float2 *)g.chan[out_idx],
			                    g.d_tc_error, g.stream);
			g.last_chan = out_idx;
			break;
		}
		FilterParams p{};
		fill_filter_params(pl, i, src, src_bytes, g.chan[in_idx], g.chan[out_idx], g.chan_bytes, g.stage_tables[i], p);
		err = launch_filter(p, g.stream);
		g.last_chan = out_idx;
	} break;
	case BeamformerShaderKind_CudaHilbert: {
		/* cuda_hilbert(input, output) (beamformer.c:567-570): rows in the DAS layout */
		const int64_t rows = (int64_t)pl.das.dec_data_dim[1] * pl.das.dec_data_dim[2];
		err = launch_analytic(g.chan[in_idx], g.chan[out_idx], rows, pl.das.dec_data_dim[0], g.d_hilbert_tw, g.stream);
		g.last_chan = out_idx;
	} break;
	case BeamformerShaderKind_DAS:
	case BeamformerShaderKind_DASFast: {
		DasParams p{};
		if (!fill_das_params(pl, kind, g.chan[in_idx], g.chan_bytes, frame.data, frame.dims, g.M, p)) return false;
		/* small volumes: split the outer loop over block groups so the grid fills the GPU */
		p.groups = 1;
		p.per_group = p.loop_end;
		const int64_t nv = (int64_t)frame.dims[0] * frame.dims[1] * frame.dims[2];
		const int64_t vblocks = (int64_t)((frame.dims[0] + 7) / 8) * frame.dims[1] * ((frame.dims[2] + 15) / 16);
		const char *generic_env = std::getenv("OGL_BF_DAS_GENERIC");
		if (das_hercules_supported(p) && !(generic_env && generic_env[0] == '1') && p.loop_end > 1) {
			p.per_group = hercules_per_group(p);
			p.groups = (p.loop_end + p.per_group - 1) / p.per_group;
		} else if (p.fast && p.loop_end > 1 && vblocks < 2048) {
			int64_t want = (2048 + vblocks - 1) / vblocks;
			if (want > p.loop_end) want = p.loop_end;
			p.per_group = (int32_t)((p.loop_end + want - 1) / want);
			p.per_group = (p.per_group + p.rx_step - 1) / p.rx_step * p.rx_step;   /* groups start on kept channels */
			p.groups = (p.loop_end + p.per_group - 1) / p.per_group;
		}
		if (p.groups > 1) {
			const uint64_t need = (uint64_t)p.groups * (uint64_t)nv * sizeof(float2);
			if (need > g.das_partial_bytes) {
				cudaStreamSynchronize(g.stream);
				cudaFree(g.das_partial);
				g.das_partial = nullptr;
				g.das_partial_bytes = 0;
				if (!cuda_ok(cudaMalloc(&g.das_partial, need))) return false;
				g.das_partial_bytes = need;
			}
			p.partial = g.das_partial;
		}
		/* OGL_BF_DAS_GENERIC=1 keeps every DAS on das_kernel (for comparisons) */
		const char *generic = std::getenv("OGL_BF_DAS_GENERIC");
		const bool herc = das_hercules_supported(p), forces = das_forces_supported(p);
		if ((herc || forces) && !(generic && generic[0] == '1')) {
			const uint64_t need = (uint64_t)das_hercules_table_bytes(p);
			if (need > g.das_table_bytes) {
				cudaStreamSynchronize(g.stream);
				cudaFree(g.das_table);
				g.das_table = nullptr;
				g.das_table_bytes = 0;
				if (!cuda_ok(cudaMalloc(&g.das_table, need))) return false;
				g.das_table_bytes = need;
			}
			err = herc ? launch_das_hercules(p, g.das_table, g.stream) : launch_das_forces(p, g.das_table, g.stream);
		} else {
			err = launch_das(p, g.stream);
		}
		frame.written = true;
	} break;
	case BeamformerShaderKind_Sum: {
		int32_t n = pl.das.output_points[3];
		if (n < 0) n = 0;
		if (n > MAX_BEAMFORMED_SAVED_FRAMES) n = MAX_BEAMFORMED_SAVED_FRAMES;
		const uint32_t base = g.frame_counter % MAX_BEAMFORMED_SAVED_FRAMES;
		const float2 *ins[MAX_BEAMFORMED_SAVED_FRAMES] = {};
		for (int32_t k = 0; k < n; k++) {
			uint32_t idx = (base + MAX_BEAMFORMED_SAVED_FRAMES + 1 - (uint32_t)n + (uint32_t)k) % MAX_BEAMFORMED_SAVED_FRAMES;
			DeviceFrame &f = g.frames[idx];
			bool same = f.data && f.written && f.dims[0] == frame.dims[0] && f.dims[1] == frame.dims[1] &&
			            f.dims[2] == frame.dims[2];
			ins[k] = same ? f.data : nullptr;
		}
		const int ai = (int)(g.averaged_counter % 2);
		DeviceFrame &af = g.averaged[ai];
		if (!ensure_frame(af, frame.dims)) return false;
		err = launch_sum(af.data, ins, n, 1.0f / (float)n, frame.dims, g.stream);
		af.written = true;
		did_sum = true;
		sum_target = ai;
	} break;
	case BeamformerShaderKind_MinMax:
		if (frame.mips > 1) err = launch_min_max(frame.data, frame.dims, frame.mips, frame.levels, g.stream);
		break;
	default:
		return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
	}
	return cuda_ok(err);
}

/* Device-resident inputs and outputs (push_data_device, beamform_batch): the
 * library's streams do not synchronise implicitly with the legacy default
 * stream, so the compute first waits for the work the caller queued there before
 * the call (the kernels or copies that wrote its input, a clear of its output).
 * Work on other streams of the caller is ordered by set_stream. Skipped while the
 * compute stream is being captured into a graph, where the caller orders the graph. */
bool order_after_caller()
{
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	if (!cuda_ok(cudaStreamIsCapturing(g.stream, &cs))) return false;
	if (cs != cudaStreamCaptureStatusNone) return true;
	if (!cuda_ok(cudaEventRecord(g.caller_ready, cudaStreamLegacy))) return false;
	return cuda_ok(cudaStreamWaitEvent(g.stream, g.caller_ready, 0));
}

uint32_t compute_base()
{
	if (!ensure_cuda()) return 0;
	if (!g.use_ext && g.latest_slot < 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (g.shader_count == 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!prepare()) return 0;

	const void *src;
	uint64_t src_bytes;
	int slot = -1;
	if (g.use_ext) {
		src = g.ext_rf;
		src_bytes = g.ext_size;
		if (!order_after_caller()) return 0;
	} else {
		slot = g.latest_slot;
		src = g.raw[slot];
		src_bytes = g.raw_size[slot];
		if (!cuda_ok(cudaStreamWaitEvent(g.stream, g.upload_done[slot], 0))) return 0;
	}

	int32_t dims[3];
	for (int i = 0; i < 3; i++) dims[i] = g.params.output_points[i] > 1 ? g.params.output_points[i] : 1;
	const int fi = (int)(g.frame_counter % MAX_BEAMFORMED_SAVED_FRAMES);
	DeviceFrame &frame = g.frames[fi];
	if (!ensure_frame(frame, dims)) return 0;

	collect_timings(false);
	PendingTiming &tm = g.timing[g.timing_next % TIMING_SLOTS];
	if (tm.active) collect_timings(true);
	g.timing_next++;
	tm.count = g.plan.count;
	cudaEventRecord(tm.ev[0], g.stream);

	g.last_chan = -1;
	bool did_sum = false;
	int sum_target = -1;
	nvtxRangePushA("beamformer compute");
	for (int i = 0; i < g.plan.count; i++) {
		nvtxRangePushA(stage_label(g.plan.shaders[i]));
		const bool ok = run_stage(i, src, src_bytes, frame, did_sum, sum_target);
		nvtxRangePop();
		if (!ok) {
			nvtxRangePop();
			return 0;
		}
		tm.shaders[i] = g.plan.shaders[i];
		cudaEventRecord(tm.ev[i + 1], g.stream);
	}
	nvtxRangePop();
	tm.active = true;

	cudaEvent_t done = g.use_ext ? g.ext_done : g.compute_done[slot];
	if (!cuda_ok(cudaEventRecord(done, g.stream))) return 0;
	if (slot >= 0) g.slot_used[slot] = true;
	g.last_done = done;

	g.latest_das_index = fi;
	if (did_sum) {
		g.latest_kind = 1;
		g.latest_index = sum_target;
		g.averaged_counter++;
	} else {
		g.latest_kind = 0;
		g.latest_index = fi;
	}
	g.frame_counter++;
	return 1;
}

uint32_t compute_indirect(uint32_t tag)
{
	if (tag >= BeamformerViewPlaneTag_Count) return fail(BF_LIB_ERR_KIND_INVALID_IMAGE_PLANE);
	return compute_base();
}

DeviceFrame *latest_frame(uint32_t which)
{
	if (which == 0) return g.latest_das_index >= 0 ? &g.frames[g.latest_das_index] : nullptr;
	if (which == 1) return (g.averaged_counter > 0) ? &g.averaged[(g.averaged_counter - 1) % 2] : nullptr;
	if (g.latest_kind == 1) return &g.averaged[g.latest_index];
	if (g.latest_kind == 0) return &g.frames[g.latest_index];
	return nullptr;
}

const char *error_text(int32_t kind)
{
	/* kinds 0..13 as the reference words them (ogl_beamformer_lib_base.h:10-24) */
	static const char *table[] = {
		"None",
		"host-library version mismatch",
		"library in invalid state",
		"compute stage overflow: maximum stages: 16",
		"invalid compute shader stage",
		"starting shader not Decode or Demodulate",
		"data kind for demodulation not Int16 or Float",
		"invalid image plane",
		"passed buffer size exceeds available space",
		"work queue full",
		"not enough space for data export",
		"failed to open shared memory region",
		"failed to acquire lock within timeout period",
		"invalid timeout value",
		"no usable CUDA device",
		"CUDA runtime error",
		"unsupported pipeline configuration",
		"invalid error kind",
	};
	const int32_t n = (int32_t)(sizeof(table) / sizeof(table[0]));
	if (kind < 0 || kind >= n - 1) return table[n - 1];
	return table[kind];
}


/* ------------------------------ batched beamforming ----------------------------- */

/* One acquisition of a batch: its plan, channel buffers and tables. */
struct BatchAcqState {
	Plan        plan{};
	void       *chan[2] = {nullptr, nullptr};
	uint64_t    chan_bytes = 0;
	StageTables tables[MAX_COMPUTE_SHADER_STAGES];
	float4     *das_table = nullptr;
	unsigned   *absmax = nullptr;       /* FP16 table scale (DAS precision 1) */
	int8_t     *hadamard = nullptr;
	int32_t     sylvester = 0, base = 0;
	float       M[16] = {};
	DasParams   das{};
	int32_t     path = DAS_BATCH_GENERIC;
	const void *rf = nullptr;
	uint64_t    rf_bytes = 0;
};

/* Acquisitions [first, first + count) of a batch: one persistent DAS launch. */
struct BatchChunk {
	int                           first = 0, count = 0;
	std::unique_ptr<DasBatchArgs> args;
	int4                         *d_items[2] = {nullptr, nullptr};   /* HERCULES tiles, general-path tiles */
	size_t                        items_cap[2] = {0, 0};
	int                           n_items[2] = {0, 0};
	int                          *d_counter = nullptr;              /* two counters */
};

struct BatchState {
	uint64_t                   signature = 0;
	std::vector<BatchAcqState> acq;
	std::vector<BatchChunk>    chunks;
	int                        interp = INTERP_NEAREST;
	bool                       half = false;          /* FP16 tables (DAS precision 1) */
	int                        ctas = 0;             /* persistent CTAs of the HERCULES launch */
	int                        ctas_general = 0;     /* and of the general-path launch */
	bool                       volume_tiles = true;
	cudaGraphExec_t            exec = nullptr;
	uint64_t                   graph_kernels = 0;
	std::vector<float>         candidate_ms;          /* autotuner: (tiles, ctas) candidates in order */
};
BatchState gb;

void free_batch()
{
	if (g.ready) cudaStreamSynchronize(g.stream);
	if (gb.exec) cudaGraphExecDestroy(gb.exec);
	for (auto &a : gb.acq) {
		cudaFree(a.chan[0]);
		cudaFree(a.chan[1]);
		for (auto &t : a.tables) { cudaFree(t.taps); cudaFree(t.phasor); }
		cudaFree(a.das_table);
		cudaFree(a.absmax);
		cudaFree(a.hadamard);
	}
	for (auto &c : gb.chunks) {
		cudaFree(c.d_items[0]);
		cudaFree(c.d_items[1]);
		cudaFree(c.d_counter);
	}
	gb = BatchState();
}

uint64_t fnv1a(uint64_t h, const void *data, size_t n)
{
	const uint8_t *b = (const uint8_t *)data;
	for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
	return h;
}

uint64_t batch_signature(const BeamformerParameters *params, uint32_t count, const void *const *rf,
                         const uint64_t *rf_size, float *const *out)
{
	uint64_t h = 1469598103934665603ull;
	h = fnv1a(h, &count, sizeof(count));
	h = fnv1a(h, params, sizeof(BeamformerParameters) * count);
	h = fnv1a(h, rf, sizeof(void *) * count);
	h = fnv1a(h, rf_size, sizeof(uint64_t) * count);
	h = fnv1a(h, out, sizeof(float *) * count);
	h = fnv1a(h, g.shaders, sizeof(g.shaders));
	h = fnv1a(h, g.slots, sizeof(g.slots));
	h = fnv1a(h, &g.shader_count, sizeof(g.shader_count));
	h = fnv1a(h, &g.data_kind, sizeof(g.data_kind));
	for (int i = 0; i < BEAMFORMER_FILTER_SLOTS; i++) h = fnv1a(h, g.taps[i].data(), g.taps[i].size() * sizeof(float));
	h = fnv1a(h, g.channel_mapping, sizeof(g.channel_mapping));
	h = fnv1a(h, g.sparse_elements, sizeof(g.sparse_elements));
	h = fnv1a(h, g.focal_vectors, sizeof(g.focal_vectors));
	h = fnv1a(h, &g.interpolation_override, sizeof(g.interpolation_override));
	h = fnv1a(h, &g.das_precision, sizeof(g.das_precision));
	h = fnv1a(h, &g.rx_step, sizeof(g.rx_step));
	return h;
}

/* The persistent DAS launch of every chunk. */
cudaError_t batch_das(cudaStream_t s)
{
	for (auto &c : gb.chunks) {
		cudaError_t e = launch_das_batch(*c.args, c.d_items[0], c.n_items[0], c.d_counter, gb.interp, false, gb.half,
		                                 gb.ctas, s);
		if (e != cudaSuccess) return e;
		e = launch_das_batch(*c.args, c.d_items[1], c.n_items[1], c.d_counter + 1, gb.interp, true, false,
		                     gb.ctas_general, s);
		if (e != cudaSuccess) return e;
	}
	return cudaSuccess;
}

/* Front end (decode / demodulate / filter stages) of every acquisition, the
 * HERCULES interpolation tables, then the persistent DAS launch. */
cudaError_t batch_launch(cudaStream_t s)
{
	for (auto &a : gb.acq) {
		const Plan &pl = a.plan;
		int last = -1;
		for (int i = 0; i + 1 < pl.count; i++) {
			const int kind = pl.shaders[i];
			const int out_idx = last < 0 ? 0 : 1 - last, in_idx = last < 0 ? 0 : last;
			cudaError_t e = cudaSuccess;
			if (kind == BeamformerShaderKind_Demodulate || kind == BeamformerShaderKind_DemodulateFloat ||
			    kind == BeamformerShaderKind_Filter) {
				FilterParams p{};
				fill_filter_params(pl, i, a.rf, a.rf_bytes, a.chan[in_idx], a.chan[out_idx], a.chan_bytes, a.tables[i], p);
				e = launch_filter(p, s);
			} else {
				DecodeParams p{};
				fill_decode_params(pl, i, a.rf, a.rf_bytes, a.chan[in_idx], a.chan[out_idx], a.chan_bytes, a.hadamard,
				                   a.sylvester, a.base, p);
				e = launch_decode(p, s);
			}
			if (e != cudaSuccess) return e;
			last = out_idx;
		}
		if (a.das_table && das_hercules_table_bytes(a.das) > 0) {
			const cudaError_t e = launch_das_table(a.das, a.das_table, s);
			if (e != cudaSuccess) return e;
		}
	}
	return batch_das(s);
}

/* Paths and the cost-ordered work lists (one per chunk of up to DAS_BATCH_MAX
 * acquisitions) for a tile choice; uploads the lists. */
bool batch_items(bool volume_tiles)
{
	for (auto &c : gb.chunks) {
		struct Entry { double cost; int acq; };
		std::vector<Entry> order;
		for (int k = 0; k < c.count; k++) {
			BatchAcqState &a = gb.acq[(size_t)(c.first + k)];
			if (a.das.family == DAS_HERCULES)
				a.path = volume_tiles && a.das.dims[1] >= 4 ? DAS_BATCH_HERC_VOLUME : DAS_BATCH_HERC_PLANE;
			DasBatchAcq &d = c.args->acq[k];
			d.p = a.das;
			d.table = a.das_table;
			d.path = a.path;
			d.staged = a.path != DAS_BATCH_GENERIC && das_hercules_use_staged(a.das) ? 1 : 0;
			/* OGL_BF_DAS_STAGED=require (tests): a staged tile that cannot stage writes NaN */
			const char *stg_env = std::getenv("OGL_BF_DAS_STAGED");
			d.p.stage_only = d.staged && stg_env && std::strcmp(stg_env, "require") == 0;
			const double vox = a.path == DAS_BATCH_HERC_VOLUME ? 256.0 : 128.0;
			order.push_back({vox * a.das.T * a.das.C, k});
		}
		std::stable_sort(order.begin(), order.end(), [](const Entry &x, const Entry &y) { return x.cost > y.cost; });
		std::vector<int4> items[2];
		for (const Entry &e : order) {
			int tiles[3];
			const int path = c.args->acq[e.acq].path;
			das_batch_tiles(c.args->acq[e.acq].p, path, tiles);
			std::vector<int4> &list = items[path == DAS_BATCH_GENERIC ? 1 : 0];
			for (int z = 0; z < tiles[2]; z++)
				for (int y = 0; y < tiles[1]; y++)
					for (int x = 0; x < tiles[0]; x++) list.push_back(make_int4(e.acq, x, y, z));
		}
		for (int l = 0; l < 2; l++) {
			if (items[l].size() > c.items_cap[l]) {
				cudaFree(c.d_items[l]);
				c.d_items[l] = nullptr;
				if (!cuda_ok(cudaMalloc(&c.d_items[l], items[l].size() * sizeof(int4)))) return false;
				c.items_cap[l] = items[l].size();
			}
			c.n_items[l] = (int)items[l].size();
			if (c.n_items[l] && !cuda_ok(cudaMemcpy(c.d_items[l], items[l].data(), items[l].size() * sizeof(int4),
			                                         cudaMemcpyHostToDevice)))
				return false;
		}
	}
	return true;
}

/* Plans, buffers and tables of a new batch; autotunes the DAS launch (tile
 * shape of HERCULES volumes x CTAs per SM, timed on the device) and captures
 * the whole batch in a CUDA graph. */
bool build_batch(const BeamformerParameters *params, uint32_t count, const void *const *rf, const uint64_t *rf_size,
                 float *const *out)
{
	free_batch();
	if (!upload_element_tables()) return false;
	gb.acq.resize(count);
	int interp = -1;
	bool any_volume = false;
	for (uint32_t i = 0; i < count; i++) {
		BatchAcqState &a = gb.acq[i];
		plan_pipeline(params[i], g.shaders, g.slots, g.shader_count, g.data_kind, g.filters, a.plan);
		const Plan &pl = a.plan;
		if (pl.count < 1 || pl.shaders[pl.count - 1] != BeamformerShaderKind_DASFast) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
		for (int s = 0; s + 1 < pl.count; s++) {
			const int k = pl.shaders[s];
			const bool ok = k == BeamformerShaderKind_Decode || k == BeamformerShaderKind_DecodeInt16ToFloat ||
			                k == BeamformerShaderKind_DecodeInt16Complex || k == BeamformerShaderKind_DecodeFloat ||
			                k == BeamformerShaderKind_DecodeFloatComplex || k == BeamformerShaderKind_CudaDecode ||
			                k == BeamformerShaderKind_Demodulate || k == BeamformerShaderKind_DemodulateFloat ||
			                k == BeamformerShaderKind_Filter;
			if (!ok) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
			if (k == BeamformerShaderKind_Demodulate || k == BeamformerShaderKind_DemodulateFloat || k == BeamformerShaderKind_Filter) {
				const FilterSpec &f = g.filters[pl.slots[s] % BEAMFORMER_FILTER_SLOTS];
				if (f.kind < 0 || f.length <= 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS), false;
			}
		}
		a.rf = rf[i];
		a.rf_bytes = rf_size[i];
		a.chan_bytes = 8ull * params[i].dec_data_dim[0] * params[i].dec_data_dim[1] * params[i].dec_data_dim[2];
		for (int b = 0; b < 2; b++) {
			if (!cuda_ok(cudaMalloc(&a.chan[b], a.chan_bytes))) return false;
			if (!cuda_ok(cudaMemset(a.chan[b], 0, a.chan_bytes))) return false;
		}
		if (pl.decode_mode == DECODE_MODE_HADAMARD) {
			std::vector<int8_t> h;
			if (!hadamard_matrix((int32_t)params[i].dec_data_dim[2], h, a.sylvester, a.base))
				return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
			if (!cuda_ok(cudaMalloc(&a.hadamard, h.size()))) return false;
			if (!cuda_ok(cudaMemcpy(a.hadamard, h.data(), h.size(), cudaMemcpyHostToDevice))) return false;
		}
		if (!build_stage_tables(pl, a.tables)) return false;
		voxel_transform(pl.das, a.M);
		int last = -1;
		for (int s = 0; s + 1 < pl.count; s++) last = last < 0 ? 0 : 1 - last;
		int32_t dims[3];
		for (int k = 0; k < 3; k++) dims[k] = pl.das.output_points[k] > 1 ? pl.das.output_points[k] : 1;
		if (!fill_das_params(pl, BeamformerShaderKind_DASFast, a.chan[last < 0 ? 0 : last], a.chan_bytes,
		                     (float2 *)out[i], dims, a.M, a.das))
			return false;
		if (last < 0) { a.das.rf = (const float2 *)rf[i]; a.das.rf_count = (int64_t)(std::min<uint64_t>(pl.rf_size, rf_size[i]) / 8); }
		if (a.das.family == DAS_HERCULES && das_hercules_supported(a.das)) {
			a.path = DAS_BATCH_HERC_PLANE;
			any_volume = any_volume || a.das.dims[1] >= 4;
			const uint64_t n = (uint64_t)das_hercules_table_bytes(a.das);
			if (n && !cuda_ok(cudaMalloc(&a.das_table, n))) return false;
			if (a.das.half_table) {
				/* each acquisition's table has its own scale */
				if (!cuda_ok(cudaMalloc(&a.absmax, sizeof(unsigned)))) return false;
				a.das.absmax = a.absmax;
				gb.half = true;
			}
		} else if (a.das.family == DAS_FORCES && !a.das.sparse_mode) {
			a.path = DAS_BATCH_GENERIC;
			if (das_forces_supported(a.das)) {
				/* the FORCES fast path reads the same per-frame table */
				if (!cuda_ok(cudaMalloc(&a.das_table, (size_t)das_hercules_table_bytes(a.das)))) return false;
			}
		} else {
			return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
		}
		if (interp >= 0 && a.das.interp != interp) return fail(BF_LIB_ERR_KIND_UNSUPPORTED), false;
		interp = a.das.interp;
	}
	gb.interp = interp;
	for (uint32_t first = 0; first < count; first += DAS_BATCH_MAX) {
		BatchChunk c;
		c.first = (int)first;
		c.count = (int)std::min<uint32_t>(count - first, DAS_BATCH_MAX);
		c.args.reset(new DasBatchArgs());
		if (!cuda_ok(cudaMalloc(&c.d_counter, 2 * sizeof(int)))) return false;
		gb.chunks.push_back(std::move(c));
	}

	/* autotuner: every (tile shape, CTAs per SM) candidate runs the batch once to
	 * warm up and once timed; the fastest is kept */
	const int sms = device_sm_count();
	const bool tile_choices[2] = {true, false};
	const int cta_choices[3] = {4, 5, 6};
	gb.ctas_general = 8 * sms;
	float best = INFINITY;
	bool best_tiles = true;
	int best_ctas = 6 * sms;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	for (int ti = 0; ti < (any_volume ? 2 : 1); ti++) {
		if (!batch_items(tile_choices[ti])) return false;
		for (int ci = 0; ci < 3; ci++) {
			gb.ctas = cta_choices[ci] * sms;
			if (!cuda_ok(batch_launch(g.stream))) return false;
			cudaEventRecord(e0, g.stream);
			if (!cuda_ok(batch_das(g.stream))) return false;
			cudaEventRecord(e1, g.stream);
			if (!cuda_ok(cudaEventSynchronize(e1))) return false;
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			gb.candidate_ms.push_back(ms);
			if (ms < best) { best = ms; best_tiles = tile_choices[ti]; best_ctas = gb.ctas; }
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	gb.volume_tiles = best_tiles;
	gb.ctas = best_ctas;
	if (!batch_items(best_tiles)) return false;

	/* the whole batch as one graph */
	cudaGraph_t graph = nullptr;
	const uint64_t k0 = g_kernel_launches;
	if (!cuda_ok(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal))) return false;
	const cudaError_t le = batch_launch(g.stream);
	const cudaError_t ce = cudaStreamEndCapture(g.stream, &graph);
	if (!cuda_ok(le) || !cuda_ok(ce)) return false;
	gb.graph_kernels = g_kernel_launches - k0;
	g_kernel_launches = k0;
	const cudaError_t ie = cudaGraphInstantiate(&gb.exec, graph, 0);
	cudaGraphDestroy(graph);
	if (!cuda_ok(ie)) return false;
	gb.signature = batch_signature(params, count, rf, rf_size, out);
	return true;
}

} /* namespace */

extern "C" {

LIB_FN uint32_t beamformer_get_api_version(void) { return BEAMFORMER_SHARED_MEMORY_VERSION; }

LIB_FN BeamformerLibErrorKind beamformer_get_last_error(void) { return g.last_error; }

LIB_FN const char *beamformer_error_string(BeamformerLibErrorKind kind) { return error_text((int32_t)kind); }

LIB_FN const char *beamformer_get_last_error_string(void) { return error_text((int32_t)g.last_error); }

LIB_FN uint32_t beamformer_set_global_timeout(int32_t timeout_ms)
{
	if (timeout_ms < -1) return fail(BF_LIB_ERR_KIND_INVALID_TIMEOUT);
	g.timeout_ms = timeout_ms;
	return 1;
}

LIB_FN uint32_t beamformer_push_pipeline(int32_t *shaders, int32_t shader_count, BeamformerDataKind data_kind)
{
	/* validate_pipeline (ogl_beamformer_lib.c:166-190) */
	if (shader_count > MAX_COMPUTE_SHADER_STAGES) return fail(BF_LIB_ERR_KIND_COMPUTE_STAGE_OVERFLOW);
	if (shader_count < 1 || !shaders) return fail(BF_LIB_ERR_KIND_INVALID_START_SHADER);
	for (int32_t i = 0; i < shader_count; i++)
		if (shaders[i] < 0 || shaders[i] > BeamformerShaderKind_ComputeCount)
			return fail(BF_LIB_ERR_KIND_INVALID_COMPUTE_STAGE);
	if (shaders[0] != BeamformerShaderKind_Demodulate && shaders[0] != BeamformerShaderKind_Decode)
		return fail(BF_LIB_ERR_KIND_INVALID_START_SHADER);
	if (shaders[0] == BeamformerShaderKind_Demodulate &&
	    !(data_kind == BeamformerDataKind_Int16 || data_kind == BeamformerDataKind_Float32))
		return fail(BF_LIB_ERR_KIND_INVALID_DEMOD_DATA_KIND);
	g.shader_count = shader_count;
	g.data_kind = (int32_t)data_kind;
	for (int32_t i = 0; i < shader_count; i++) g.shaders[i] = shaders[i];
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_set_pipeline_stage_parameters(int32_t stage_index, int32_t parameter)
{
	if (g.shader_count == 0) return 0;
	int32_t s = stage_index % MAX_COMPUTE_SHADER_STAGES;
	if (s < 0) s += MAX_COMPUTE_SHADER_STAGES;
	g.slots[s] = (uint8_t)parameter;
	g.dirty = true;
	return 1;
}

static uint32_t create_filter(int32_t kind, float p0, float p1, float fs, int16_t length, uint8_t slot)
{
	if (length < 1 || !(fs > 0)) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	const int s = slot % BEAMFORMER_FILTER_SLOTS;
	FilterSpec &f = g.filters[s];
	f.kind = kind; f.length = length; f.sampling_frequency = fs; f.param0 = p0; f.param1 = p1;
	g.taps[s].assign((size_t)length, 0.0f);
	if (kind == BeamformerFilterKind_Kaiser) kaiser_low_pass(p1, fs, p0, length, g.taps[s].data());
	else                                      matched_filter(p0, p1, fs, length, g.taps[s].data());
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_create_kaiser_low_pass_filter(float beta, float cutoff_frequency, float sampling_frequency,
                                                         int16_t length, uint8_t slot)
{
	return create_filter(BeamformerFilterKind_Kaiser, beta, cutoff_frequency, sampling_frequency, length, slot);
}

LIB_FN uint32_t beamformer_create_matched_filter(float xdc_center_frequency, float transmit_frequency,
                                                 float sampling_frequency, int16_t length, uint8_t slot)
{
	return create_filter(BeamformerFilterKind_Matched, xdc_center_frequency, transmit_frequency, sampling_frequency,
	                     length, slot);
}

LIB_FN uint32_t beamformer_push_channel_mapping(int16_t *mapping, uint32_t count)
{
	if (count > 256) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	if (count && !mapping) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	std::memcpy(g.channel_mapping, mapping, count * sizeof(int16_t));
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_sparse_elements(int16_t *elements, uint32_t count)
{
	if (count > 256) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	if (count && !elements) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	std::memcpy(g.sparse_elements, elements, count * sizeof(int16_t));
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_focal_vectors(float *vectors, uint32_t count)
{
	if (count > 256) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	if (count && !vectors) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	std::memcpy(g.focal_vectors, vectors, count * 2 * sizeof(float));
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_parameters(BeamformerParameters *bp)
{
	if (!bp) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	g.params = *bp;
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_parameters_ui(BeamformerUIParameters *ui)
{
	if (!ui) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	std::memcpy((char *)&g.params + offsetof(BeamformerParameters, output_min_coordinate), ui, sizeof(*ui));
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_parameters_head(BeamformerParametersHead *head)
{
	if (!head) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	std::memcpy(&g.params, head, sizeof(*head));
	g.dirty = true;
	return 1;
}

LIB_FN uint32_t beamformer_push_data(void *data, uint32_t size)
{
	return push_data_base(data, size, g.timeout_ms);
}

LIB_FN uint32_t beamformer_push_data_with_compute(void *data, uint32_t size, uint32_t image_plane_tag)
{
	uint32_t r = push_data_base(data, size, g.timeout_ms);
	if (r) r = compute_indirect(image_plane_tag);
	return r;
}

LIB_FN uint32_t beamformer_start_compute(void) { return compute_indirect(0); }

LIB_FN uint32_t beamformer_wait_for_compute_dispatch(int32_t timeout_ms)
{
	/* compute is dispatched onto the stream by the call that requests it */
	(void)timeout_ms;
	return 1;
}

LIB_FN uint32_t beamform_data_synchronized(void *data, uint32_t data_size, int32_t output_points[3], float *out_data,
                                           int32_t timeout_ms)
{
	if (!output_points) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	for (int i = 0; i < 3; i++) {
		output_points[i] = output_points[i] > 1 ? output_points[i] : 1;
		if (g.params.output_points[i] != output_points[i]) {
			g.params.output_points[i] = output_points[i];
			g.dirty = true;
		}
	}
	uint64_t out_size = (uint64_t)(uint32_t)output_points[0] * (uint32_t)output_points[1] * (uint32_t)output_points[2] *
	                    sizeof(float) * 2;
	if (out_size > SCRATCH_SIZE) return fail(BF_LIB_ERR_KIND_EXPORT_SPACE_OVERFLOW);
	if (!beamformer_push_data_with_compute(data, data_size, 0)) return 0;
	if (!wait_event(g.last_done, timeout_ms)) return fail(BF_LIB_ERR_KIND_SYNC_VARIABLE);
	DeviceFrame *f = latest_frame(2);
	if (!f || !f->data) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	uint64_t have = (uint64_t)f->dims[0] * f->dims[1] * f->dims[2] * sizeof(float2);
	if (have > out_size) return fail(BF_LIB_ERR_KIND_EXPORT_SPACE_OVERFLOW);
	if (!out_data) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!cuda_ok(cudaMemcpyAsync(out_data, f->data, have, cudaMemcpyDeviceToHost, g.stream))) return 0;
	if (!cuda_ok(cudaStreamSynchronize(g.stream))) return 0;
	return 1;
}

LIB_FN uint32_t beamformer_compute_timings(BeamformerComputeStatsTable *output, int32_t timeout_ms)
{
	if (!output) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (g.ready) {
		if (g.last_done && !wait_event(g.last_done, timeout_ms)) return fail(BF_LIB_ERR_KIND_SYNC_VARIABLE);
		collect_timings(false);
	}
	*output = g.stats;
	return 1;
}

LIB_FN int32_t beamformer_live_parameters_get_dirty_flag(void)
{
	if (!g.live_dirty) return -1;
	int32_t flag = __builtin_ctz(g.live_dirty);
	g.live_dirty &= ~(1u << flag);
	return flag;
}

LIB_FN uint32_t beamformer_set_live_parameters(BeamformerLiveImagingParameters *lp)
{
	if (!lp) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	g.live = *lp;
	return 1;
}

LIB_FN BeamformerLiveImagingParameters *beamformer_get_live_parameters(void) { return &g.live; }

/* ------------------------------- extensions ------------------------------ */

LIB_FN uint32_t beamformer_gb300_push_data_device(const void *device_data, uint64_t size)
{
	if (size > BEAMFORMER_MAX_RF_DATA_SIZE) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	if (!device_data && size) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!ensure_cuda()) return 0;
	g.ext_rf = device_data;
	g.ext_size = size;
	g.use_ext = true;
	note_upload();
	return 1;
}

LIB_FN uint32_t beamformer_gb300_set_stream(void *cuda_stream)
{
	if (!ensure_cuda()) return 0;
	g.stream = cuda_stream ? (cudaStream_t)cuda_stream : g.own_stream;
	return 1;
}

LIB_FN void *beamformer_gb300_get_stream(void)
{
	if (!ensure_cuda()) return nullptr;
	return (void *)g.stream;
}

LIB_FN uint32_t beamformer_gb300_synchronize(int32_t timeout_ms)
{
	if (!g.ready) return 1;
	if (!wait_event(g.last_done, timeout_ms)) return fail(BF_LIB_ERR_KIND_SYNC_VARIABLE);
	if (!cuda_ok(cudaStreamSynchronize(g.stream))) return 0;
	if (g.d_tc_error) {
		/* a bounded wait that ran out (tensor-core FIR, staged DAS: the kernel stopped early) */
		unsigned e = 0;
		if (!cuda_ok(cudaMemcpy(&e, g.d_tc_error, sizeof(e), cudaMemcpyDeviceToHost))) return 0;
		if (e) {
			cudaMemset(g.d_tc_error, 0, sizeof(unsigned));
			return fail(BF_LIB_ERR_KIND_CUDA_RUNTIME);
		}
	}
	return 1;
}

LIB_FN uint32_t beamformer_gb300_export_frame(uint32_t which, uint32_t mip_level, float *out, uint64_t out_size,
                                              int32_t dims_out[3])
{
	if (!g.ready) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	DeviceFrame *f = latest_frame(which);
	if (!f || !f->data) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if ((int32_t)mip_level >= f->mips) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	const float2 *src = f->data;
	int32_t d[3] = {f->dims[0], f->dims[1], f->dims[2]};
	if (mip_level > 0) {
		src = f->levels;
		for (uint32_t l = 1; l <= mip_level; l++) {
			int32_t x = f->dims[0] >> l, y = f->dims[1] >> l, z = f->dims[2] >> l;
			x = x ? x : 1; y = y ? y : 1; z = z ? z : 1;
			if (l < mip_level) src += (uint64_t)x * y * z;
			d[0] = x; d[1] = y; d[2] = z;
		}
	}
	if (dims_out) std::memcpy(dims_out, d, sizeof(d));
	uint64_t bytes = (uint64_t)d[0] * d[1] * d[2] * sizeof(float2);
	if (!out) return 1;
	if (bytes > out_size) return fail(BF_LIB_ERR_KIND_EXPORT_SPACE_OVERFLOW);
	if (!cuda_ok(cudaStreamSynchronize(g.stream))) return 0;
	return cuda_ok(cudaMemcpy(out, src, bytes, cudaMemcpyDefault)) ? 1 : 0;    /* host or device out */
}

LIB_FN uint32_t beamformer_gb300_export_channel_data(void *out, uint64_t out_size, uint64_t *size_out)
{
	if (!g.ready || g.last_chan < 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (size_out) *size_out = g.chan_used;
	if (!out) return 1;
	if (g.chan_used > out_size) return fail(BF_LIB_ERR_KIND_EXPORT_SPACE_OVERFLOW);
	if (!cuda_ok(cudaStreamSynchronize(g.stream))) return 0;
	return cuda_ok(cudaMemcpy(out, g.chan[g.last_chan], g.chan_used, cudaMemcpyDeviceToHost)) ? 1 : 0;
}

LIB_FN uint32_t beamformer_gb300_get_filter(uint8_t slot, float *taps, int32_t capacity, int32_t *length_out)
{
	const int s = slot % BEAMFORMER_FILTER_SLOTS;
	const int32_t n = (int32_t)g.taps[s].size();
	if (length_out) *length_out = n;
	if (!taps) return 1;
	if (capacity < n) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	std::memcpy(taps, g.taps[s].data(), (size_t)n * sizeof(float));
	return 1;
}

LIB_FN uint32_t beamformer_gb300_set_receive_subsampling(int32_t step)
{
	if (step < 1 || step > 256) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	g.rx_step = step;
	return 1;
}

LIB_FN uint32_t beamformer_gb300_set_filter_precision(int32_t precision)
{
	if (precision < 0 || precision > 2) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	if (precision != g.precision) {
		g.precision = precision;
		g.dirty = true;
	}
	return 1;
}

LIB_FN uint32_t beamformer_gb300_set_das_precision(int32_t precision)
{
	if (precision < 0 || precision > 1) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	if (precision != g.das_precision) {
		g.das_precision = precision;
		g.dirty = true;
	}
	return 1;
}

LIB_FN uint32_t beamformer_gb300_set_interpolation(int32_t mode)
{
	if (mode < -1 || mode > 2) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	g.interpolation_override = mode;
	return 1;
}

/* See include/ogl_beamformer_lib.h. Allocates nothing: no cudaMalloc, no
 * cudaFree, no allocating library call; the partial sums and the focal/sparse
 * tables live in static device arrays of bf_das.cu. Divisions and square roots
 * take the IEEE path, which the allocated path's faster forms equal bit for bit.
 * The call is self-contained: das_parameters->interpolate selects nearest or
 * cubic, every receive channel is summed, and the library-wide settings of
 * set_interpolation, set_receive_subsampling and set_das_precision do not apply. */
LIB_FN uint32_t beamformer_gb300_das_no_alloc(const BeamformerParameters *das_parameters, const float *focal_vectors,
                                              const int16_t *sparse_elements, const void *channel_data,
                                              uint64_t channel_data_bytes, float *frame, void *cuda_stream)
{
	if (!das_parameters || !channel_data || !frame) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		return fail(BF_LIB_ERR_KIND_CUDA_DEVICE);
	}
	const BeamformerParameters &d = *das_parameters;
	DasParams p{};
	for (int i = 0; i < 3; i++) p.dims[i] = d.output_points[i] > 1 ? d.output_points[i] : 1;
	p.S = (int32_t)d.dec_data_dim[0];
	p.C = (int32_t)d.dec_data_dim[1];
	p.T = (int32_t)d.dec_data_dim[2];
	const int64_t dense = (int64_t)p.C * p.T * p.S;
	const int64_t have = (int64_t)(channel_data_bytes / sizeof(float2));
	p.rf = (const float2 *)channel_data;
	p.rf_count = have < dense ? have : dense;
	p.frame = (float2 *)frame;
	voxel_transform(d, p.M);
	std::memcpy(p.X, d.xdc_transform, sizeof(p.X));
	p.das_id = (int32_t)d.das_shader_id;
	switch (d.das_shader_id) {
	case DASShaderKind_FORCES: case DASShaderKind_UFORCES:       p.family = DAS_FORCES; break;
	case DASShaderKind_HERCULES: case DASShaderKind_UHERCULES:   p.family = DAS_HERCULES; break;
	case DASShaderKind_RCA_VLS: case DASShaderKind_RCA_TPW:
	case DASShaderKind_FLASH:                                     p.family = DAS_RCA; break;
	default:                                                      p.family = DAS_NONE; break;
	}
	p.sparse_mode = d.das_shader_id == DASShaderKind_UFORCES || d.das_shader_id == DASShaderKind_UHERCULES;
	p.fast = !d.coherency_weighting;
	p.coherency = d.coherency_weighting != 0;
	p.interp = d.interpolate ? INTERP_CUBIC : INTERP_NEAREST;
	p.tx_rows = !((d.transmit_mode & 2) != 0);
	p.rx_cols = (d.transmit_mode & 1) != 0;
	p.rx_rows = !p.rx_cols;
	p.loop_end = (d.das_shader_id == DASShaderKind_RCA_VLS || d.das_shader_id == DASShaderKind_RCA_TPW) ? p.T : p.C;
	p.fs = d.sampling_frequency;
	p.fc = d.center_frequency;
	p.c = d.speed_of_sound;
	p.toff = d.time_offset;
	const float r360 = 360.0f * DEG2RAD_F;
	p.r360_fc = r360 * d.center_frequency;
	p.apod_scale = d.f_number * (180.0f * DEG2RAD_F);
	p.apod_hi = 0.25f * r360;
	p.inv_sqrt_T = 1.0f / sqrtf((float)p.T);
	p.px = d.xdc_element_pitch[0];
	p.py = d.xdc_element_pitch[1];
	p.cy_forces = p.py * (float)(p.C / 2);
	p.rc = 1.0f / p.c;
	p.rfs = 1.0f / p.fs;
	p.c_lo = p.fs_lo = INFINITY;
	p.c_hi = p.fs_hi = 0.0f;
	p.fast_sqrt = 0;
	p.dense_rows = p.rf_count >= dense && dense < (1ll << 31) && p.S >= 4;
	p.rx_step = 1;
	p.groups = 1;
	p.per_group = p.loop_end;
	const int64_t vblocks = (int64_t)((p.dims[0] + 7) / 8) * p.dims[1] * ((p.dims[2] + 15) / 16);
	if (p.fast && p.loop_end > 1 && vblocks < 2048) {
		int64_t want = (2048 + vblocks - 1) / vblocks;
		if (want > p.loop_end) want = p.loop_end;
		p.per_group = (int32_t)((p.loop_end + want - 1) / want);
		p.groups = (p.loop_end + p.per_group - 1) / p.per_group;
	}
	/* as many channel groups as the static partial-sum array holds (at least one:
	 * a single group writes the frame directly and needs no partial sums) */
	const int64_t nv = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	if (p.groups > 1 && (int64_t)p.groups * nv > das_no_alloc_capacity()) {
		const int64_t fit = das_no_alloc_capacity() / nv;
		if (fit <= 1) {
			p.groups = 1;
			p.per_group = p.loop_end;
		} else {
			p.per_group = (int32_t)((p.loop_end + fit - 1) / fit);
			p.groups = (p.loop_end + p.per_group - 1) / p.per_group;
		}
	}
	if (p.groups > 1 && (int64_t)p.groups * nv > das_no_alloc_capacity()) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
	float4 focal[256];
	for (int i = 0; i < 256; i++) {
		const float angle = focal_vectors ? focal_vectors[2 * i] * DEG2RAD_F : 0.0f;
		const float depth = focal_vectors ? focal_vectors[2 * i + 1] : 0.0f;
		focal[i] = make_float4(sinf(angle), cosf(angle), depth, std::isinf(depth) ? 1.0f : 0.0f);
	}
	int16_t sparse[256];
	for (int i = 0; i < 256; i++) sparse[i] = sparse_elements ? sparse_elements[i] : (int16_t)i;
	return cuda_ok(launch_das_no_alloc(p, focal, sparse, (cudaStream_t)cuda_stream)) ? 1 : 0;
}

LIB_FN uint32_t beamformer_gb300_measure_shared_bandwidth(double *bytes_per_second)
{
	if (!bytes_per_second) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!ensure_cuda()) return 0;
	return cuda_ok(measure_shared_bandwidth(bytes_per_second, g.stream)) ? 1 : 0;
}

LIB_FN uint64_t beamformer_gb300_kernel_launch_count(void) { return g_kernel_launches; }

LIB_FN void beamformer_gb300_shutdown(void)
{
	das_no_alloc_forget_devices();
	if (!g.ready) return;
	cudaDeviceSynchronize();
	free_batch();
	for (auto &f : g.frames) free_frame(f);
	for (auto &f : g.averaged) free_frame(f);
	for (int i = 0; i < RF_SLOTS; i++) {
		cudaFree(g.raw[i]);
		cudaEventDestroy(g.upload_done[i]);
		cudaEventDestroy(g.compute_done[i]);
	}
	cudaEventDestroy(g.ext_done);
	cudaEventDestroy(g.caller_ready);
	for (auto &t : g.timing)
		for (auto &e : t.ev) cudaEventDestroy(e);
	cudaFree(g.chan[0]); cudaFree(g.chan[1]);
	cudaFree(g.hadamard);
	cudaFree(g.das_partial);
	cudaFree(g.das_table);
	cudaFree(g.d_absmax);
	cudaFree(g.tc_table);
	cudaFree(g.d_tc_error);
	cudaFree(g.d_mismatch);
	cudaFree(g.d_chmap); cudaFree(g.d_sparse); cudaFree(g.d_focal);
	cudaFree(g.d_hilbert_tw);
	for (auto &st : g.stage_tables) { cudaFree(st.taps); cudaFree(st.phasor); }
	cudaStreamDestroy(g.own_stream);
	cudaStreamDestroy(g.upload_stream);
	/* keep what the caller pushed; drop every device object */
	Context fresh;
	fresh.params = g.params;
	std::memcpy(fresh.shaders, g.shaders, sizeof(g.shaders));
	std::memcpy(fresh.slots, g.slots, sizeof(g.slots));
	fresh.shader_count = g.shader_count;
	fresh.data_kind = g.data_kind;
	std::memcpy(fresh.channel_mapping, g.channel_mapping, sizeof(g.channel_mapping));
	std::memcpy(fresh.sparse_elements, g.sparse_elements, sizeof(g.sparse_elements));
	std::memcpy(fresh.focal_vectors, g.focal_vectors, sizeof(g.focal_vectors));
	for (int i = 0; i < BEAMFORMER_FILTER_SLOTS; i++) { fresh.filters[i] = g.filters[i]; fresh.taps[i] = g.taps[i]; }
	fresh.timeout_ms = g.timeout_ms;
	fresh.interpolation_override = g.interpolation_override;
	fresh.precision = g.precision;
	fresh.das_precision = g.das_precision;
	fresh.rx_step = g.rx_step;
	g = fresh;
}


LIB_FN uint32_t beamformer_gb300_beamform_batch(const BeamformerParameters *parameters, uint32_t count,
                                                const void *const *rf, const uint64_t *rf_size, float *const *out,
                                                int32_t timeout_ms)
{
	if (!parameters || !rf || !rf_size || !out || count == 0) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (g.shader_count <= 0) return fail(BF_LIB_ERR_KIND_INVALID_COMPUTE_STAGE);
	if (g.precision != 0) return fail(BF_LIB_ERR_KIND_UNSUPPORTED);
	for (uint32_t i = 0; i < count; i++)
		if (!rf[i] || !out[i]) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (!ensure_cuda()) return 0;
	if (gb.signature != batch_signature(parameters, count, rf, rf_size, out) || !gb.exec) {
		if (!build_batch(parameters, count, rf, rf_size, out)) {
			free_batch();
			return 0;
		}
	}
	if (!order_after_caller()) return 0;
	if (!cuda_ok(cudaGraphLaunch(gb.exec, g.stream))) return 0;
	g_kernel_launches += gb.graph_kernels;
	if (!cuda_ok(cudaEventRecord(g.ext_done, g.stream))) return 0;
	g.last_done = g.ext_done;
	if (!wait_event(g.ext_done, timeout_ms)) return fail(BF_LIB_ERR_KIND_SYNC_VARIABLE);
	return 1;
}

LIB_FN uint32_t beamformer_gb300_batch_tuning(int32_t *volume_tiles, int32_t *ctas, float *candidate_ms,
                                              int32_t capacity, int32_t *count_out)
{
	if (!gb.exec) return fail(BF_LIB_ERR_KIND_INVALID_ACCESS);
	if (volume_tiles) *volume_tiles = gb.volume_tiles ? 1 : 0;
	if (ctas) *ctas = gb.ctas;
	const int32_t n = (int32_t)gb.candidate_ms.size();
	if (count_out) *count_out = n;
	if (candidate_ms) {
		if (capacity < n) return fail(BF_LIB_ERR_KIND_BUFFER_OVERFLOW);
		std::memcpy(candidate_ms, gb.candidate_ms.data(), (size_t)n * sizeof(float));
	}
	return 1;
}

} /* extern "C" */
