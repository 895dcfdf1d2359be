/*
 * bf_server.cpp -- ogl_beamformer_server: a headless server for the reference's
 * shared-memory client protocol, computing on the GB300 through this library.
 *
 * Unmodified clients of the reference's client library (helpers/ogl_beamformer_lib.c:
 * MATLAB, tests/throughput.c, tests/decode.c) talk to a running `ogl` process
 * through a 2 GB POSIX shared-memory region (os_linux.c:42-60, name
 * "/ogl_beamformer_shared_memory") holding BeamformerSharedMemory
 * (beamformer_work_queue.h:117-160, version 11): parameters, pipeline, tables, a
 * work queue of 64 entries and a scratch area for RF data and exports, guarded by
 * futex locks (os_linux.c:158-197). This server creates that region and serves it
 * the way beamformer.c does (complete_queue :842-1111, beamformer_rf_upload
 * :1230-1276):
 *   - RF upload: when a client holds the UploadRF lock, take ScratchSpace, copy
 *     scratch_rf_size bytes to the device (beamformer_push_data), release
 *     ScratchSpace and UploadRF;
 *   - UploadBuffer: channel mapping / focal vectors / sparse elements to the
 *     library under the region's lock, region marked clean;
 *   - CreateFilter: Kaiser or matched filter into the slot;
 *   - Compute / ComputeIndirect: parameters and pipeline taken when their regions
 *     are dirty, DispatchCompute released, the pipeline run on the latest RF;
 *   - ExportBuffer: DispatchCompute released, ScratchSpace taken, the latest frame
 *     (the averaged one after a Sum stage) or the timing table copied into the
 *     scratch area, ScratchSpace and ExportSync released;
 *   - ReloadShader: nothing to reload; committed.
 * The layout below is restated field by field with its offsets checked at
 * compile time; the locks follow the reference's protocol (a lock word is taken
 * by compare-and-swap 0 -> 1 and waited on with FUTEX_WAIT; release stores 0 and
 * wakes every waiter).
 *
 * beamformer_gb300_serve() runs the server loop in the calling thread; the
 * ogl_beamformer_server executable (bf_server_main.cpp) wraps it.
 */
#include "ogl_beamformer_lib.h"

#include <atomic>
#include <cerrno>
#include <chrono>
#include <csignal>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>

#include <fcntl.h>
#include <linux/futex.h>
#include <sys/mman.h>
#include <sys/syscall.h>
#include <sys/stat.h>
#include <unistd.h>

namespace {

constexpr const char *SHM_NAME = "/ogl_beamformer_shared_memory";
constexpr uint64_t SHM_SIZE = 2ull << 30;
constexpr uint64_t SCRATCH_OFF = 8192;                /* sizeof(header) rounded up to 4096 */
constexpr uint64_t SCRATCH_SIZE = SHM_SIZE - SCRATCH_OFF;

enum Lock : int32_t {
	LockNone, LockComputePipeline, LockChannelMapping, LockFocalVectors, LockParameters, LockScratchSpace,
	LockSparseElements, LockUploadRF, LockExportSync, LockDispatchCompute, LockCount
};
enum WorkKind : int32_t { WorkCompute, WorkComputeIndirect, WorkCreateFilter, WorkReloadShader, WorkExportBuffer,
                          WorkUploadBuffer };
enum UploadKind : int32_t { UploadChannelMapping, UploadFocalVectors, UploadSparseElements };
enum ExportKind : int32_t { ExportBeamformedData, ExportStats };

struct CreateFilterContext {
	int32_t kind;
	float   p0, p1;                 /* kaiser: beta, cutoff; matched: xdc centre, tx frequency */
	float   sampling_frequency;
	int32_t length;
	int32_t slot;
};
struct UploadContext { int32_t kind; uint32_t size; int32_t shared_memory_offset; };
struct ExportContext { int32_t kind; uint32_t size; };

struct Work {
	int32_t kind;
	int32_t lock;
	union {
		uint64_t            generic;
		CreateFilterContext create_filter;
		UploadContext       upload;
		ExportContext       export_context;
		int32_t             plane;
	};
};

struct Queue {
	std::atomic<uint64_t> queue;    /* low 32 bits: write index, high: read index */
	Work                  items[64];
};

struct SharedMemory {
	uint32_t version;
	uint32_t invalid;
	int32_t  locks[LockCount];
	uint32_t dirty_regions;
	uint8_t  pad0[64 - 52];
	float    focal_vectors[256][2];
	int16_t  channel_mapping[256];
	int16_t  sparse_elements[256];
	BeamformerParameters parameters;
	int32_t  shaders[16];
	uint8_t  shader_parameters[16];
	int32_t  shader_count;
	int32_t  data_kind;
	uint32_t scratch_rf_size;
	BeamformerLiveImagingParameters live_imaging_parameters;
	uint32_t live_imaging_dirty_flags;
	Queue    external_work_queue;
};
static_assert(offsetof(SharedMemory, locks) == 8, "layout");
static_assert(offsetof(SharedMemory, dirty_regions) == 48, "layout");
static_assert(offsetof(SharedMemory, focal_vectors) == 64, "layout");
static_assert(offsetof(SharedMemory, channel_mapping) == 2112, "layout");
static_assert(offsetof(SharedMemory, sparse_elements) == 2624, "layout");
static_assert(offsetof(SharedMemory, parameters) == 3136, "layout");
static_assert(offsetof(SharedMemory, shaders) == 3344, "layout");
static_assert(offsetof(SharedMemory, shader_parameters) == 3408, "layout");
static_assert(offsetof(SharedMemory, shader_count) == 3424, "layout");
static_assert(offsetof(SharedMemory, data_kind) == 3428, "layout");
static_assert(offsetof(SharedMemory, scratch_rf_size) == 3432, "layout");
static_assert(offsetof(SharedMemory, live_imaging_parameters) == 3436, "layout");
static_assert(offsetof(SharedMemory, live_imaging_dirty_flags) == 3500, "layout");
static_assert(offsetof(SharedMemory, external_work_queue) == 3504, "layout");
static_assert(sizeof(Work) == 32 && offsetof(Work, generic) == 8, "layout");
static_assert(offsetof(Queue, items) == 8, "layout");
static_assert(sizeof(SharedMemory) <= SCRATCH_OFF, "layout");
static_assert(sizeof(BeamformerComputeStatsTable) <= SCRATCH_SIZE, "layout");

std::atomic<bool> g_stop{false};

long futex(int32_t *addr, int op, int32_t val, const struct timespec *ts)
{
	return syscall(SYS_futex, addr, op, val, ts, nullptr, 0);
}

/* take a lock word: 0 -> 1 by compare-and-swap, else wait on its value (up to
 * timeout_ms; -1 forever) */
bool lock(SharedMemory *sm, int32_t index, int32_t timeout_ms)
{
	int32_t *w = sm->locks + index;
	auto *a = reinterpret_cast<std::atomic<int32_t> *>(w);
	const auto t0 = std::chrono::steady_clock::now();
	while (true) {
		int32_t expected = 0;
		if (a->compare_exchange_strong(expected, 1)) return true;
		struct timespec ts = {0, 10 * 1000 * 1000};
		if (timeout_ms >= 0) {
			const auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0);
			if (el.count() >= timeout_ms) return false;
		}
		futex(w, FUTEX_WAIT, expected, &ts);
		if (g_stop) return false;
	}
}

void unlock(SharedMemory *sm, int32_t index)
{
	auto *a = reinterpret_cast<std::atomic<int32_t> *>(sm->locks + index);
	a->store(0);
	futex(sm->locks + index, FUTEX_WAKE, 0x7fffffff, nullptr);
}

/* the reference's post_sync_barrier: release a lock a client handed over */
void release_if_held(SharedMemory *sm, int32_t index)
{
	if (reinterpret_cast<std::atomic<int32_t> *>(sm->locks + index)->load()) unlock(sm, index);
}

void mark_clean(SharedMemory *sm, int32_t index)
{
	reinterpret_cast<std::atomic<uint32_t> *>(&sm->dirty_regions)->fetch_and(~(1u << (index - 1)));
}

struct Server {
	SharedMemory *sm = nullptr;
	uint8_t      *scratch = nullptr;
	bool          have_rf = false;
	bool          summed = false;       /* the last pipeline had a Sum stage */

	void log_error(const char *what)
	{
		std::fprintf(stderr, "ogl_beamformer_server: %s: %s\n", what, beamformer_get_last_error_string());
	}

	/* beamformer_rf_upload (beamformer.c:1230-1276) */
	void rf_upload()
	{
		if (!reinterpret_cast<std::atomic<int32_t> *>(sm->locks + LockUploadRF)->load()) return;
		if (!lock(sm, LockScratchSpace, -1)) return;
		const uint32_t size = sm->scratch_rf_size;
		if (size && size <= SCRATCH_SIZE) {
			if (!beamformer_push_data(scratch, size)) log_error("push_data");
			else have_rf = true;
		}
		mark_clean(sm, LockScratchSpace);
		unlock(sm, LockScratchSpace);
		release_if_held(sm, LockUploadRF);
	}

	/* parameters and pipeline as the client left them; pushed to the library when
	 * they differ from what it holds (clients also write output_points directly,
	 * without the dirty flag, as beamform_data_synchronized does) */
	BeamformerParameters last_params{};
	int32_t last_shaders[16] = {}, last_count = -1, last_kind = -1;
	uint8_t last_slots[16] = {};

	void take_parameters()
	{
		const uint32_t mask = (1u << (LockParameters - 1)) | (1u << (LockComputePipeline - 1));
		reinterpret_cast<std::atomic<uint32_t> *>(&sm->dirty_regions)->fetch_and(~mask);
		if (std::memcmp(&last_params, &sm->parameters, sizeof(last_params)) != 0) {
			if (!beamformer_push_parameters(&sm->parameters)) log_error("push_parameters");
			last_params = sm->parameters;
		}
		const int32_t n = sm->shader_count < 16 ? sm->shader_count : 16;
		if (n > 0 && (n != last_count || sm->data_kind != last_kind ||
		              std::memcmp(last_shaders, sm->shaders, 4 * (size_t)n) != 0 ||
		              std::memcmp(last_slots, sm->shader_parameters, (size_t)n) != 0)) {
			if (!beamformer_push_pipeline(sm->shaders, n, (BeamformerDataKind)sm->data_kind)) log_error("push_pipeline");
			for (int32_t i = 0; i < n; i++) beamformer_set_pipeline_stage_parameters(i, sm->shader_parameters[i]);
			last_count = n;
			last_kind = sm->data_kind;
			std::memcpy(last_shaders, sm->shaders, 4 * (size_t)n);
			std::memcpy(last_slots, sm->shader_parameters, (size_t)n);
		}
	}

	void compute()
	{
		take_parameters();
		release_if_held(sm, LockDispatchCompute);
		summed = false;
		for (int32_t i = 0; i < sm->shader_count && i < 16; i++)
			summed = summed || sm->shaders[i] == BeamformerShaderKind_Sum;
		if (have_rf && !beamformer_start_compute()) log_error("start_compute");
	}

	void export_buffer(const Work &w)
	{
		release_if_held(sm, LockDispatchCompute);
		lock(sm, w.lock, -1);
		const ExportContext &ec = w.export_context;
		if (ec.kind == ExportBeamformedData) {
			int32_t dims[3] = {0, 0, 0};
			const uint32_t which = summed ? 1u : 0u;
			if (beamformer_gb300_export_frame(which, 0, nullptr, 0, dims)) {
				const uint64_t bytes = (uint64_t)dims[0] * dims[1] * dims[2] * 2 * sizeof(float);
				if (bytes <= ec.size && bytes <= SCRATCH_SIZE &&
				    !beamformer_gb300_export_frame(which, 0, (float *)scratch, bytes, dims))
					log_error("export_frame");
			} else {
				log_error("export_frame");
			}
		} else if (ec.kind == ExportStats) {
			if (sizeof(BeamformerComputeStatsTable) <= ec.size &&
			    !beamformer_compute_timings((BeamformerComputeStatsTable *)scratch, -1))
				log_error("compute_timings");
		}
		unlock(sm, w.lock);
		release_if_held(sm, LockExportSync);
	}

	void upload_buffer(const Work &w)
	{
		lock(sm, w.lock, -1);
		switch (w.upload.kind) {
		case UploadChannelMapping: beamformer_push_channel_mapping(sm->channel_mapping, 256); break;
		case UploadFocalVectors:   beamformer_push_focal_vectors(&sm->focal_vectors[0][0], 256); break;
		case UploadSparseElements: beamformer_push_sparse_elements(sm->sparse_elements, 256); break;
		default: break;
		}
		mark_clean(sm, w.lock);
		unlock(sm, w.lock);
	}

	void create_filter(const Work &w)
	{
		const CreateFilterContext &f = w.create_filter;
		const uint8_t slot = (uint8_t)(f.slot % BEAMFORMER_FILTER_SLOTS);
		bool ok = true;
		if (f.kind == BeamformerFilterKind_Kaiser)
			ok = beamformer_create_kaiser_low_pass_filter(f.p0, f.p1, f.sampling_frequency, (int16_t)f.length, slot);
		else if (f.kind == BeamformerFilterKind_Matched)
			ok = beamformer_create_matched_filter(f.p0, f.p1, f.sampling_frequency, (int16_t)f.length, slot);
		if (!ok) log_error("create_filter");
	}

	/* complete_queue (beamformer.c:842-1111): every queued item in order */
	bool drain()
	{
		Queue &q = sm->external_work_queue;
		bool any = false;
		while (true) {
			const uint64_t val = q.queue.load();
			const uint64_t widx = val & 63, ridx = (val >> 32) & 63;
			if (ridx == widx) break;
			any = true;
			const Work &w = q.items[ridx];
			switch (w.kind) {
			case WorkCompute:
			case WorkComputeIndirect: rf_upload(); compute(); break;
			case WorkExportBuffer:    export_buffer(w); break;
			case WorkUploadBuffer:    upload_buffer(w); break;
			case WorkCreateFilter:    create_filter(w); break;
			default:                  break;     /* ReloadShader: no shader sources to reload */
			}
			q.queue.fetch_add(0x100000000ull);
		}
		return any;
	}
};

} /* namespace */

extern "C" {

/* Serve the reference's shared-memory protocol in the calling thread until
 * beamformer_gb300_serve_stop() or, with idle_exit_ms >= 0, that long without
 * work. Returns 0, or -1 when the region cannot be created. */
__attribute__((visibility("default"))) int32_t beamformer_gb300_serve(int32_t idle_exit_ms)
{
	g_stop = false;
	shm_unlink(SHM_NAME);
	const int fd = shm_open(SHM_NAME, O_CREAT | O_RDWR, S_IRUSR | S_IWUSR);
	if (fd < 0 || ftruncate(fd, (off_t)SHM_SIZE) != 0) {
		std::perror("ogl_beamformer_server: shm");
		if (fd >= 0) close(fd);
		return -1;
	}
	void *base = mmap(nullptr, SHM_SIZE, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
	close(fd);
	if (base == MAP_FAILED) {
		std::perror("ogl_beamformer_server: mmap");
		shm_unlink(SHM_NAME);
		return -1;
	}
	Server s;
	s.sm = (SharedMemory *)base;
	s.scratch = (uint8_t *)base + SCRATCH_OFF;
	std::memset(base, 0, sizeof(SharedMemory));
	s.sm->version = BEAMFORMER_SHARED_MEMORY_VERSION;
	beamformer_set_global_timeout(-1);
	/* the computing tables start as the fresh region holds them (zero), whatever
	 * an earlier in-process user of the library left there: a client that never
	 * uploads a table sees the same state on every start */
	beamformer_push_channel_mapping(s.sm->channel_mapping, 256);
	beamformer_push_focal_vectors(&s.sm->focal_vectors[0][0], 256);
	beamformer_push_sparse_elements(s.sm->sparse_elements, 256);

	auto last = std::chrono::steady_clock::now();
	while (!g_stop) {
		s.rf_upload();
		const bool any = s.drain();
		const auto now = std::chrono::steady_clock::now();
		if (any) {
			last = now;
		} else {
			if (idle_exit_ms >= 0 &&
			    std::chrono::duration_cast<std::chrono::milliseconds>(now - last).count() > idle_exit_ms)
				break;
			std::this_thread::sleep_for(std::chrono::microseconds(50));
		}
	}
	beamformer_gb300_synchronize(-1);
	s.sm->invalid = 1;                 /* later client calls fail, as after the reference exits */
	munmap(base, SHM_SIZE);
	shm_unlink(SHM_NAME);
	return 0;
}

__attribute__((visibility("default"))) void beamformer_gb300_serve_stop(void) { g_stop = true; }

} /* extern "C" */
