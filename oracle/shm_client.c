/*
 * shm_client.c -- test infrastructure: a restatement of the client side of the
 * reference's shared-memory protocol (helpers/ogl_beamformer_lib.c), used by the
 * tests to drive the GB300 server (beamformer_gb300_serve) where the reference's
 * own client library cannot be built (it is compiled from the reference checkout).
 * The reference's client library itself is exercised against the server in
 * tests/test_shm_server.py wherever oracle/_ref holds it.
 *
 * Region "/ogl_beamformer_shared_memory", 2 GB, BeamformerSharedMemory version 11:
 * locks at +8 (10 x i32), dirty_regions at +48, focal_vectors at +64,
 * channel_mapping at +2112, parameters at +3136, shaders at +3344,
 * shader_parameters at +3408, shader_count at +3424, data_kind at +3428,
 * scratch_rf_size at +3432, work queue at +3504 (u64 write/read indices, 64 x
 * 32-byte items), scratch space at +8192 (beamformer_work_queue.h:117-160).
 * Locks (os_linux.c:177-197): compare-and-swap 0 -> 1, FUTEX_WAIT on failure,
 * release = store 0 + FUTEX_WAKE.
 */
#include <fcntl.h>
#include <linux/futex.h>
#include <stdint.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/syscall.h>
#include <time.h>
#include <unistd.h>

#define SHM_SIZE      (2ull << 30)
#define SCRATCH_OFF   8192ull
#define OFF_LOCKS     8
#define OFF_DIRTY     48
#define OFF_FOCAL     64
#define OFF_CHMAP     2112
#define OFF_SPARSE    2624
#define OFF_PARAMS    3136
#define OFF_SHADERS   3344
#define OFF_SHPARAMS  3408
#define OFF_SHCOUNT   3424
#define OFF_DATAKIND  3428
#define OFF_RFSIZE    3432
#define OFF_QUEUE     3504
#define PARAMS_SIZE   208

enum { L_None, L_ComputePipeline, L_ChannelMapping, L_FocalVectors, L_Parameters, L_ScratchSpace,
       L_SparseElements, L_UploadRF, L_ExportSync, L_DispatchCompute };
enum { W_Compute, W_ComputeIndirect, W_CreateFilter, W_ReloadShader, W_ExportBuffer, W_UploadBuffer };

static uint8_t *g_base;

static int32_t *lockw(int i) { return (int32_t *)(g_base + OFF_LOCKS) + i; }

static int try_lock(int i, int32_t timeout_ms)
{
	struct timespec t0;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	for (;;) {
		int32_t expected = 0;
		if (__atomic_compare_exchange_n(lockw(i), &expected, 1, 0, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) return 1;
		if (timeout_ms == 0) return 0;
		if (timeout_ms > 0) {
			struct timespec t1;
			clock_gettime(CLOCK_MONOTONIC, &t1);
			int64_t el = (t1.tv_sec - t0.tv_sec) * 1000 + (t1.tv_nsec - t0.tv_nsec) / 1000000;
			if (el >= timeout_ms) return 0;
		}
		struct timespec ts = {0, 10 * 1000 * 1000};
		syscall(SYS_futex, lockw(i), FUTEX_WAIT, expected, &ts, 0, 0);
	}
}

static void release(int i)
{
	__atomic_store_n(lockw(i), 0, __ATOMIC_SEQ_CST);
	syscall(SYS_futex, lockw(i), FUTEX_WAKE, 0x7fffffff, 0, 0, 0);
}

static void mark_dirty(int i) { __atomic_or_fetch((uint32_t *)(g_base + OFF_DIRTY), 1u << (i - 1), __ATOMIC_SEQ_CST); }

/* beamform_work_queue_push: a zeroed item, or 0 when full */
static uint8_t *push_work(void)
{
	uint64_t *q = (uint64_t *)(g_base + OFF_QUEUE);
	uint64_t val = __atomic_load_n(q, __ATOMIC_SEQ_CST);
	uint64_t widx = val & 63, ridx = (val >> 32) & 63;
	if (((widx + 1) & 63) == ridx) return 0;
	uint8_t *item = g_base + OFF_QUEUE + 8 + 32 * widx;
	memset(item, 0, 32);
	return item;
}

static void push_commit(void) { __atomic_add_fetch((uint64_t *)(g_base + OFF_QUEUE), 1, __ATOMIC_SEQ_CST); }

int shmc_open(void)
{
	if (g_base) return 1;
	int fd = shm_open("/ogl_beamformer_shared_memory", O_RDWR, 0600);
	if (fd < 0) return 0;
	void *m = mmap(0, SHM_SIZE, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
	close(fd);
	if (m == MAP_FAILED) return 0;
	g_base = m;
	return *(uint32_t *)g_base == 11 && !*(uint32_t *)(g_base + 4);
}

void shmc_close(void)
{
	if (g_base) munmap(g_base, SHM_SIZE);
	g_base = 0;
}

int shmc_lock_states(int32_t out[10])
{
	for (int i = 0; i < 10; i++) out[i] = __atomic_load_n(lockw(i), __ATOMIC_SEQ_CST);
	return 1;
}

static int locked_upload(int off, const void *data, uint32_t size, int lk, int32_t timeout_ms, int *was_dirty)
{
	if (!try_lock(lk, timeout_ms)) return 0;
	if (was_dirty) *was_dirty = (*(uint32_t *)(g_base + OFF_DIRTY) >> (lk - 1)) & 1;
	memcpy(g_base + off, data, size);
	mark_dirty(lk);
	release(lk);
	return 1;
}

int shmc_push_parameters(const void *bp, int32_t timeout_ms)
{
	return locked_upload(OFF_PARAMS, bp, PARAMS_SIZE, L_Parameters, timeout_ms, 0);
}

int shmc_push_pipeline(const int32_t *shaders, int32_t count, int32_t data_kind, int32_t timeout_ms)
{
	if (count < 1 || count > 16 || !try_lock(L_ComputePipeline, timeout_ms)) return 0;
	*(int32_t *)(g_base + OFF_SHCOUNT) = count;
	*(int32_t *)(g_base + OFF_DATAKIND) = data_kind;
	memcpy(g_base + OFF_SHADERS, shaders, 4 * (size_t)count);
	mark_dirty(L_ComputePipeline);
	release(L_ComputePipeline);
	return 1;
}

/* beamformer_upload_buffer: region copy, then an UploadBuffer item with the lock */
static int upload_buffer(int off, const void *data, uint32_t size, int kind, int lk, int32_t timeout_ms)
{
	uint8_t *w = push_work();
	int dirty = 0;
	if (!w || !locked_upload(off, data, size, lk, timeout_ms, &dirty)) return 0;
	if (!dirty) {
		*(int32_t *)(w + 8) = kind;
		*(uint32_t *)(w + 12) = size;
		*(int32_t *)(w + 16) = off;
		*(int32_t *)(w + 0) = W_UploadBuffer;
		*(int32_t *)(w + 4) = lk;
		push_commit();
	}
	return 1;
}

int shmc_push_channel_mapping(const int16_t *map, uint32_t count, int32_t timeout_ms)
{
	return count <= 256 && upload_buffer(OFF_CHMAP, map, 2 * count, 0, L_ChannelMapping, timeout_ms);
}

int shmc_push_focal_vectors(const float *v, uint32_t count, int32_t timeout_ms)
{
	return count <= 256 && upload_buffer(OFF_FOCAL, v, 8 * count, 1, L_FocalVectors, timeout_ms);
}

int shmc_create_kaiser(float beta, float cutoff, float fs, int16_t length, uint8_t slot)
{
	uint8_t *w = push_work();
	if (!w) return 0;
	*(int32_t *)(w + 0) = W_CreateFilter;
	*(int32_t *)(w + 8) = 0;                 /* Kaiser */
	*(float *)(w + 12) = beta;
	*(float *)(w + 16) = cutoff;
	*(float *)(w + 20) = fs;
	*(int32_t *)(w + 24) = length;
	*(int32_t *)(w + 28) = slot % 4;
	push_commit();
	return 1;
}

static int push_data(const void *data, uint32_t size, int32_t timeout_ms)
{
	if (size > SHM_SIZE - SCRATCH_OFF || !try_lock(L_UploadRF, timeout_ms)) return 0;
	if (!locked_upload((int)SCRATCH_OFF, data, size, L_ScratchSpace, 0, 0)) return 0;
	*(uint32_t *)(g_base + OFF_RFSIZE) = size;
	return 1;
}

static int compute_indirect(void)
{
	uint8_t *w = push_work();
	if (!w) return 0;
	*(int32_t *)(w + 0) = W_ComputeIndirect;
	*(int32_t *)(w + 8) = 0;
	push_commit();
	try_lock(L_DispatchCompute, 0);
	return 1;
}

int shmc_push_data_with_compute(const void *data, uint32_t size, int32_t timeout_ms)
{
	return push_data(data, size, timeout_ms) && compute_indirect();
}

static int export_buffer(int kind, uint32_t size)
{
	uint8_t *w = push_work();
	if (!w || !try_lock(L_ExportSync, 0)) return 0;
	*(int32_t *)(w + 8) = kind;
	*(uint32_t *)(w + 12) = size;
	*(int32_t *)(w + 0) = W_ExportBuffer;
	*(int32_t *)(w + 4) = L_ScratchSpace;
	push_commit();
	return 1;
}

static int read_output(void *out, uint64_t size, int32_t timeout_ms)
{
	if (!try_lock(L_ExportSync, timeout_ms)) return 0;
	release(L_ExportSync);
	if (!try_lock(L_ScratchSpace, 0)) return 0;
	memcpy(out, g_base + SCRATCH_OFF, size);
	release(L_ScratchSpace);
	return 1;
}

int shmc_beamform_data_synchronized(const void *data, uint32_t size, int32_t pts[3], float *out, int32_t timeout_ms)
{
	for (int i = 0; i < 3; i++) {
		if (pts[i] < 1) pts[i] = 1;
		((int32_t *)(g_base + OFF_PARAMS + 144))[i] = pts[i];     /* parameters.output_points */
	}
	uint64_t osize = (uint64_t)(uint32_t)pts[0] * (uint32_t)pts[1] * (uint32_t)pts[2] * 8;
	if (osize > SHM_SIZE - SCRATCH_OFF) return 0;
	if (!shmc_push_data_with_compute(data, size, timeout_ms)) return 0;
	if (!export_buffer(0, (uint32_t)osize)) return 0;
	try_lock(L_DispatchCompute, 0);
	return read_output(out, osize, timeout_ms);
}

int shmc_compute_timings(void *out, uint32_t size, int32_t timeout_ms)
{
	if (!export_buffer(1, size)) return 0;
	try_lock(L_DispatchCompute, 0);
	return read_output(out, size, timeout_ms);
}
