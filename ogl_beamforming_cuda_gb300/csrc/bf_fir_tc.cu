/*
 * bf_fir_tc.cu -- demodulation + decimating FIR as a Toeplitz contraction on the
 * fifth-generation tensor cores: the precision variant of the Demodulate stage
 * (reference: shaders/filter.glsl:55-91, demodulation of decoded real pairs).
 *
 * Reference semantics (per (channel, transmit) row, outputs n < S', taps h):
 *   w[j] = sqrt(2) e^{i theta j} (x[2j] - i x[2j+1]),  theta = 2 pi fc / (fs / 2)
 *   y[n] = sum_{k=1..L} h[k-1] w[nD - k]
 * Rewritten as  y[n] = e^{i theta n D} z[n],  z[n] = sum_k g[k] v[nD - k]  with
 * g[k] = sqrt(2) h[k-1] e^{-i theta k} and v[j] = x[2j] - i x[2j+1]: the per-sample
 * rotation becomes complex taps plus one rotation per output (epilogue).
 *
 * Contraction. A block of B = 32 / D consecutive outputs of a row reads a window
 * of 64 (1 + E / 64) real input samples, E = 2L rounded up to 64, starting at the
 * real sample 64 q - E (q = output block). With 128 rows per CTA:
 *   Z[128 rows x 2B] = X[128 rows x K] . G[K x 2B],  K = 64 + E,
 * where X holds the rows' windows (fp16 or bf16 decoded samples) and G is the
 * fixed Toeplitz arrangement of (Re, Im) g over real-sample offsets (columns
 * 0..B-1 give Re z, B..2B-1 Im z). Consecutive output blocks' windows overlap in
 * all but one 64-sample atom, so a CTA keeps its windows as a ring of 64-column
 * atoms (128 rows x 128 bytes, 128-byte swizzled, loaded by TMA) and each block
 * needs one new atom: every input element is read from memory once per CTA.
 *
 * Per block: one thread waits for the block's atoms, issues 4 (1 + E / 64)
 * tcgen05.mma (M = 128, N = 2B, K = 16, fp16/bf16 operands, FP32 accumulate in
 * tensor memory, double-buffered columns) and commits to an mbarrier; all four
 * warps read their 32 accumulator lanes with tcgen05.ld, rotate by e^{i theta n D},
 * stage the rows in a padded shared-memory tile and store complex f32 [row][n] as
 * whole row segments (16 bytes per lane, coalesced). The next block's MMAs are
 * issued before the epilogue of the current one; each warp releases an
 * accumulator buffer on an mbarrier once it has read it (no block-wide barrier
 * per block). Every wait is bounded (about one second); a wait that runs out
 * sets the error word and the CTA stops after draining its loads.
 */
#include "bf_kernels.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

namespace bf {

constexpr int TC_RING = 8;                      /* window atoms resident per CTA */
constexpr int TC_M = 128;                       /* rows per CTA (MMA M) */
constexpr int TC_ATOM_BYTES = TC_M * 128;       /* 128 rows x 64 16-bit samples */
constexpr long long TC_WAIT_CYCLES = 2000000000ll;   /* ~1 s at 2 GHz */

struct FirTcParams {
	float2       *out;          /* complex f32 [row][n] */
	const float2 *rot;          /* e^{i theta n D} for n < n_out */
	int32_t       rows;         /* (channel, transmit) rows */
	int32_t       n_out;        /* outputs per row */
	int32_t       B;            /* outputs per block: 32 / D */
	int32_t       atoms;        /* window atoms per block: 1 + E / 64 */
	int32_t       q_blocks;     /* ceil(n_out / B) */
	int32_t       splits;       /* CTAs per 128-row block */
	int32_t       x_first;      /* -E: real-sample coordinate of block 0's window */
	uint32_t      idesc;        /* tcgen05 instruction descriptor */
	unsigned     *error;        /* set to 1 when a wait runs out */
	long long     stall_cycles; /* > 0 (tests only): the first wait is on a barrier nothing
	                               arrives at, bounded by this many cycles, so it runs out */
	int32_t       vec_store;    /* rows start 16-byte aligned (n_out even): 16-byte stores */
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}

/* bounded wait for the phase with the given parity to complete */
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = TC_WAIT_CYCLES)
{
	const long long t0 = clock64();
	while (true) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if (clock64() - t0 > limit) return false;
	}
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
	             :: "r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar) : "memory");
}

/* shared-memory matrix descriptor: K-major operand in 128-byte swizzled atoms
 * (8 rows x 128 B = 1024 B per core-matrix group, SBO = 1024 B; the leading
 * offset is unused for this layout), descriptor version 1 */
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr)
{
	uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
	d |= (uint64_t)1 << 16;
	d |= (uint64_t)(1024 >> 4) << 32;
	d |= (uint64_t)1 << 46;
	d |= (uint64_t)2 << 61;
	return d;
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "setp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
	             :: "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after()  { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* 16 consecutive f32 accumulator columns of this warp's 32 lanes */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
	             "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
	#pragma unroll
	for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

/* 32 consecutive f32 accumulator columns of this warp's 32 lanes */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v)
{
	uint32_t r[32];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
	             "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
	             "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
	               "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
	               "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
	#pragma unroll
	for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

template <int N>    /* accumulator columns: 2 B (Re and Im of B outputs) */
__global__ void __launch_bounds__(128, 1)
fir_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap, FirTcParams p)
{
	constexpr int B = N / 2;
	extern __shared__ uint8_t smem_raw[];
	uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	uint8_t *ring = smem;                                        /* TC_RING atoms */
	uint8_t *gsm  = ring + TC_RING * TC_ATOM_BYTES;              /* atoms x (N rows x 128 B) */
	uint64_t *bars = (uint64_t *)(gsm + (size_t)p.atoms * N * 128);
	float4 *epi = (float4 *)(bars + TC_RING + 6);              /* 4 warps x 32 rows x (N / 4 + 1) chunks */
	__shared__ uint32_t tmem_slot;
	__shared__ volatile int stop;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int rb = blockIdx.x / p.splits, split = blockIdx.x - rb * p.splits;
	const int row0 = rb * TC_M;
	const int qpb = (p.q_blocks + p.splits - 1) / p.splits;
	const int q0 = split * qpb, q1 = min(p.q_blocks, q0 + qpb);
	if (q0 >= q1) return;                      /* uniform over the CTA, before any allocation */
	const int nq = q1 - q0;
	const int total_atoms = nq + p.atoms - 1;

	const uint32_t full0 = smem_u32(bars), mma0 = smem_u32(bars + TC_RING), gbar = smem_u32(bars + TC_RING + 2);
	const uint32_t never = smem_u32(bars + TC_RING + 3);        /* no thread or copy arrives here */
	const uint32_t aempty0 = smem_u32(bars + TC_RING + 4);      /* accumulator buffer read by all 4 warps */
	/* two accumulator buffers of N f32 columns; allocations are powers of two >= 32 */
	constexpr uint32_t tcols = N <= 16 ? 32u : N <= 32 ? 64u : 128u;
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		             :: "r"(smem_u32(&tmem_slot)), "r"(tcols) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0) {
		for (int i = 0; i < TC_RING; i++) mbar_init(full0 + 8 * i, 1);
		mbar_init(mma0, 1);
		mbar_init(mma0 + 8, 1);
		mbar_init(gbar, 1);
		mbar_init(never, 1);
		mbar_init(aempty0, 4);
		mbar_init(aempty0 + 8, 4);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		stop = 0;
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;

	int issued = 0;                            /* atoms issued (thread 0) */
	auto issue_atom = [&](int a) {
		const uint32_t slot = (uint32_t)(a % TC_RING);
		mbar_expect_tx(full0 + 8 * slot, TC_ATOM_BYTES);
		tma_load_2d(smem_u32(ring) + slot * TC_ATOM_BYTES, &xmap, p.x_first + 64 * (q0 + a), row0, full0 + 8 * slot);
	};
	/* MMAs of local block i into accumulator columns (i % 2) * N; false if a wait ran out */
	auto mma_block = [&](int i) -> bool {
		for (int a = 0; a < p.atoms; a++)
			if (!mbar_wait(full0 + 8 * ((i + a) % TC_RING), (uint32_t)(((i + a) / TC_RING) & 1))) return false;
		tc_fence_after();
		const uint32_t d = tmem + (uint32_t)((i & 1) * N);
		for (int a = 0; a < p.atoms; a++) {
			const uint32_t abase = smem_u32(ring) + (uint32_t)((i + a) % TC_RING) * TC_ATOM_BYTES;
			const uint32_t bbase = smem_u32(gsm) + (uint32_t)(a * N * 128);
			#pragma unroll
			for (int ks = 0; ks < 4; ks++)
				mma_f16(d, sw128_desc(abase + 32 * ks), sw128_desc(bbase + 32 * ks), p.idesc, (a | ks) != 0);
		}
		mma_commit(mma0 + 8 * (i & 1));
		return true;
	};

	bool ok = true;
	if (tid == 0) {
		mbar_expect_tx(gbar, (uint32_t)(p.atoms * N * 128));
		for (int a = 0; a < p.atoms; a++) tma_load_2d(smem_u32(gsm) + (uint32_t)(a * N * 128), &gmap, 64 * a, 0, gbar);
		for (; issued < total_atoms && issued < TC_RING; issued++) issue_atom(issued);
		ok = (p.stall_cycles <= 0 || mbar_wait(never, 0, p.stall_cycles)) && mbar_wait(gbar, 0) && mma_block(0);
		if (!ok) stop = 1;
	}
	__syncthreads();

	/* No block-wide barrier per block: a warp releases accumulator buffer i % 2
	 * (one arrival on its "empty" mbarrier) once it has read it, and thread 0 waits
	 * for that before the MMAs of block i + 2 overwrite it; an input atom's slot is
	 * refilled as soon as the MMAs of the last block reading it are complete. */
	for (int i = 0; i < nq && !stop; i++) {
		if (tid == 0 && i + 1 < nq) {
			/* buffer (i + 1) % 2 last held block i - 1 */
			if (i >= 1 && !mbar_wait(aempty0 + 8 * ((i + 1) & 1), (uint32_t)(((i - 1) >> 1) & 1))) stop = 1;
			else if (!mma_block(i + 1)) stop = 1;
		}
		/* every thread: accumulators of block i */
		const bool done = __all_sync(0xFFFFFFFFu, mbar_wait(mma0 + 8 * (i & 1), (uint32_t)((i >> 1) & 1)));
		tc_fence_after();
		/* block i's MMAs are complete: its first atom's slot takes atom i + TC_RING */
		if (tid == 0 && done && !stop && issued < total_atoms) issue_atom(issued++);
		if (done) {
			/* this warp's lanes, the N columns of accumulator buffer i % 2 */
			float v[64];
			const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((i & 1) * N);
			if (N == 16) {
				tmem_ld16(ta, v);
			} else {
				tmem_ld32(ta, v);
				if (N == 64) tmem_ld32(ta + 32, v + 32);
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(aempty0 + 8 * (i & 1)) : "memory");
			/* rotate this lane's row into the warp's staging tile (row = lane, 16-byte
			 * chunks of two outputs, rows padded by one chunk: conflict-free both ways),
			 * then store whole row segments: CPR lanes per row, 32 / CPR rows per
			 * instruction, 16 bytes per lane (coalesced) */
			constexpr int CPR = B / 2;
			float4 *tile = epi + warp * 32 * (CPR + 1);
			const int nb = (q0 + i) * B;
			#pragma unroll
			for (int j = 0; j < B; j += 2) {
				const int n = nb + j;
				const float2 r0 = __ldg(p.rot + min(n, p.n_out - 1)), r1 = __ldg(p.rot + min(n + 1, p.n_out - 1));
				const float a = v[j], b = v[B + j], c = v[j + 1], d = v[B + j + 1];
				tile[lane * (CPR + 1) + j / 2] =
				    make_float4(a * r0.x - b * r0.y, a * r0.y + b * r0.x, c * r1.x - d * r1.y, c * r1.y + d * r1.x);
			}
			__syncwarp();
			#pragma unroll
			for (int k = 0; k < 32; k += 32 / CPR) {
				const int rl = k + lane / CPR, ch = lane % CPR;
				const int row = row0 + warp * 32 + rl, n = nb + 2 * ch;
				const float4 y = tile[rl * (CPR + 1) + ch];
				if (row < p.rows && n < p.n_out) {
					float2 *o = p.out + (size_t)row * p.n_out + n;
					if (p.vec_store && n + 1 < p.n_out) {
						*(float4 *)o = y;
					} else {
						o[0] = make_float2(y.x, y.y);
						if (n + 1 < p.n_out) o[1] = make_float2(y.z, y.w);
					}
				}
			}
			__syncwarp();
		} else {
			stop = 1;
		}
	}
	__syncthreads();
	if (tid == 0 && stop) {
		atomicExch(p.error, 1u);
		/* drain the loads still in flight (the tap table and the ring's atoms)
		 * before the shared memory is released */
		mbar_wait(gbar, 0);
		for (int a = max(0, issued - TC_RING); a < issued; a++)
			mbar_wait(full0 + 8 * (a % TC_RING), (uint32_t)((a / TC_RING) & 1));
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(tcols) : "memory");
}

/* ------------------------------------ host ------------------------------------ */

/* the driver's cuTensorMapEncodeTiled (12.0 interface), looked up once; null when
 * the driver does not provide it */
void *tensor_map_encoder()
{
	static std::once_flag once;
	static void *fn = nullptr;
	std::call_once(once, [] {
		void *f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = f;
		cudaGetLastError();
	});
	return fn;
}

/* 2D map over the first `cols` columns of a [rows][pitch] 16-bit array (columns at
 * or beyond `cols` read as 0), 128-byte swizzled boxes of 64 x box_rows */
static bool make_map(CUtensorMap *m, const void *base, uint64_t cols, uint64_t pitch, uint64_t rows,
                     uint32_t box_rows, bool bf16)
{
	const auto enc = (PFN_cuTensorMapEncodeTiled_v12000)tensor_map_encoder();
	if (!enc) return false;
	const cuuint64_t dims[2] = {cols, rows};
	const cuuint64_t strides[1] = {pitch * 2};
	const cuuint32_t box[2] = {64, box_rows};
	const cuuint32_t estr[2] = {1, 1};
	return enc(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base),
	           dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
	           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static uint16_t to_half_bits(double v, bool bf16)
{
	float f = (float)v;
	if (bf16) {
		uint32_t u;
		std::memcpy(&u, &f, 4);
		u += 0x7FFFu + ((u >> 16) & 1u);     /* round to nearest even */
		return (uint16_t)(u >> 16);
	}
	__half h = __float2half_rn(f);
	uint16_t b;
	std::memcpy(&b, &h, 2);
	return b;
}

bool fir_tc_supported(uint32_t decimation, uint32_t taps)
{
	if (decimation != 1 && decimation != 2 && decimation != 4) return false;
	const uint32_t E = (2 * taps + 63) / 64 * 64;
	return taps >= 1 && 1 + E / 64 <= TC_RING - 2;
}

int64_t fir_tc_table_bytes(uint32_t decimation, uint32_t taps, uint32_t n_out)
{
	const uint32_t B = 32 / decimation, E = (2 * taps + 63) / 64 * 64;
	return (int64_t)(2 * B) * (64 + E) * 2 + (int64_t)n_out * sizeof(float2);
}

bool fir_tc_tables(uint32_t decimation, const float *h, uint32_t taps, double demod_frequency, double demod_fs,
                   uint32_t n_out, bool bf16, void *table)
{
	if (!fir_tc_supported(decimation, taps)) return false;
	const uint32_t D = decimation, B = 32 / D, N = 2 * B, E = (2 * taps + 63) / 64 * 64, K = 64 + E;
	const double theta = 2.0 * M_PI * demod_frequency / demod_fs;
	std::vector<uint16_t> G((size_t)N * K, 0);
	for (uint32_t j = 0; j < B; j++)
		for (uint32_t k = 1; k <= taps; k++) {
			const double gr = std::sqrt(2.0) * (double)h[k - 1] * std::cos(theta * k);
			const double gi = -std::sqrt(2.0) * (double)h[k - 1] * std::sin(theta * k);
			const int64_t col = 2 * ((int64_t)j * D - (int64_t)k) + E;     /* real sample 2(jD - k) of the window */
			G[(size_t)j * K + col]           = to_half_bits(gr, bf16);
			G[(size_t)j * K + col + 1]       = to_half_bits(gi, bf16);
			G[(size_t)(B + j) * K + col]     = to_half_bits(gi, bf16);
			G[(size_t)(B + j) * K + col + 1] = to_half_bits(-gr, bf16);
		}
	std::vector<float2> rot(n_out);
	for (uint32_t n = 0; n < n_out; n++) {
		const double a = std::fmod(theta * (double)n * D, 2.0 * M_PI);
		rot[n] = make_float2((float)std::cos(a), (float)std::sin(a));
	}
	uint8_t *t = (uint8_t *)table;
	if (cudaMemcpy(t, G.data(), G.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess) return false;
	return cudaMemcpy(t + G.size() * 2, rot.data(), rot.size() * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
}

/* x: [rows][row_samples] 16-bit; samples at or beyond valid_samples read as 0 */
cudaError_t launch_fir_tc(const void *x, uint32_t rows, uint32_t row_samples, uint32_t valid_samples,
                          uint32_t decimation, uint32_t taps, uint32_t n_out, bool bf16, const void *table,
                          float2 *out, unsigned *error, cudaStream_t s)
{
	if (!fir_tc_supported(decimation, taps) || rows == 0 || n_out == 0 || row_samples % 8 != 0 ||
	    valid_samples == 0 || valid_samples > row_samples)
		return cudaErrorInvalidValue;
	const uint32_t D = decimation, B = 32 / D, N = 2 * B, E = (2 * taps + 63) / 64 * 64, K = 64 + E;
	CUtensorMap xmap, gmap;
	if (!make_map(&xmap, x, valid_samples, row_samples, rows, TC_M, bf16)) return cudaErrorInvalidValue;
	if (!make_map(&gmap, table, K, K, N, N, bf16)) return cudaErrorInvalidValue;
	FirTcParams p{};
	p.out = out;
	p.rot = (const float2 *)((const uint8_t *)table + (size_t)N * K * 2);
	p.rows = (int32_t)rows;
	p.n_out = (int32_t)n_out;
	p.B = (int32_t)B;
	p.atoms = (int32_t)(K / 64);
	p.q_blocks = (int32_t)((n_out + B - 1) / B);
	p.x_first = -(int32_t)E;
	/* D = f32 (bit 4), A and B fp16 (0) or bf16 (1) at bits 7 and 10, both K-major,
	 * N >> 3 at bit 17, M >> 4 at bit 24 */
	const uint32_t ab = bf16 ? 1u : 0u;
	p.idesc = (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
	p.error = error;
	/* test hook: OGL_BF_TEST_FIR_STALL_CYCLES=n makes every CTA's first wait run out
	 * after n cycles (the error word is then set and the kernel stops early) */
	if (const char *stall = std::getenv("OGL_BF_TEST_FIR_STALL_CYCLES")) p.stall_cycles = std::atoll(stall);
	const int row_blocks = (int)((rows + TC_M - 1) / TC_M);
	/* at least ~4 CTAs per SM's worth of work, at least 4 output blocks per CTA */
	int splits = (4 * device_sm_count() + row_blocks - 1) / row_blocks;
	splits = std::min(splits, std::max(1, p.q_blocks / 4));
	p.splits = splits;
	p.vec_store = (n_out % 2 == 0 && ((uintptr_t)out & 15) == 0) ? 1 : 0;
	const size_t smem = 1024 + (size_t)TC_RING * TC_ATOM_BYTES + (size_t)p.atoms * N * 128 + (TC_RING + 6) * 8 +
	                    (size_t)4 * 32 * (N / 4 + 1) * 16;
	/* the dynamic shared memory this launch needs, within the device's opt-in limit
	 * less the kernel's static shared memory */
	int dev = 0, optin = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
	if (e != cudaSuccess) return e;
	const void *fn = N == 16 ? (const void *)fir_tc<16> : N == 32 ? (const void *)fir_tc<32> : (const void *)fir_tc<64>;
	cudaFuncAttributes fa{};
	if ((e = cudaFuncGetAttributes(&fa, fn)) != cudaSuccess) return e;
	if (smem + fa.sharedSizeBytes > (size_t)optin) return cudaErrorInvalidValue;
	if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) return e;
	const int grid = row_blocks * splits;
	switch (N) {
	case 16: fir_tc<16><<<grid, 128, smem, s>>>(xmap, gmap, p); break;
	case 32: fir_tc<32><<<grid, 128, smem, s>>>(xmap, gmap, p); break;
	default: fir_tc<64><<<grid, 128, smem, s>>>(xmap, gmap, p); break;
	}
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
