/*
 * bf_unet_tc.cu -- the learned variant's 3 x 3 x 3 convolution forward as an
 * implicit GEMM on the fifth-generation tensor cores (tcgen05), BF16 operands and
 * FP32 accumulation in tensor memory. Same contract as bf_unet_conv3d's direct
 * kernel (channels-first [C][D][H][W] activations, weights [Cout][Cin][27], zero
 * padding, bias, optional ReLU and residual), for BF16 inputs.
 *
 * GEMM. out[co][v] = sum_k A[v][k] B[co][k] with M = voxels (tiles of 128
 * consecutive voxels in x-fastest order), N = output channels (padded to a
 * multiple of 16) and K = 27 taps x input channels, input channels padded to a
 * multiple of 8 so that every 8-element group of K belongs to one tap:
 * k = tap * cin_p + ci, A[v][k] = in[ci][v + offset(tap)] (0 outside the volume).
 * K runs in chunks of 64 (one 128-byte row of a swizzle atom).
 *
 * Per chunk a CTA of 128 threads builds its A tile (128 voxel rows x 64 K, BF16)
 * in shared memory in the 128-byte-swizzled K-major layout that tcgen05 reads
 * (row r at r * 128 bytes, 16-byte group j at position j ^ (r mod 8)): thread r
 * gathers its voxel's 64 values (8 input channels at one tap per group) and
 * stores them as 8 16-byte words. The B tile (the chunk's weights, N x 64) is
 * arranged once per call in global memory in the same layout by
 * prepare_weights_tc and copied with one cp.async.bulk. One thread then issues
 * four tcgen05.mma (M = 128, N, K = 16) into the tensor-memory accumulator and
 * commits to an mbarrier; A and B are double-buffered, so the next chunk's
 * gather runs while the tensor core works. After the last chunk every warp reads
 * its 32 voxel rows of the accumulator with tcgen05.ld, adds the bias (ReLU,
 * residual) and stores each output channel's 32 consecutive voxels (coalesced).
 * CTAs are persistent over the voxel tiles.
 *
 * Two forms share that GEMM:
 *  - conv3d_tma (volumes whose rows tile by 128 voxels: W a divisor of 128 with
 *    H a multiple of 128 / W, or W a multiple of 128). The input is first
 *    rewritten channels-last ([D][H][W][cin_p], cin_p a multiple of 16). One
 *    K = 16 step is then (tap, 16 input channels), and its A operand is ONE 4D
 *    TMA box of the channels-last tensor: 16 channels x 128 voxels at the tile's
 *    origin shifted by the tap, zero-filled outside the volume by the copy engine,
 *    landing in the 32-byte-swizzled K-major layout that tcgen05 reads. Warp 0
 *    loads (four boxes and the chunk's weights per stage, a ring of stages), warp
 *    1 issues the MMAs into one of two tensor-memory accumulators, warps 2-5 read
 *    the other accumulator and store the previous tile.
 *  - conv3d_tc (any volume): the threads gather each chunk's A tile from the
 *    channels-first input, 8 channels per 16-byte group, into 128-byte-swizzled
 *    rows.
 *
 * Every wait is bounded (about one second); a wait that runs out sets the error
 * word (bf_unet_tc_errors), the CTA waits (bounded) for its copies and tensor
 * operations in flight, frees its tensor memory and stops.
 */
#include "bf_kernels.h"
#include "bf_unet.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace bf {
namespace {

constexpr int TCM = 128;                         /* voxels per tile: the MMA's M */
constexpr int TCK = 64;                          /* K per chunk */
constexpr int A_BYTES = TCM * TCK * 2;           /* 16 KB */
constexpr long long TC_WAIT = 2000000000ll;      /* ~1 s at 2 GHz */

__device__ unsigned g_unet_tc_error;

struct ConvTc {
	const __nv_bfloat16 *in;
	const uint8_t       *bk;        /* [chunk][np rows][128 B], swizzled */
	const float         *bias;
	const void          *residual;
	void                *out;
	int32_t              cin, cin_p, cout, np, nch;
	int32_t              W, H, D;
	int64_t              V;
	int32_t              relu, tiles;
	uint32_t             idesc;
};

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity)
{
	const long long t0 = clock64();
	while (true) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if (clock64() - t0 > TC_WAIT) return false;
	}
}

/* K-major operand in 128-byte swizzled atoms (8 rows x 128 B, SBO 1024 B),
 * descriptor version 1 */
__device__ __forceinline__ uint64_t sw128(uint32_t addr)
{
	uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
	d |= (uint64_t)1 << 16;
	d |= (uint64_t)(1024 >> 4) << 32;
	d |= (uint64_t)1 << 46;
	d |= (uint64_t)2 << 61;
	return d;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after()  { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void ld16(uint32_t taddr, float *v)
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

__device__ __forceinline__ void put(float *p, int64_t i, float v) { p[i] = v; }
__device__ __forceinline__ void put(__nv_bfloat16 *p, int64_t i, float v) { p[i] = __float2bfloat16_rn(v); }
__device__ __forceinline__ float get(const float *p, int64_t i) { return __ldg(p + i); }
__device__ __forceinline__ float get(const __nv_bfloat16 *p, int64_t i) { return __bfloat162float(p[i]); }

/* B tiles: element (n, k) of chunk c at c * np * 128 + n * 128 + ((k / 8) ^ (n % 8)) * 16 + (k % 8) * 2,
 * k = c * 64 + k' -> tap = k / cin_p, ci = k % cin_p; zero beyond cout, cin and the 27 taps */
__global__ void __launch_bounds__(256)
prepare_weights_tc(const __nv_bfloat16 *__restrict__ w, uint16_t *__restrict__ bk, int cin, int cin_p, int cout, int np,
                   int nch)
{
	const int64_t total = (int64_t)nch * np * TCK;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
		const int kk = (int)(i % TCK);
		const int64_t r = i / TCK;
		const int n = (int)(r % np), c = (int)(r / np);
		const int k = c * TCK + kk, tap = k / cin_p, ci = k - tap * cin_p;
		uint16_t v = 0;
		if (n < cout && ci < cin && tap < 27) v = __bfloat16_as_ushort(w[((int64_t)n * cin + ci) * 27 + tap]);
		const int64_t o = ((int64_t)c * np + n) * TCK + (((kk >> 3) ^ (n & 7)) << 3) + (kk & 7);
		bk[o] = v;
	}
}

template <typename TO>
__global__ void __launch_bounds__(128)
conv3d_tc(const __grid_constant__ ConvTc p)
{
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	uint8_t *abuf = sm;                                        /* 2 x A_BYTES */
	const int bbytes = p.np * 128;
	uint8_t *bbuf = sm + 2 * A_BYTES;                          /* 2 x bbytes */
	uint64_t *bars = (uint64_t *)(bbuf + 2 * bbytes);          /* copy[2], mma[2] */
	__shared__ uint32_t tmem_slot;

	const int tid = threadIdx.x, warp = tid >> 5;
	const uint32_t cbar0 = su32(bars), mbar0 = su32(bars + 2);
	const uint32_t tcols = p.np <= 32 ? 32u : p.np <= 64 ? 64u : 128u;
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		             :: "r"(su32(&tmem_slot)), "r"(tcols) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0) {
		for (int i = 0; i < 4; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(cbar0 + 8 * i), "r"(1) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;

	const int64_t plane = (int64_t)p.H * p.W;
	/* element offsets of the 27 taps (channels-first, x fastest) */
	__shared__ int64_t toff[27];
	if (tid < 27) toff[tid] = (int64_t)(tid / 9 - 1) * plane + (int64_t)((tid / 3) % 3 - 1) * p.W + (tid % 3 - 1);
	__syncthreads();
	uint32_t g = 0;                  /* chunks issued so far (phase bookkeeping) */
	int last_b[2] = {-1, -1};        /* last chunk committed / copied on each buffer (thread 0) */
	bool fail = false;
	const int bb = bbytes;
	for (int tile = blockIdx.x; tile < p.tiles && !fail; tile += gridDim.x) {
		const int64_t v = (int64_t)tile * TCM + tid;
		const bool vin = v < p.V;
		const int x = (int)(v % p.W), y = (int)((v / p.W) % p.H), z = (int)(v / plane);
		/* taps whose neighbour lies inside the volume */
		uint32_t mask = 0;
		if (vin)
			#pragma unroll
			for (int t = 0; t < 27; t++) {
				const int xx = x + t % 3 - 1, yy = y + (t / 3) % 3 - 1, zz = z + t / 9 - 1;
				mask |= (uint32_t)(xx >= 0 && xx < p.W && yy >= 0 && yy < p.H && zz >= 0 && zz < p.D) << t;
			}
		int tap = 0, ci0 = 0;            /* of the next 8-element group of K */
		for (int c = 0; c < p.nch; c++, g++) {
			const int b = (int)(g & 1);
			bool ok = true;
			if (g >= 2) ok = bar_wait(mbar0 + 8 * b, ((g - 2) >> 1) & 1);    /* buffer b free */
			if (tid == 0 && ok) {
				/* this chunk's weights: the copy runs while the threads gather */
				const uint32_t cb = cbar0 + 8 * b, dst = su32(bbuf + b * bb);
				const uint8_t *src = p.bk + (size_t)c * bb;
				asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(cb), "r"(bb) : "memory");
				asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
				             :: "r"(dst), "l"(src), "r"(bb), "r"(cb) : "memory");
				last_b[b] = (int)g;
			}
			/* gather this thread's voxel row: 8 groups of 8 input channels at one tap */
			uint8_t *arow = abuf + b * A_BYTES + tid * 128;
			#pragma unroll 4
			for (int grp = 0; grp < 8; grp++) {
				uint32_t w4[4] = {0u, 0u, 0u, 0u};
				if (tap < 27 && ((mask >> tap) & 1u)) {
					const __nv_bfloat16 *src = p.in + (int64_t)ci0 * p.V + v + toff[tap];
					if (ci0 + 8 <= p.cin) {
						#pragma unroll
						for (int i = 0; i < 8; i++)
							w4[i >> 1] |= (uint32_t)__bfloat16_as_ushort(src[(int64_t)i * p.V]) << ((i & 1) * 16);
					} else {
						#pragma unroll
						for (int i = 0; i < 8; i++)
							if (ci0 + i < p.cin)
								w4[i >> 1] |= (uint32_t)__bfloat16_as_ushort(src[(int64_t)i * p.V]) << ((i & 1) * 16);
					}
				}
				*(uint4 *)(arow + ((grp ^ (tid & 7)) << 4)) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
				ci0 += 8;
				if (ci0 >= p.cin_p) { ci0 = 0; tap++; }
			}
			/* the gather (generic proxy) before the tensor core reads it (async proxy) */
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			if (__syncthreads_or(!ok)) { fail = true; break; }
			if (tid == 0) {
				if (!bar_wait(cbar0 + 8 * b, (g >> 1) & 1)) {
					fail = true;
				} else {
					tc_fence_after();
					const uint32_t a0 = su32(abuf + b * A_BYTES), b0 = su32(bbuf + b * bb);
					#pragma unroll
					for (int ks = 0; ks < 4; ks++) {
						const uint32_t acc = (c | ks) != 0;
						asm volatile("{\n\t.reg .pred q;\n\t"
						             "setp.ne.b32 q, %4, 0;\n\t"
						             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n\t}"
						             :: "r"(tmem), "l"(sw128(a0 + 32 * ks)), "l"(sw128(b0 + 32 * ks)), "r"(p.idesc), "r"(acc)
						             : "memory");
					}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
					             :: "r"(mbar0 + 8 * b) : "memory");
				}
			}
			if (__syncthreads_or(tid == 0 && fail)) { fail = true; break; }
		}
		if (fail) break;
		/* epilogue: the last chunk's MMAs complete the accumulator */
		const uint32_t gl = g - 1;
		const bool done = bar_wait(mbar0 + 8 * (gl & 1), (gl >> 1) & 1);
		if (__syncthreads_or(!done)) { fail = true; break; }
		tc_fence_after();
		const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16);
		for (int c0 = 0; c0 < p.np; c0 += 16) {
			float acc[16];
			ld16(ta + (uint32_t)c0, acc);
			if (vin) {
				#pragma unroll
				for (int j = 0; j < 16; j++) {
					const int co = c0 + j;
					if (co >= p.cout) break;
					float val = acc[j] + (p.bias ? __ldg(p.bias + co) : 0.0f);
					if (p.relu) val = fmaxf(val, 0.0f);
					const int64_t o = (int64_t)co * p.V + v;
					if (p.residual) val += get((const TO *)p.residual, o);
					put((TO *)p.out, o, val);
				}
			}
		}
		tc_fence_before();
		__syncthreads();
	}
	if (fail && tid == 0) {
		atomicExch(&g_unet_tc_error, 1u);
		/* bounded drain of this CTA's copies and tensor operations in flight */
		for (int b = 0; b < 2; b++)
			if (last_b[b] >= 0) {
				bar_wait(cbar0 + 8 * b, ((uint32_t)last_b[b] >> 1) & 1);
				bar_wait(mbar0 + 8 * b, ((uint32_t)last_b[b] >> 1) & 1);
			}
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(tcols) : "memory");
}

/* ------------------------------ TMA form ------------------------------ */

constexpr int TS = 4;                    /* stages in the ring */
constexpr int STEP_A = TCM * 32;         /* one K = 16 step of A: 128 rows x 32 B */

struct ConvTma {
	const uint8_t *bk;       /* [K step][np rows][32 B], 32-byte swizzled */
	const float   *bias;
	const void    *residual;
	void          *out;
	int32_t        cout, np, cg, ksteps, nch;   /* cg = cin_p / 16 */
	int32_t        W, H;
	int64_t        V;
	int32_t        relu, tiles;
	uint32_t       idesc;
};

/* K-major operand in 32-byte swizzled atoms (8 rows x 32 B, SBO 256 B; the
 * leading offset is unused when one MMA's K spans one atom), version 1 */
__device__ __forceinline__ uint64_t sw32(uint32_t addr)
{
	uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
	d |= (uint64_t)1 << 16;
	d |= (uint64_t)(256 >> 4) << 32;
	d |= (uint64_t)1 << 46;
	d |= (uint64_t)6 << 61;
	return d;
}

/* bounded wait that also gives up when another role of the CTA has given up;
 * the role whose own wait runs out records the error */
__device__ __forceinline__ bool wait_role(uint32_t bar, uint32_t parity, volatile int *abort_flag)
{
	const long long t0 = clock64();
	while (true) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if (*abort_flag) return false;
		if (clock64() - t0 > TC_WAIT) {
			*abort_flag = 1;
			atomicExch(&g_unet_tc_error, 1u);
			return false;
		}
	}
}

/* B steps: element (n, kk) of K step ks (tap = ks / cg, ci = (ks % cg) * 16 + kk) at
 * (ks * np + n) * 32 + ((kk / 8) ^ ((n / 4) % 2)) * 16 + (kk % 8) * 2 bytes; zero beyond
 * cout, cin and the 27 taps */
__global__ void __launch_bounds__(256)
prepare_weights_tma(const __nv_bfloat16 *__restrict__ w, uint16_t *__restrict__ bk, int cin, int cg, int cout, int np,
                    int steps)
{
	const int64_t total = (int64_t)steps * np * 16;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
		const int kk = (int)(i & 15);
		const int64_t r = i >> 4;
		const int n = (int)(r % np), ks = (int)(r / np);
		const int tap = ks / cg, ci = (ks - tap * cg) * 16 + kk;
		uint16_t v = 0;
		if (n < cout && ci < cin && tap < 27) v = __bfloat16_as_ushort(w[((int64_t)n * cin + ci) * 27 + tap]);
		bk[((int64_t)ks * np + n) * 16 + ((((kk >> 3) ^ ((n >> 2) & 1))) << 3) + (kk & 7)] = v;
	}
}

__device__ __forceinline__ uint32_t bf16_bits(const uint16_t *p, int64_t i) { return __ldg(p + i); }
__device__ __forceinline__ uint32_t bf16_bits(const float *p, int64_t i)
{
	return __bfloat16_as_ushort(__float2bfloat16_rn(__ldg(p + i)));
}

/* channels-first [cin][V] (BF16, or FP32 rounded to BF16) -> channels-last
 * [V][cg * 16] BF16 (channels beyond cin are 0); thread per (voxel, 16-channel
 * block): 16 coalesced loads, one 32-byte store */
template <typename TI>
__global__ void __launch_bounds__(256)
to_channels_last(const TI *__restrict__ in, uint4 *__restrict__ out, int cin, int cg, int64_t V)
{
	const int b = blockIdx.y;
	for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
		uint32_t w[8];
		#pragma unroll
		for (int k = 0; k < 16; k += 2) {
			const int c0 = b * 16 + k;
			const uint32_t lo = c0 < cin ? bf16_bits(in, (int64_t)c0 * V + v) : 0u;
			const uint32_t hi = c0 + 1 < cin ? bf16_bits(in, (int64_t)(c0 + 1) * V + v) : 0u;
			w[k >> 1] = lo | (hi << 16);
		}
		uint4 *o = out + (v * cg + b) * 2;
		o[0] = make_uint4(w[0], w[1], w[2], w[3]);
		o[1] = make_uint4(w[4], w[5], w[6], w[7]);
	}
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c, int x, int y, int z, uint32_t bar)
{
	asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
	             " [%0], [%1, {%2, %3, %4, %5}], [%6];"
	             :: "r"(dst), "l"((uint64_t)map), "r"(c), "r"(x), "r"(y), "r"(z), "r"(bar) : "memory");
}

/* 192 threads: warp 0 loads, warp 1 issues the MMAs (and owns tensor memory),
 * warps 2-5 run the epilogue (warp w reads accumulator lanes 32 (w % 4) ...). */
template <typename TO>
__global__ void __launch_bounds__(192, 1)
conv3d_tma(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ ConvTma p)
{
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	const int bstep = p.np * 32, bchunk = 4 * bstep, stage = 4 * STEP_A + bchunk;
	uint64_t *bars = (uint64_t *)(sm + TS * stage);   /* full[TS], empty[TS], acc_full[2], acc_empty[2] */
	__shared__ uint32_t tmem_slot;
	__shared__ int abort_word;
	volatile int *abort_flag = &abort_word;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t full0 = su32(bars), empty0 = full0 + 8 * TS, afull0 = empty0 + 8 * TS, aempty0 = afull0 + 16;
	const uint32_t tcols = 2 * p.np <= 32 ? 32u : 2 * p.np <= 64 ? 64u : 2 * p.np <= 128 ? 128u : 256u;
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		             :: "r"(su32(&tmem_slot)), "r"(tcols) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0) {
		for (int i = 0; i < 2 * TS + 2; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(full0 + 8 * i), "r"(1) : "memory");
		for (int i = 0; i < 2; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(aempty0 + 8 * i), "r"(4) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		abort_word = 0;
		asm volatile("prefetch.tensormap [%0];" :: "l"((uint64_t)&xmap) : "memory");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;
	const int64_t plane = (int64_t)p.H * p.W;
	uint32_t issued = 0;                 /* chunks loaded (warp 0, lane 0) */
	int64_t mma_chunks = 0;              /* chunks whose MMAs were committed (warp 1, lane 0) */

	if (warp == 0) {
		if (lane == 0) {
			uint32_t q = 0;
			for (int tile = blockIdx.x; tile < p.tiles && !*abort_flag; tile += gridDim.x) {
				const int64_t v0 = (int64_t)tile * TCM;
				const int x0 = (int)(v0 % p.W), y0 = (int)((v0 / p.W) % p.H), z0 = (int)(v0 / plane);
				int tap = 0, c16 = 0;
				for (int c = 0; c < p.nch; c++, q++) {
					const int s = (int)(q % TS);
					const uint32_t u = q / TS;
					if (u > 0 && !wait_role(empty0 + 8 * s, (u - 1) & 1, abort_flag)) break;
					if (*abort_flag) break;
					const int steps = min(4, p.ksteps - 4 * c);
					const uint32_t fb = full0 + 8 * s, st = su32(sm + s * stage);
					asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
					             :: "r"(fb), "r"(steps * STEP_A + bchunk) : "memory");
					for (int j = 0; j < steps; j++) {
						tma_load_4d(st + j * STEP_A, &xmap, c16 * 16, x0 + tap % 3 - 1, y0 + (tap / 3) % 3 - 1,
						            z0 + tap / 9 - 1, fb);
						if (++c16 == p.cg) { c16 = 0; tap++; }
					}
					asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
					             :: "r"(st + 4 * STEP_A), "l"(p.bk + (size_t)c * bchunk), "r"(bchunk), "r"(fb)
					             : "memory");
					issued = q + 1;
				}
			}
		}
		__syncwarp();
	} else if (warp == 1) {
		if (lane == 0) {
			uint32_t q = 0, i = 0;
			bool stop = false;
			for (int tile = blockIdx.x; tile < p.tiles && !stop; tile += gridDim.x, i++) {
				const uint32_t a = i & 1, ua = i >> 1;
				if (ua > 0 && !wait_role(aempty0 + 8 * a, (ua - 1) & 1, abort_flag)) break;
				tc_fence_after();
				const uint32_t acc_t = tmem + a * (uint32_t)p.np;
				for (int c = 0; c < p.nch; c++, q++) {
					const int s = (int)(q % TS);
					if (!wait_role(full0 + 8 * s, (q / TS) & 1, abort_flag)) { stop = true; break; }
					tc_fence_after();
					const int steps = min(4, p.ksteps - 4 * c);
					const uint32_t a0 = su32(sm + s * stage), b0 = a0 + 4 * STEP_A;
					for (int j = 0; j < steps; j++) {
						const uint32_t acc = (c | j) != 0;
						asm volatile("{\n\t.reg .pred q;\n\t"
						             "setp.ne.b32 q, %4, 0;\n\t"
						             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n\t}"
						             :: "r"(acc_t), "l"(sw32(a0 + j * STEP_A)), "l"(sw32(b0 + j * bstep)), "r"(p.idesc),
						                "r"(acc)
						             : "memory");
					}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
					             :: "r"(empty0 + 8 * s) : "memory");
					mma_chunks = (int64_t)q + 1;
				}
				if (stop) break;
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
				             :: "r"(afull0 + 8 * a) : "memory");
			}
		}
		__syncwarp();
	} else {
		const int quarter = warp & 3;
		uint32_t i = 0;
		for (int tile = blockIdx.x; tile < p.tiles; tile += gridDim.x, i++) {
			const uint32_t a = i & 1, ua = i >> 1;
			int ok = 1;
			if (lane == 0) ok = wait_role(afull0 + 8 * a, ua & 1, abort_flag);
			if (!__shfl_sync(0xffffffffu, ok, 0)) break;
			tc_fence_after();
			const int64_t v = (int64_t)tile * TCM + quarter * 32 + lane;
			const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + a * (uint32_t)p.np;
			for (int c0 = 0; c0 < p.np; c0 += 16) {
				float acc[16];
				ld16(ta + (uint32_t)c0, acc);
				#pragma unroll
				for (int j = 0; j < 16; j++) {
					const int co = c0 + j;
					if (co >= p.cout) break;
					float val = acc[j] + (p.bias ? __ldg(p.bias + co) : 0.0f);
					if (p.relu) val = fmaxf(val, 0.0f);
					const int64_t o = (int64_t)co * p.V + v;
					if (p.residual) val += get((const TO *)p.residual, o);
					put((TO *)p.out, o, val);
				}
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(aempty0 + 8 * a) : "memory");
		}
	}
	__syncthreads();
	if (*abort_flag) {
		/* bounded drain of the loads and tensor operations still in flight */
		if (tid == 0)
			for (uint32_t q = issued > (uint32_t)TS ? issued - TS : 0u; q < issued; q++)
				bar_wait(full0 + 8 * (q % TS), (q / TS) & 1);
		if (tid == 32 && mma_chunks > 0) {
			const uint32_t q = (uint32_t)(mma_chunks - 1);
			bar_wait(empty0 + 8 * (q % TS), (q / TS) & 1);
		}
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 1)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(tcols) : "memory");
}

/* ------------------------------ slab form ------------------------------ */

constexpr int SLAB_ROWS = TCM + 2;               /* 128 positions and the x halo */
constexpr int SLAB_PLANE = SLAB_ROWS * 16;       /* one 8-channel plane of a slab: 2080 B */
constexpr int SLAB_MAX_STAGES = 8;
constexpr int SLAB_BARS = 256;                   /* barrier area ahead of the stages */

struct ConvSlab {
	const uint8_t *planes;   /* [G][PR][8] bf16: zero-padded channels-last planes */
	const uint8_t *bk;       /* [9 (dz, dy)][3 dx][G][np][8] bf16 */
	const float   *bias;
	const void    *residual;
	void          *out;
	int64_t        PR;       /* rows (positions) per plane */
	int64_t        V;
	int32_t        G, np, cout, stages, stage_bytes, a_bytes, b_bytes;
	int32_t        resident;  /* all 27 taps' weights (9 b_bytes) stay in shared memory, copied once */
	int32_t        W, H, D, Wp, Hp;
	int32_t        P0, tiles;
	int32_t        relu;
	uint32_t       idesc;
};

/* K-major operand without swizzling: core matrices of 8 rows x 16 B (rows 16 B
 * apart); SBO between core matrices along M (N), LBO between them along K;
 * descriptor version 1 */
__device__ __forceinline__ uint64_t interleaved(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
	uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

/* channels-first [cin][V] (BF16, or FP32 rounded to BF16) -> planes [G][PR][8]:
 * plane g holds channels 8 g ... 8 g + 7 of every position P of the volume
 * padded by one zero voxel on each face ((D + 2) x (H + 2) x (W + 2), x
 * fastest), positions beyond it zero. Block per (padded row, plane), threads
 * over the row's positions: 8 coalesced loads and one 16-byte store each (a
 * warp stores 512 contiguous bytes); the row arithmetic runs once per block. */
template <typename TI>
__global__ void __launch_bounds__(128)
to_padded_planes(const TI *__restrict__ in, uint4 *__restrict__ planes, int cin, int W, int H, int D, int64_t PR)
{
	const int g = blockIdx.y;
	const int Wp = W + 2, Hp = H + 2;
	const int64_t V = (int64_t)W * H * D, rows = PR / Wp;
	for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
		const int zp = (int)(row / Hp), yp = (int)(row - (int64_t)zp * Hp);
		const bool inner = zp >= 1 && zp <= D && yp >= 1 && yp <= H;
		const int64_t vrow = ((int64_t)(zp - 1) * H + (yp - 1)) * W - 1;    /* voxel of xp = 0 */
		uint4 *dst = planes + (int64_t)g * PR + row * Wp;
		for (int xp = threadIdx.x; xp < Wp; xp += blockDim.x) {
			uint32_t w[4] = {0u, 0u, 0u, 0u};
			if (inner && xp >= 1 && xp <= W) {
				const int64_t v = vrow + xp;
				#pragma unroll
				for (int k = 0; k < 8; k += 2) {
					const int c0 = g * 8 + k;
					const uint32_t lo = c0 < cin ? bf16_bits(in, (int64_t)c0 * V + v) : 0u;
					const uint32_t hi = c0 + 1 < cin ? bf16_bits(in, (int64_t)(c0 + 1) * V + v) : 0u;
					w[k >> 1] = lo | (hi << 16);
				}
			}
			dst[xp] = make_uint4(w[0], w[1], w[2], w[3]);
		}
	}
}

/* weights [9 (dz, dy)][3 dx][G][np][8]: element (n, channel 8 g + c) of tap
 * (dz, dy, dx); zero beyond cout and cin */
__global__ void __launch_bounds__(256)
prepare_weights_slab(const __nv_bfloat16 *__restrict__ w, uint16_t *__restrict__ bk, int cin, int G, int cout, int np)
{
	const int64_t total = (int64_t)27 * G * np * 8;
	for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
		const int c = (int)(i & 7);
		int64_t r = i >> 3;
		const int n = (int)(r % np);
		r /= np;
		const int g = (int)(r % G);
		const int tap = (int)(r / G);          /* (dz, dy) * 3 + dx = the tap index */
		const int ci = g * 8 + c;
		uint16_t v = 0;
		if (n < cout && ci < cin) v = __bfloat16_as_ushort(w[((int64_t)n * cin + ci) * 27 + tap]);
		bk[i] = v;
	}
}

/* 192 threads: warp 0 loads, warp 1 issues the MMAs (and owns tensor memory),
 * warps 2-5 run the epilogue. One stage is one (dz, dy) slab of a tile: per
 * 8-channel plane the 130 consecutive padded positions from the tile's first
 * position + (dz, dy) offset - 1 (one bulk copy each), and the weights of the
 * three dx taps; the dx taps are the same rows read from offsets 0, 16 and 32 B. */
template <typename TO>
__global__ void __launch_bounds__(192, 1)
conv3d_slab(const __grid_constant__ ConvSlab p)
{
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	uint64_t *bars = (uint64_t *)sm;          /* full[8], empty[8], acc_full[2], acc_empty[2], weights */
	uint8_t *wres = sm + SLAB_BARS;                         /* resident weights (p.resident) */
	uint8_t *stages = wres + (p.resident ? 9 * p.b_bytes : 0);
	__shared__ uint32_t tmem_slot;
	__shared__ int abort_word;
	volatile int *abort_flag = &abort_word;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int S = p.stages;
	const uint32_t full0 = su32(bars), empty0 = full0 + 8 * SLAB_MAX_STAGES, afull0 = empty0 + 8 * SLAB_MAX_STAGES,
	               aempty0 = afull0 + 16, wbar = aempty0 + 16;
	const uint32_t tcols = 2 * p.np <= 32 ? 32u : 2 * p.np <= 64 ? 64u : 2 * p.np <= 128 ? 128u : 256u;
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		             :: "r"(su32(&tmem_slot)), "r"(tcols) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0) {
		for (int i = 0; i < 2 * SLAB_MAX_STAGES + 2; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(full0 + 8 * i), "r"(1) : "memory");
		for (int i = 0; i < 2; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(aempty0 + 8 * i), "r"(4) : "memory");
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(wbar), "r"(1) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		abort_word = 0;
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;
	const uint32_t hw32 = (uint32_t)p.Hp * (uint32_t)p.Wp;
	if (tid == 0 && p.resident) {
		const uint32_t wb = (uint32_t)(9 * p.b_bytes);
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(wbar), "r"(wb) : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		             :: "r"(su32(wres)), "l"(p.bk), "r"(wb), "r"(wbar) : "memory");
	}
	uint32_t issued = 0;
	int64_t mma_chunks = 0;

	if (warp == 0) {
		if (lane == 0) {
			uint32_t q = 0;
			for (int tile = blockIdx.x; tile < p.tiles && !*abort_flag; tile += gridDim.x) {
				const int64_t first = (int64_t)p.P0 + (int64_t)tile * TCM - 1;
				for (int sl = 0; sl < 9; sl++, q++) {
					const int s = (int)(q % S);
					const uint32_t u = q / S;
					if (u > 0 && !wait_role(empty0 + 8 * s, (u - 1) & 1, abort_flag)) break;
					if (*abort_flag) break;
					const int64_t start = first + ((int64_t)(sl / 3 - 1) * p.Hp + (sl % 3 - 1)) * p.Wp;
					const uint32_t fb = full0 + 8 * s, st = su32(stages + (size_t)s * p.stage_bytes);
					asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
					             :: "r"(fb), "r"(p.a_bytes + (p.resident ? 0 : p.b_bytes)) : "memory");
					for (int g = 0; g < p.G; g++)
						asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
						             :: "r"(st + g * SLAB_PLANE), "l"(p.planes + ((int64_t)g * p.PR + start) * 16),
						                "r"(SLAB_PLANE), "r"(fb)
						             : "memory");
					if (!p.resident)
						asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
						             :: "r"(st + p.a_bytes), "l"(p.bk + (size_t)sl * p.b_bytes), "r"(p.b_bytes), "r"(fb)
						             : "memory");
					issued = q + 1;
				}
			}
		}
		__syncwarp();
	} else if (warp == 1) {
		if (lane == 0) {
			uint32_t q = 0, i = 0;
			bool stop = false;
			const uint32_t bplane = (uint32_t)p.np * 16;
			if (p.resident && !wait_role(wbar, 0, abort_flag)) stop = true;
			for (int tile = blockIdx.x; tile < p.tiles && !stop; tile += gridDim.x, i++) {
				const uint32_t a = i & 1, ua = i >> 1;
				if (ua > 0 && !wait_role(aempty0 + 8 * a, (ua - 1) & 1, abort_flag)) break;
				tc_fence_after();
				const uint32_t acc_t = tmem + a * (uint32_t)p.np;
				for (int sl = 0; sl < 9; sl++, q++) {
					const int s = (int)(q % S);
					if (!wait_role(full0 + 8 * s, (q / S) & 1, abort_flag)) { stop = true; break; }
					tc_fence_after();
					const uint32_t a0 = su32(stages + (size_t)s * p.stage_bytes);
					const uint32_t b0 = p.resident ? su32(wres) + (uint32_t)(sl * p.b_bytes) : a0 + (uint32_t)p.a_bytes;
					/* the descriptors of one stage differ only in their start field (16-byte
					 * units, bits 0-13; shared addresses stay below 2^18): built once, offset per MMA */
					const uint64_t da0 = interleaved(a0, SLAB_PLANE, 128), db0 = interleaved(b0, bplane, 128);
					for (int dx = 0; dx < 3; dx++)
						for (int j = 0; j < p.G; j += 2) {
							const uint32_t acc = (sl | dx | j) != 0;
							const uint64_t da = da0 + (uint64_t)((uint32_t)(j * SLAB_PLANE + dx * 16) >> 4);
							const uint64_t db = db0 + (uint64_t)(((uint32_t)(dx * p.G + j) * bplane) >> 4);
							asm volatile("{\n\t.reg .pred q;\n\t"
							             "setp.ne.b32 q, %4, 0;\n\t"
							             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n\t}"
							             :: "r"(acc_t), "l"(da), "l"(db), "r"(p.idesc), "r"(acc) : "memory");
						}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
					             :: "r"(empty0 + 8 * s) : "memory");
					mma_chunks = (int64_t)q + 1;
				}
				if (stop) break;
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
				             :: "r"(afull0 + 8 * a) : "memory");
			}
		}
		__syncwarp();
	} else {
		const int quarter = warp & 3;
		uint32_t i = 0;
		for (int tile = blockIdx.x; tile < p.tiles; tile += gridDim.x, i++) {
			const uint32_t a = i & 1, ua = i >> 1;
			int ok = 1;
			if (lane == 0) ok = wait_role(afull0 + 8 * a, ua & 1, abort_flag);
			if (!__shfl_sync(0xffffffffu, ok, 0)) break;
			tc_fence_after();
			/* positions are below 2^31 (checked on the host): 32-bit division */
			const uint32_t P = (uint32_t)p.P0 + (uint32_t)tile * TCM + quarter * 32 + lane;
			const uint32_t zp = P / hw32, rem = P - zp * hw32;
			const uint32_t yp = rem / (uint32_t)p.Wp, xp = rem - yp * (uint32_t)p.Wp;
			const bool inside = zp >= 1 && zp <= (uint32_t)p.D && yp >= 1 && yp <= (uint32_t)p.H && xp >= 1 &&
			                    xp <= (uint32_t)p.W;
			const int64_t v = ((int64_t)(zp - 1) * p.H + (yp - 1)) * (int64_t)p.W + (xp - 1);
			const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + a * (uint32_t)p.np;
			for (int c0 = 0; c0 < p.np; c0 += 16) {
				float acc[16];
				ld16(ta + (uint32_t)c0, acc);
				if (inside) {
					#pragma unroll
					for (int j = 0; j < 16; j++) {
						const int co = c0 + j;
						if (co >= p.cout) break;
						float val = acc[j] + (p.bias ? __ldg(p.bias + co) : 0.0f);
						if (p.relu) val = fmaxf(val, 0.0f);
						const int64_t o = (int64_t)co * p.V + v;
						if (p.residual) val += get((const TO *)p.residual, o);
						put((TO *)p.out, o, val);
					}
				}
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(aempty0 + 8 * a) : "memory");
		}
	}
	__syncthreads();
	if (*abort_flag) {
		if (tid == 0) {
			if (p.resident) bar_wait(wbar, 0);
			for (uint32_t q = issued > (uint32_t)S ? issued - S : 0u; q < issued; q++)
				bar_wait(full0 + 8 * (q % S), (q / S) & 1);
		}
		if (tid == 32 && mma_chunks > 0) {
			const uint32_t q = (uint32_t)(mma_chunks - 1);
			bar_wait(empty0 + 8 * (q % S), (q / S) & 1);
		}
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 1)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(tcols) : "memory");
}

std::mutex g_bk_lock;
uint16_t *g_bk = nullptr;
size_t g_bk_bytes = 0;
uint8_t *g_cl = nullptr;
size_t g_cl_bytes = 0;

/* grows *buf to at least `bytes` (cudaFree synchronises: no earlier launch still reads it) */
cudaError_t grow(uint8_t **buf, size_t *have, size_t bytes)
{
	if (bytes <= *have) return cudaSuccess;
	cudaFree(*buf);
	*buf = nullptr;
	*have = 0;
	const cudaError_t e = cudaMalloc((void **)buf, bytes);
	if (e == cudaSuccess) *have = bytes;
	return e;
}

/* rows of the volume tile by 128 voxels, so every 128-voxel tile is one TMA box */
bool tma_geometry(const int32_t dims[3])
{
	const int W = dims[0], H = dims[1];
	if (W <= 0 || H <= 0 || dims[2] <= 0) return false;
	if (W <= TCM) return TCM % W == 0 && H % (TCM / W) == 0;
	return W % TCM == 0;
}

/* resident CTAs per SM for `smem` bytes of dynamic shared memory, 192 threads and
 * `tcols` tensor-memory columns held for the CTA's whole life */
cudaError_t resident_ctas(size_t smem, int tcols, int &occ)
{
	int dev = 0, sm_bytes = 0, reserved = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
	if (e != cudaSuccess) return e;
	occ = sm_bytes / (int)(smem + (size_t)reserved + 64);
	occ = std::max(1, std::min({occ, 2048 / 192, 512 / tcols}));
	return cudaSuccess;
}

bool conv3d_tma_launch(const void *in, int in_type, int cin, const uint16_t *w, const float *bias, const void *residual, void *out,
                       int out_type, int cout, const int32_t dims[3], int relu, cudaStream_t s, cudaError_t &err)
{
	const auto enc = (PFN_cuTensorMapEncodeTiled_v12000)tensor_map_encoder();
	if (!enc) return false;
	const int cg = (cin + 15) / 16, np = (cout + 15) / 16 * 16;
	if (np > 128 || cg > 32) return false;
	const int ksteps = 27 * cg, nch = (ksteps + 3) / 4;
	const int64_t V = (int64_t)dims[0] * dims[1] * dims[2];
	ConvTma p{};
	std::lock_guard<std::mutex> hold(g_bk_lock);
	if ((err = grow((uint8_t **)&g_bk, &g_bk_bytes, (size_t)nch * 4 * np * 32)) != cudaSuccess) return true;
	if ((err = grow(&g_cl, &g_cl_bytes, (size_t)V * cg * 32)) != cudaSuccess) return true;
	CUtensorMap xmap;
	const cuuint64_t gdim[4] = {(cuuint64_t)cg * 16, (cuuint64_t)dims[0], (cuuint64_t)dims[1], (cuuint64_t)dims[2]};
	const cuuint64_t gstr[3] = {(cuuint64_t)cg * 32, (cuuint64_t)cg * 32 * dims[0],
	                            (cuuint64_t)cg * 32 * dims[0] * dims[1]};
	const cuuint32_t box[4] = {16, (cuuint32_t)std::min(dims[0], TCM), (cuuint32_t)std::max(1, TCM / dims[0]), 1};
	const cuuint32_t estr[4] = {1, 1, 1, 1};
	if (enc(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, g_cl, gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
	        CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
	    CUDA_SUCCESS)
		return false;
	const int64_t wtotal = (int64_t)nch * 4 * np * 16;
	prepare_weights_tma<<<(int)std::min<int64_t>((wtotal + 255) / 256, 1024), 256, 0, s>>>(
	    (const __nv_bfloat16 *)w, g_bk, cin, cg, cout, np, nch * 4);
	g_kernel_launches++;
	if ((err = cudaGetLastError()) != cudaSuccess) return true;
	const dim3 cgrid((unsigned)std::min<int64_t>((V + 255) / 256, (int64_t)device_sm_count() * 16), (unsigned)cg);
	if (in_type == BF_UNET_F32) to_channels_last<<<cgrid, 256, 0, s>>>((const float *)in, (uint4 *)g_cl, cin, cg, V);
	else                        to_channels_last<<<cgrid, 256, 0, s>>>((const uint16_t *)in, (uint4 *)g_cl, cin, cg, V);
	g_kernel_launches++;
	if ((err = cudaGetLastError()) != cudaSuccess) return true;
	p.bk = (const uint8_t *)g_bk;
	p.bias = bias;
	p.residual = residual;
	p.out = out;
	p.cout = cout;
	p.np = np;
	p.cg = cg;
	p.ksteps = ksteps;
	p.nch = nch;
	p.W = dims[0];
	p.H = dims[1];
	p.V = V;
	p.relu = relu;
	p.tiles = (int)(V / TCM);
	p.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(np >> 3) << 17) | ((uint32_t)(TCM >> 4) << 24);
	const size_t smem = 1024 + (size_t)TS * (4 * STEP_A + 4 * np * 32) + (2 * TS + 4) * 8;
	const void *fn = out_type == BF_UNET_F32 ? (const void *)conv3d_tma<float> : (const void *)conv3d_tma<__nv_bfloat16>;
	if ((err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
		return true;
	const int tcols = 2 * np <= 32 ? 32 : 2 * np <= 64 ? 64 : 2 * np <= 128 ? 128 : 256;
	int occ = 1;
	if ((err = resident_ctas(smem, tcols, occ)) != cudaSuccess) return true;
	const int grid = (int)std::min<int64_t>(p.tiles, (int64_t)device_sm_count() * occ);
	if (out_type == BF_UNET_F32) conv3d_tma<float><<<grid, 192, smem, s>>>(xmap, p);
	else                         conv3d_tma<__nv_bfloat16><<<grid, 192, smem, s>>>(xmap, p);
	g_kernel_launches++;
	err = cudaGetLastError();
	return true;
}

bool conv3d_slab_launch(const void *in, int in_type, int cin, const uint16_t *w, const float *bias, const void *residual,
                        void *out, int out_type, int cout, const int32_t dims[3], int relu, cudaStream_t s,
                        cudaError_t &err)
{
	const int G = (cin + 15) / 16 * 2, np = (cout + 15) / 16 * 16;
	if (np > 128) return false;
	const int W = dims[0], H = dims[1], D = dims[2];
	const int64_t Wp = W + 2, Hp = H + 2;
	/* whole padded rows, at least 256 positions past the volume (a tile's last
	 * slab may read up to 127 + 2 positions beyond it) */
	const int64_t PR = ((D + 2) * Hp + (256 + Wp - 1) / Wp) * Wp;
	if (PR > INT32_MAX) return false;
	ConvSlab p{};
	p.a_bytes = G * SLAB_PLANE;
	p.b_bytes = 3 * G * np * 16;
	/* the weights stay resident when they take at most 48 KB (the full-resolution
	 * layers); otherwise each stage carries its slab's three taps */
	p.resident = 9 * p.b_bytes <= 48 * 1024;
	p.stage_bytes = (p.a_bytes + (p.resident ? 0 : p.b_bytes) + 127) / 128 * 128;
	if (p.stage_bytes > 100 * 1024) return false;
	const int wres_bytes = p.resident ? 9 * p.b_bytes : 0;
	p.stages = std::max(2, std::min(SLAB_MAX_STAGES, (112 * 1024 - wres_bytes) / p.stage_bytes));
	std::lock_guard<std::mutex> hold(g_bk_lock);
	if ((err = grow((uint8_t **)&g_bk, &g_bk_bytes, (size_t)p.b_bytes * 9)) != cudaSuccess) return true;
	if ((err = grow(&g_cl, &g_cl_bytes, (size_t)G * PR * 16)) != cudaSuccess) return true;
	const int64_t wtotal = (int64_t)27 * G * np * 8;
	prepare_weights_slab<<<(int)std::min<int64_t>((wtotal + 255) / 256, 1024), 256, 0, s>>>(
	    (const __nv_bfloat16 *)w, g_bk, cin, G, cout, np);
	g_kernel_launches++;
	if ((err = cudaGetLastError()) != cudaSuccess) return true;
	const dim3 cgrid((unsigned)std::min<int64_t>(PR / Wp, (int64_t)device_sm_count() * 32), (unsigned)G);
	const int cthreads = Wp >= 128 ? 128 : (int)(Wp + 31) / 32 * 32;
	if (in_type == BF_UNET_F32)
		to_padded_planes<<<cgrid, cthreads, 0, s>>>((const float *)in, (uint4 *)g_cl, cin, W, H, D, PR);
	else
		to_padded_planes<<<cgrid, cthreads, 0, s>>>((const uint16_t *)in, (uint4 *)g_cl, cin, W, H, D, PR);
	g_kernel_launches++;
	if ((err = cudaGetLastError()) != cudaSuccess) return true;
	p.planes = g_cl;
	p.bk = (const uint8_t *)g_bk;
	p.bias = bias;
	p.residual = residual;
	p.out = out;
	p.PR = PR;
	p.V = (int64_t)W * H * D;
	p.G = G;
	p.np = np;
	p.cout = cout;
	p.W = W;
	p.H = H;
	p.D = D;
	p.Wp = (int32_t)Wp;
	p.Hp = (int32_t)Hp;
	p.P0 = (int32_t)((Hp + 1) * Wp + 1);
	const int64_t P1 = ((int64_t)D * Hp + H) * Wp + W;
	p.tiles = (int32_t)((P1 - p.P0 + TCM) / TCM);
	p.relu = relu;
	p.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(np >> 3) << 17) | ((uint32_t)(TCM >> 4) << 24);
	const size_t smem = 1024 + SLAB_BARS + (size_t)wres_bytes + (size_t)p.stages * p.stage_bytes;
	const void *fn = out_type == BF_UNET_F32 ? (const void *)conv3d_slab<float> : (const void *)conv3d_slab<__nv_bfloat16>;
	if ((err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
		return true;
	const int tcols = 2 * np <= 32 ? 32 : 2 * np <= 64 ? 64 : 2 * np <= 128 ? 128 : 256;
	int occ = 1;
	if ((err = resident_ctas(smem, tcols, occ)) != cudaSuccess) return true;
	const int grid = (int)std::min<int64_t>(p.tiles, (int64_t)device_sm_count() * occ);
	if (out_type == BF_UNET_F32) conv3d_slab<float><<<grid, 192, smem, s>>>(p);
	else                         conv3d_slab<__nv_bfloat16><<<grid, 192, smem, s>>>(p);
	g_kernel_launches++;
	err = cudaGetLastError();
	return true;
}

} /* namespace */

/* true when a tensor-core form was launched (err: its launch status); false to
 * fall back to the direct kernel. BF16 inputs run on either form, FP32 inputs
 * (rounded to BF16) on the TMA form only. */
bool conv3d_tc_launch(const void *in, int in_type, int cin, const uint16_t *w, const float *bias, const void *residual, void *out,
                      int out_type, int cout, const int32_t dims[3], int relu, cudaStream_t s, cudaError_t &err)
{
	const char *env = std::getenv("OGL_BF_UNET_SIMT");
	if (env && env[0] == '1') return false;
	/* OGL_BF_UNET_TC selects a form: slab (the default), tma (volumes whose rows
	 * tile by 128 voxels) or gather (BF16 inputs) */
	const char *form = std::getenv("OGL_BF_UNET_TC");
	const bool gather_only = form && std::strcmp(form, "gather") == 0;
	const bool tma = form && std::strcmp(form, "tma") == 0;
	if (!gather_only && !tma &&
	    conv3d_slab_launch(in, in_type, cin, w, bias, residual, out, out_type, cout, dims, relu, s, err))
		return true;
	if (tma && tma_geometry(dims) &&
	    conv3d_tma_launch(in, in_type, cin, w, bias, residual, out, out_type, cout, dims, relu, s, err))
		return true;
	if (in_type != BF_UNET_BF16) return false;
	const int cin_p = (cin + 7) / 8 * 8, np = (cout + 15) / 16 * 16;
	if (np > 128 || cin_p > 512) return false;
	const int nch = (27 * cin_p + TCK - 1) / TCK;
	const size_t bk_bytes = (size_t)nch * np * 128;
	ConvTc p{};
	std::lock_guard<std::mutex> hold(g_bk_lock);
	if ((err = grow((uint8_t **)&g_bk, &g_bk_bytes, bk_bytes)) != cudaSuccess) return true;
	p.bk = (const uint8_t *)g_bk;
	const int64_t total = (int64_t)nch * np * TCK;
	prepare_weights_tc<<<(int)std::min<int64_t>((total + 255) / 256, 1024), 256, 0, s>>>(
	    (const __nv_bfloat16 *)w, g_bk, cin, cin_p, cout, np, nch);
	g_kernel_launches++;
	if ((err = cudaGetLastError()) != cudaSuccess) return true;
	p.in = (const __nv_bfloat16 *)in;
	p.bias = bias;
	p.residual = residual;
	p.out = out;
	p.cin = cin;
	p.cin_p = cin_p;
	p.cout = cout;
	p.np = np;
	p.nch = nch;
	p.W = dims[0];
	p.H = dims[1];
	p.D = dims[2];
	p.V = (int64_t)dims[0] * dims[1] * dims[2];
	p.relu = relu;
	p.tiles = (int)((p.V + TCM - 1) / TCM);
	/* D = f32 (bit 4), A and B bf16 (bits 7 and 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24 */
	p.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(np >> 3) << 17) | ((uint32_t)(TCM >> 4) << 24);
	const size_t smem = 1024 + 2 * (size_t)A_BYTES + 2 * (size_t)np * 128 + 4 * 8;
	const void *fn = out_type == BF_UNET_F32 ? (const void *)conv3d_tc<float> : (const void *)conv3d_tc<__nv_bfloat16>;
	if ((err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
		return true;
	const int grid = (int)std::min<int64_t>(p.tiles, (int64_t)device_sm_count() * 4);
	if (out_type == BF_UNET_F32) conv3d_tc<float><<<grid, 128, smem, s>>>(p);
	else                         conv3d_tc<__nv_bfloat16><<<grid, 128, smem, s>>>(p);
	g_kernel_launches++;
	err = cudaGetLastError();
	return true;
}

} /* namespace bf */

extern "C" uint32_t bf_unet_tc_errors(void *stream)
{
	unsigned e = 0;
	if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return 1;
	if (cudaMemcpyFromSymbol(&e, bf::g_unet_tc_error, sizeof(e)) != cudaSuccess) return 1;
	if (e) {
		const unsigned zero = 0;
		cudaMemcpyToSymbol(bf::g_unet_tc_error, &zero, sizeof(zero));
	}
	return e;
}
