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
 * Every wait is bounded (about one second); a wait that runs out sets the error
 * word (bf_unet_tc_errors), the CTA waits (bounded) for its copies and tensor
 * operations in flight, frees its tensor memory and stops.
 */
#include "bf_kernels.h"
#include "bf_unet.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
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

std::mutex g_bk_lock;
uint16_t *g_bk = nullptr;
size_t g_bk_bytes = 0;

} /* namespace */

/* true when the tensor-core form was launched (BF16 input); false to fall back */
bool conv3d_tc_launch(const void *in, int cin, const uint16_t *w, const float *bias, const void *residual, void *out,
                      int out_type, int cout, const int32_t dims[3], int relu, cudaStream_t s, cudaError_t &err)
{
	const char *env = std::getenv("OGL_BF_UNET_SIMT");
	if (env && env[0] == '1') return false;
	const int cin_p = (cin + 7) / 8 * 8, np = (cout + 15) / 16 * 16;
	if (np > 128 || cin_p > 512) return false;
	const int nch = (27 * cin_p + TCK - 1) / TCK;
	const size_t bk_bytes = (size_t)nch * np * 128;
	ConvTc p{};
	{
		std::lock_guard<std::mutex> hold(g_bk_lock);
		if (bk_bytes > g_bk_bytes) {
			cudaFree(g_bk);                      /* synchronises: no earlier launch still reads it */
			g_bk = nullptr;
			g_bk_bytes = 0;
			if ((err = cudaMalloc(&g_bk, bk_bytes)) != cudaSuccess) return true;
			g_bk_bytes = bk_bytes;
		}
		p.bk = (const uint8_t *)g_bk;
	}
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
