/*
 * bf_das_batch.cu -- delay-and-sum of many acquisitions in one persistent launch
 * (the batched variant; no counterpart in the reference, which beamforms one
 * acquisition per compute).
 *
 * The acquisitions of a batch may differ in transmit count, sample count,
 * output grid and DAS mode. Their voxel tiles form one work list, ordered by
 * estimated cost (largest first); a grid of a few CTAs per SM takes tiles from
 * it with an atomic counter until it is empty, so small planes run beside large
 * volumes and no SM idles while work remains. A CTA copies the parameters of its
 * tile's acquisition into shared memory and runs the same per-tile code as the
 * single-acquisition kernels: the HERCULES fast path (bf_das_hercules.cuh) with
 * volume or plane tiles, or the general path (bf_das_generic.cuh) for FORCES.
 * Every voxel of every acquisition is written once, in the same arithmetic and
 * accumulation order as the single-acquisition launch.
 */
#include "bf_kernels.h"
#include "bf_das_math.cuh"
#include "bf_das_generic.cuh"
#include "bf_das_hercules.cuh"

namespace bf {

template <int INTERP>
__global__ void __launch_bounds__(DAS_THREADS, 6)
das_batch(const DasBatchAcq *__restrict__ acq, const int4 *__restrict__ items, int n_items, int *next)
{
	__shared__ DasParams sp;
	__shared__ const float4 *stab;
	__shared__ int spath, sitem, sacq;
	if (threadIdx.x == 0) sacq = -1;
	constexpr int WORDS = (int)(sizeof(DasParams) / 4);
	while (true) {
		__syncthreads();                        /* the previous tile is done with sp and sitem */
		if (threadIdx.x == 0) sitem = atomicAdd(next, 1);
		__syncthreads();
		const int it = sitem;
		if (it >= n_items) return;              /* uniform over the CTA */
		const int4 w = __ldg(items + it);
		if (w.x != sacq) {
			__syncthreads();                    /* every thread has read sacq */
			const uint32_t *src = (const uint32_t *)&acq[w.x].p;
			for (int k = threadIdx.x; k < WORDS; k += blockDim.x) ((uint32_t *)&sp)[k] = __ldg(src + k);
			if (threadIdx.x == 0) {
				stab = acq[w.x].table;
				spath = acq[w.x].path;
				sacq = w.x;
			}
			__syncthreads();
		}
		const int path = spath;
		if (path == DAS_BATCH_HERC_VOLUME) {
			hercules_tile<INTERP, 4>(sp, stab, w.y, w.z, w.w, 0);
		} else if (path == DAS_BATCH_HERC_PLANE) {
			hercules_tile<INTERP, 1>(sp, stab, w.y, w.z, w.w, 0);
		} else {
			const int vx = w.y * DAS_TX + (int)(threadIdx.x & (DAS_TX - 1));
			const int vz = w.w * DAS_TZ + (int)(threadIdx.x / DAS_TX);
			const int vy = w.z;
			if (vx < sp.dims[0] && vz < sp.dims[2]) {
				const float2 v = das_voxel<DAS_FORCES, INTERP, true>(sp, vx, vy, vz, 0, sp.loop_end);
				sp.frame[((int64_t)vz * sp.dims[1] + vy) * sp.dims[0] + vx] = v;
			}
		}
	}
}

/* Tile grid of one acquisition on a path (see HercTile and das_kernel's 8 x 16). */
void das_batch_tiles(const DasParams &p, int path, int tiles[3])
{
	if (path == DAS_BATCH_HERC_VOLUME) {
		tiles[0] = (p.dims[0] + HercTile<4>::X - 1) / HercTile<4>::X;
		tiles[1] = (p.dims[1] + HercTile<4>::Y - 1) / HercTile<4>::Y;
		tiles[2] = (p.dims[2] + HercTile<4>::Z * HercTile<4>::NV - 1) / (HercTile<4>::Z * HercTile<4>::NV);
	} else if (path == DAS_BATCH_HERC_PLANE) {
		tiles[0] = (p.dims[0] + HercTile<1>::X - 1) / HercTile<1>::X;
		tiles[1] = p.dims[1];
		tiles[2] = (p.dims[2] + HercTile<1>::Z - 1) / HercTile<1>::Z;
	} else {
		tiles[0] = (p.dims[0] + DAS_TX - 1) / DAS_TX;
		tiles[1] = p.dims[1];
		tiles[2] = (p.dims[2] + DAS_TZ - 1) / DAS_TZ;
	}
}

cudaError_t launch_das_batch(const DasBatchAcq *acq, const int4 *items, int n_items, int *counter, int interp,
                             int ctas, cudaStream_t s)
{
	if (n_items <= 0) return cudaSuccess;
	cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
	if (e != cudaSuccess) return e;
	switch (interp) {
	case INTERP_CUBIC:  das_batch<INTERP_CUBIC><<<ctas, DAS_THREADS, 0, s>>>(acq, items, n_items, counter); break;
	case INTERP_LINEAR: das_batch<INTERP_LINEAR><<<ctas, DAS_THREADS, 0, s>>>(acq, items, n_items, counter); break;
	default:            das_batch<INTERP_NEAREST><<<ctas, DAS_THREADS, 0, s>>>(acq, items, n_items, counter); break;
	}
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
