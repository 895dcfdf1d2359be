/*
 * bf_das_batch.cu -- delay-and-sum of many acquisitions in one persistent launch
 * (the batched variant; no counterpart in the reference, which beamforms one
 * acquisition per compute).
 *
 * The acquisitions of a batch may differ in transmit count, sample count,
 * output grid and DAS mode. Their voxel tiles form one work list, ordered by
 * estimated cost (largest first); a grid of a few CTAs per SM takes tiles from
 * it with an atomic counter until it is empty, so small planes run beside large
 * volumes and no SM idles while work remains. The acquisitions' parameters travel
 * by value in the kernel's parameter space (up to DAS_BATCH_MAX per launch), so a
 * tile reads them through the constant cache as a single launch does, and runs
 * the same per-tile code as the single-acquisition kernels: the HERCULES fast
 * path (bf_das_hercules.cuh) with volume or plane tiles, or for FORCES the fast
 * path (bf_das_forces.cuh; the general path for nearest interpolation). The two paths are two persistent launches
 * with their own work lists, so each keeps its own register budget.
 * Every voxel of every acquisition is written once, in the same arithmetic and
 * accumulation order as the single-acquisition launch.
 */
#include "bf_kernels.h"
#include "bf_das_math.cuh"
#include "bf_das_generic.cuh"
#include "bf_das_hercules.cuh"
#include "bf_das_staged.cuh"
#include "bf_das_forces.cuh"

namespace bf {

/* GENERAL = false: HERCULES tiles (up to 80 registers, 6 CTAs per SM), from the
 * FP32 table (staged in shared memory, as das_hercules_staged, for acquisitions
 * marked `staged`; dynamic shared memory stg_smem_bytes) or, with H (DAS
 * precision 1), the FP16 table; true: tiles of the general path (FORCES),
 * compiled on their own (64 registers, 8 CTAs per SM) with their parameters
 * copied to registers per tile. */
template <int INTERP, bool GENERAL, bool H = false>
__global__ void __launch_bounds__(DAS_THREADS, GENERAL ? 8 : 6)
das_batch(const __grid_constant__ DasBatchArgs args, const int4 *__restrict__ items, int n_items, int *next)
{
	extern __shared__ __align__(128) uint8_t batch_smem[];
	__shared__ int sitem;
	while (true) {
		__syncthreads();                        /* every thread has read the previous item */
		if (threadIdx.x == 0) sitem = atomicAdd(next, 1);
		__syncthreads();
		const int it = sitem;
		if (it >= n_items) return;              /* uniform over the CTA */
		const int4 w = __ldg(items + it);
		const DasBatchAcq &a = args.acq[w.x];
		if (!GENERAL) {
			if constexpr (INTERP != INTERP_NEAREST && !H && DAS_THREADS == 128) {
				if (a.staged) {
					if (a.path == DAS_BATCH_HERC_VOLUME)
						hercules_tile_staged<INTERP, 4, false>(a.p, a.table, w.y, w.z, w.w, 0, batch_smem);
					else
						hercules_tile_staged<INTERP, 1, false>(a.p, a.table, w.y, w.z, w.w, 0, batch_smem);
					continue;
				}
			}
			if (a.path == DAS_BATCH_HERC_VOLUME) hercules_tile<INTERP, 4, DAS_THREADS, H>(a.p, a.table, w.y, w.z, w.w, 0);
			else                                 hercules_tile<INTERP, 1, DAS_THREADS, H>(a.p, a.table, w.y, w.z, w.w, 0);
		} else {
			const int vx = w.y * DAS_TX + (int)(threadIdx.x & (DAS_TX - 1));
			const int vz = w.w * DAS_TZ + (int)(threadIdx.x / DAS_TX);
			const int vy = w.z;
			/* a register copy: the loop then reads its constants from registers, not
			 * through a runtime-indexed parameter load per use */
			const DasParams p = a.p;
			if (vx < p.dims[0] && vz < p.dims[2]) {
				/* acquisitions with a table take the FORCES fast path */
				const float2 v = INTERP != INTERP_NEAREST && a.table
				                     ? forces_voxel<INTERP == INTERP_NEAREST ? INTERP_CUBIC : INTERP>(p, a.table, vx, vy, vz,
				                                                                                     0, p.loop_end)
				                     : das_voxel<DAS_FORCES, INTERP, true>(p, vx, vy, vz, 0, p.loop_end);
				p.frame[((int64_t)vz * p.dims[1] + vy) * p.dims[0] + vx] = v;
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

cudaError_t launch_das_batch(const DasBatchArgs &args, const int4 *items, int n_items, int *counter, int interp,
                             bool general, bool half, int ctas, cudaStream_t s)
{
	if (n_items <= 0) return cudaSuccess;
	for (int i = 0; i < DAS_BATCH_MAX; i++)
		if (args.acq[i].p.frame && args.acq[i].p.rx_step < 1) return cudaErrorInvalidValue;
	cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
	if (e != cudaSuccess) return e;
	/* shared memory of the staged tiles (volume and plane tiles stage the same windows) */
	const size_t stg = interp == INTERP_CUBIC ? stg_smem_bytes<INTERP_CUBIC, 4, false>()
	                   : interp == INTERP_LINEAR ? stg_smem_bytes<INTERP_LINEAR, 4, false>() : 0;
	static_assert(stg_smem_bytes<INTERP_CUBIC, 4, false>() == stg_smem_bytes<INTERP_CUBIC, 1, false>() &&
	              stg_smem_bytes<INTERP_LINEAR, 4, false>() == stg_smem_bytes<INTERP_LINEAR, 1, false>(),
	              "volume and plane tiles share one shared-memory size");
#define BF_BATCH(I) (general ? das_batch<I, true><<<ctas, DAS_THREADS, 0, s>>>(args, items, n_items, counter) \
                     : half  ? das_batch<I, false, true><<<ctas, DAS_THREADS, 0, s>>>(args, items, n_items, counter) \
                             : das_batch<I, false><<<ctas, DAS_THREADS, stg, s>>>(args, items, n_items, counter))
	switch (interp) {
	case INTERP_CUBIC:  BF_BATCH(INTERP_CUBIC); break;
	case INTERP_LINEAR: BF_BATCH(INTERP_LINEAR); break;
	default:            BF_BATCH(INTERP_NEAREST); break;
	}
#undef BF_BATCH
	g_kernel_launches++;
	return cudaGetLastError();
}

} /* namespace bf */
