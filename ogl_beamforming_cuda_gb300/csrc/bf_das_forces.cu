/*
 * bf_das_forces.cu -- delay-and-sum for FORCES acquisitions, the fast path
 * (das.glsl:259-277, DAS_FAST; dispatched by beamformer.c:608-681).
 *
 * FORCES: per voxel q (transducer coordinates) and receive element r on the x
 * axis, the receive distance |(q.x - r px, q.z)| and the apodization of
 * q.x - r px are fixed for all transmits; per transmit t the distance to the
 * transmit centre (t px, floor(C / 2) py, 0) is fixed for all receive channels;
 * every (r, t) term with the receive apodization above 0 samples channel row
 * (r, t) at ((d_t + d_r) / c + t_off) fs.
 *
 * The general kernel (das_voxel) evaluates that chain with IEEE square roots and
 * divisions and four channel-data loads per cubic term. Here, as in the HERCULES
 * fast path, a voxel first proves that every square-root argument and divided
 * distance lies in the ranges where the fast square root and the reciprocal
 * division were checked equal to IEEE on this device, and that every sample
 * index lies inside the record; such a voxel runs a branch-free loop that keeps
 * the reference's operation order (sample indices bit-equal) and reads the
 * per-frame interpolation table (one 32-byte cubic segment per term, already
 * rotated by the demodulation phase of its sample; the term rotates by
 * theta (f - 1/2)). Voxels without the proof run das_voxel unchanged. The
 * accumulation order is the reference's: per receive channel over transmits,
 * then into the voxel.
 */
#include "bf_das_forces.cuh"

namespace bf {

/* One thread per voxel, 8 (x) by 16 (z) voxels of one y slice per block (as
 * das_kernel), the outer loop split over groups of blocks as das_kernel's. */
template <int INTERP>
__global__ void __launch_bounds__(DAS_THREADS, 8)
das_forces(DasParams p, const float4 *__restrict__ tab)
{
	const int vx = blockIdx.x * DAS_TX + (threadIdx.x & (DAS_TX - 1));
	const int vz = blockIdx.z * DAS_TZ + (threadIdx.x / DAS_TX);
	const int vy = blockIdx.y / p.groups;
	const int grp = blockIdx.y - vy * p.groups;
	if (vx >= p.dims[0] || vz >= p.dims[2]) return;
	const int u_begin = grp * p.per_group;
	const int u_end   = min(p.loop_end, u_begin + p.per_group);
	const float2 s = forces_voxel<INTERP>(p, tab, vx, vy, vz, u_begin, u_end);
	const int64_t nvox = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	const int64_t o = ((int64_t)vz * p.dims[1] + vy) * p.dims[0] + vx;
	if (p.groups > 1) p.partial[grp * nvox + o] = s;
	else              p.frame[o] = s;
}

/* FORCES (not UFORCES), the fast path, dense channel rows, cubic or linear
 * interpolation: the per-frame table applies. */
bool das_forces_supported(const DasParams &p)
{
	return p.family == DAS_FORCES && !p.half_table && p.fast && !p.sparse_mode && !p.coherency && p.dense_rows &&
	       p.rf_count >= (int64_t)p.C * p.T * p.S && p.loop_end == p.C &&
	       (p.interp == INTERP_CUBIC || p.interp == INTERP_LINEAR) && p.rx_step == 1;
}

cudaError_t launch_das_forces(const DasParams &p, float4 *table, cudaStream_t s)
{
	const int64_t n = (int64_t)p.dims[0] * p.dims[1] * p.dims[2];
	if (n == 0) return cudaSuccess;
	if (!das_forces_supported(p) || p.groups < 1 || (p.groups > 1 && !p.partial) || !table)
		return cudaErrorInvalidValue;
	cudaError_t e = launch_das_table(p, table, s);
	if (e != cudaSuccess) return e;
	const dim3 grid((p.dims[0] + DAS_TX - 1) / DAS_TX, p.dims[1] * p.groups, (p.dims[2] + DAS_TZ - 1) / DAS_TZ);
	if (p.interp == INTERP_CUBIC) das_forces<INTERP_CUBIC><<<grid, DAS_THREADS, 0, s>>>(p, table);
	else                          das_forces<INTERP_LINEAR><<<grid, DAS_THREADS, 0, s>>>(p, table);
	g_kernel_launches++;
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	if (p.groups > 1) return launch_das_reduce(p.partial, p.frame, n, p.groups, s);
	return cudaSuccess;
}

} /* namespace bf */
