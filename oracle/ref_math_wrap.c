/*
 * ref_math_wrap.c -- exports the reference's own host math for the parity
 * checks (TEST INFRASTRUCTURE). Compiled by oracle/build_ref.py against the
 * reference checkout's headers and sources; nothing here restates the math, it
 * only calls it:
 *   make_hadamard_transpose  math.c:33-122
 *   kaiser_low_pass_filter   math.c:125-142
 *   matched_filter           math.c:144-181
 *   cephes_i0                external/cephes.c:24-103
 *   das_voxel_transform_matrix beamformer.c:483-518 (cut out by build_ref.py)
 */
#include "compiler.h"
#include "util.h"
#include "beamformer_parameters.h"
#include "beamformer_work_queue.h"
#include "os_linux.c"

#define X(type, id, pretty, fixed_tx) DASShaderKind_##type = id,
typedef enum { DAS_TYPES DASShaderKind_Count } DASShaderKind;
#undef X

#include "ref_voxel_gen.inc"

static Arena ref_arena(void)
{
	static Arena base;
	if (!base.beg) base = os_alloc_arena(MB(64));
	Arena a = base;
	mem_clear(a.beg, 0, (iz)MB(8));
	return a;
}

/* Copies `count` ints starting at the returned matrix. On x86 the reference's
 * Kronecker product (orders 12 2^k and 20 2^k) writes outside the dim*dim block
 * through its unparenthesised store macro, so callers may ask for more than
 * dim*dim entries to see everything it wrote. */
int ref_hadamard(int dim, int *out, int count)
{
	Arena a = ref_arena();
	i32 *h = make_hadamard_transpose(&a, dim);
	if (!h) return 0;
	for (int i = 0; i < count; i++) out[i] = h[i];
	return 1;
}

void ref_kaiser(float cutoff, float fs, float beta, int length, float *out)
{
	Arena a = ref_arena();
	f32 *k = kaiser_low_pass_filter(&a, cutoff, fs, beta, length);
	for (int i = 0; i < length; i++) out[i] = k[i];
}

void ref_matched(float xdc_fc, float tx_f, float fs, int length, float *out)
{
	Arena a = ref_arena();
	f32 *k = matched_filter(&a, xdc_fc, tx_f, fs, length);
	for (int i = 0; i < length; i++) out[i] = k[i];
}

double ref_i0(double x) { return cephes_i0(x); }

void ref_voxel_transform(BeamformerParameters *bp, float *out)
{
	m4 m = das_voxel_transform_matrix(bp);
	for (int i = 0; i < 16; i++) out[i] = m.E[i];
}
