/*
 * sanitize_host.cpp -- host-code check run under AddressSanitizer and
 * UndefinedBehaviorSanitizer (tests/test_sanitizers.py builds it with
 * -fsanitize=address,undefined together with the library's host planning code,
 * csrc/bf_host.cpp, and the CPU oracle, oracle/bf_oracle.c).
 *
 * It exercises the host code that every compute runs before its kernels --
 * pipeline planning, Hadamard matrices, Kaiser and matched filters, the voxel
 * transform, mip counts -- over seeded random parameters and pipelines, and
 * cross-checks each against the oracle's restatement of the reference
 * (beamformer.c:303-518, math.c:33-181). It then runs the oracle's decode,
 * demodulate, filter, DAS, sum and min/max stages on small inputs. Any
 * out-of-bounds access or undefined operation aborts the run; any mismatch
 * returns 1.
 */
#include "bf_host.h"
#include "bf_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

static int g_fail = 0, g_checks = 0;

static void check(bool ok, const char *what, int a = 0, int b = 0)
{
	g_checks++;
	if (!ok) {
		g_fail++;
		if (g_fail < 20) std::printf("MISMATCH %s (%d, %d)\n", what, a, b);
	}
}

static bool strides_eq(const bf::Strides &s, uint32_t ic, uint32_t is, uint32_t it, uint32_t oc, uint32_t os, uint32_t ot)
{
	return s.in_channel == ic && s.in_sample == is && s.in_transmit == it && s.out_channel == oc &&
	       s.out_sample == os && s.out_transmit == ot;
}

static BeamformerParameters random_params(std::mt19937 &rng)
{
	std::uniform_int_distribution<int> pick(0, 1000000);
	const uint32_t Ts[] = {2, 4, 8, 12, 16, 20, 32, 64, 128};
	const uint32_t Ss[] = {64, 128, 256, 512, 1024, 2048};
	BeamformerParameters bp{};
	const uint32_t T = Ts[pick(rng) % 9], S = Ss[pick(rng) % 6], C = 8u << (pick(rng) % 5);
	bp.dec_data_dim[0] = S; bp.dec_data_dim[1] = C; bp.dec_data_dim[2] = T; bp.dec_data_dim[3] = 1;
	bp.rf_raw_dim[0] = S * T; bp.rf_raw_dim[1] = C;
	bp.decode = pick(rng) % 2;
	bp.das_shader_id = pick(rng) % 11;
	bp.transmit_mode = pick(rng) % 4;
	bp.decimation_rate = 1 + pick(rng) % 4;
	bp.sampling_frequency = 4e7f + (float)(pick(rng) % 100) * 1e5f;
	bp.center_frequency = bp.sampling_frequency / 4;
	bp.speed_of_sound = 1540.0f;
	bp.time_offset = (float)(pick(rng) % 10) * 1e-7f;
	bp.xdc_element_pitch[0] = bp.xdc_element_pitch[1] = 1e-4f;
	for (int i = 0; i < 4; i++) bp.xdc_transform[i * 5] = 1.0f;
	bp.xdc_transform[12] = -0.003f;
	bp.output_points[0] = 1 + pick(rng) % 64; bp.output_points[1] = 1 + pick(rng) % 3;
	bp.output_points[2] = 1 + pick(rng) % 64; bp.output_points[3] = 1 + pick(rng) % 16;
	bp.output_min_coordinate[0] = -0.005f; bp.output_min_coordinate[2] = 0.005f;
	bp.output_max_coordinate[0] = 0.005f; bp.output_max_coordinate[1] = 0.002f; bp.output_max_coordinate[2] = 0.03f;
	bp.off_axis_pos = (float)(pick(rng) % 5) * 1e-4f;
	bp.beamform_plane = pick(rng) % 2;
	bp.f_number = 0.5f + (float)(pick(rng) % 4) * 0.5f;
	bp.interpolate = pick(rng) % 2;
	return bp;
}

static void check_planning(std::mt19937 &rng)
{
	std::uniform_int_distribution<int> pick(0, 1000000);
	const int32_t stages[] = {BeamformerShaderKind_Decode, BeamformerShaderKind_Demodulate, BeamformerShaderKind_Filter,
	                          BeamformerShaderKind_DAS, BeamformerShaderKind_DASFast, BeamformerShaderKind_Sum,
	                          BeamformerShaderKind_MinMax, BeamformerShaderKind_CudaHilbert,
	                          BeamformerShaderKind_CudaDecode};
	for (int it = 0; it < 4000; it++) {
		BeamformerParameters bp = random_params(rng);
		int32_t shaders[16];
		uint8_t slots[16];
		const int32_t count = 1 + pick(rng) % 6;
		shaders[0] = pick(rng) % 2 ? BeamformerShaderKind_Decode : BeamformerShaderKind_Demodulate;
		for (int i = 1; i < count; i++) shaders[i] = stages[pick(rng) % 9];
		for (int i = 0; i < 16; i++) slots[i] = (uint8_t)(pick(rng) % 4);
		const int32_t data_kind = pick(rng) % 4;
		bf::FilterSpec fs[BEAMFORMER_FILTER_SLOTS];
		BfoFilterSpec ofs[4];
		for (int i = 0; i < 4; i++) {
			fs[i].kind = pick(rng) % 2;
			fs[i].length = 1 + pick(rng) % 128;
			fs[i].sampling_frequency = 2e7f;
			fs[i].param0 = 5.65f;
			fs[i].param1 = 5e6f;
			ofs[i] = {fs[i].kind, fs[i].length, fs[i].sampling_frequency, fs[i].param0, fs[i].param1};
		}
		bf::Plan pl;
		bf::plan_pipeline(bp, shaders, slots, count, data_kind, fs, pl);
		BfoPlan op;
		std::memset(&op, 0, sizeof(op));
		bfo_plan(&bp, shaders, slots, count, data_kind, ofs, &op);
		check(pl.count == op.shader_count, "stage count", pl.count, op.shader_count);
		for (int i = 0; i < pl.count && i < op.shader_count; i++) {
			check(pl.shaders[i] == op.shaders[i], "planned shader", pl.shaders[i], op.shaders[i]);
			check(pl.slots[i] == op.filter_slots[i], "filter slot", pl.slots[i], op.filter_slots[i]);
		}
		const BfoDecodeUBO &d = op.decode;
		check(strides_eq(pl.decode_st, d.input_channel_stride, d.input_sample_stride, d.input_transmit_stride,
		                 d.output_channel_stride, d.output_sample_stride, d.output_transmit_stride), "decode strides", it);
		check(pl.transmit_count == d.transmit_count && pl.decode_mode == d.decode_mode, "decode mode", it);
		const BfoFilterUBO &m = op.demod;
		check(strides_eq(pl.demod_st, m.input_channel_stride, m.input_sample_stride, m.input_transmit_stride,
		                 m.output_channel_stride, m.output_sample_stride, m.output_transmit_stride), "demod strides", it);
		const BfoFilterUBO &f = op.filter;
		check(strides_eq(pl.filter_st, f.input_channel_stride, f.input_sample_stride, f.input_transmit_stride,
		                 f.output_channel_stride, f.output_sample_stride, f.output_transmit_stride), "filter strides", it);
		check(pl.rf_size == op.rf_size, "rf size", (int)pl.rf_size, (int)op.rf_size);
		check(std::memcmp(pl.das.dec_data_dim, op.das.dec_data_dim, sizeof(pl.das.dec_data_dim)) == 0, "das dims", it);
		check(pl.das.sampling_frequency == op.das.sampling_frequency, "das fs", it);
		check(pl.das.center_frequency == op.das.center_frequency, "das fc", it);
		check(pl.das.time_offset == op.das.time_offset, "das time offset", it);
		check(pl.das.decimation_rate == op.das.decimation_rate, "das decimation", it);

		float M[16], OM[16];
		bf::voxel_transform(bp, M);
		bfo_voxel_transform(&bp, OM);
		bool same = true;
		for (int i = 0; i < 16; i++) same = same && std::fabs(M[i] - OM[i]) <= 1e-6f * (1.0f + std::fabs(OM[i]));
		check(same, "voxel transform", it);
		const int32_t dims[3] = {(int32_t)bp.output_points[0], (int32_t)bp.output_points[1], (int32_t)bp.output_points[2]};
		check(bf::frame_mips(dims) == bfo_frame_mips(dims), "mip count", it);
	}
}

static void check_matrices_and_filters(std::mt19937 &rng)
{
	for (int order = 1; order <= 320; order++) {
		std::vector<int8_t> h;
		int32_t syl = 0, base = 0;
		const bool ok = bf::hadamard_matrix(order, h, syl, base);
		std::vector<int32_t> oh((size_t)order * order + 1, 0);
		const bool ook = bfo_hadamard_transpose(order, oh.data()) != 0;
		check(ok == ook, "hadamard availability", order);
		if (ok && ook) {
			bool same = true;
			for (int i = 0; i < order * order; i++) same = same && h[i] == oh[i];
			check(same, "hadamard entries", order);
		}
	}
	std::uniform_real_distribution<float> u(0.0f, 1.0f);
	for (int length = 1; length <= 300; length++) {
		const float fs = 1e7f + 9e7f * u(rng), cutoff = fs * (0.05f + 0.4f * u(rng)), beta = 10.0f * u(rng);
		std::vector<float> a(length), b(length);
		bf::kaiser_low_pass(cutoff, fs, beta, length, a.data());
		bfo_kaiser_low_pass(cutoff, fs, beta, length, b.data());
		float peak = 0, err = 0;
		for (int i = 0; i < length; i++) { peak = std::fmax(peak, std::fabs(b[i])); err = std::fmax(err, std::fabs(a[i] - b[i])); }
		check(err <= 1e-5f * peak + 1e-12f, "kaiser taps", length);
		const float ftx = fs / 4 * (0.8f + 0.4f * u(rng));
		bf::matched_filter(fs / 4, ftx, fs, length, a.data());
		bfo_matched_filter(fs / 4, ftx, fs, length, b.data());
		peak = 0; err = 0;
		for (int i = 0; i < length; i++) { peak = std::fmax(peak, std::fabs(b[i])); err = std::fmax(err, std::fabs(a[i] - b[i])); }
		check(err <= 1e-5f * peak + 1e-12f, "matched taps", length);
	}
}

static void run_oracle_stages(std::mt19937 &rng)
{
	std::uniform_int_distribution<int> pick(-30000, 30000);
	for (int rep = 0; rep < 6; rep++) {
		BeamformerParameters bp = random_params(rng);
		const uint32_t S = 64, C = 8, T = 4 << (rep % 3);
		bp.dec_data_dim[0] = S; bp.dec_data_dim[1] = C; bp.dec_data_dim[2] = T;
		bp.rf_raw_dim[0] = S * T; bp.rf_raw_dim[1] = C;
		bp.decode = 1;
		bp.das_shader_id = rep % 2 ? DASShaderKind_FORCES : DASShaderKind_HERCULES;
		bp.decimation_rate = 1 + rep % 2;
		bp.output_points[0] = 8; bp.output_points[1] = 1 + rep % 2; bp.output_points[2] = 8; bp.output_points[3] = 2;
		int32_t shaders[5] = {BeamformerShaderKind_Decode, BeamformerShaderKind_Demodulate, BeamformerShaderKind_DASFast,
		                      BeamformerShaderKind_Sum, BeamformerShaderKind_MinMax};
		uint8_t slots[16] = {};
		BfoFilterSpec ofs[4] = {{0, 16, bp.sampling_frequency / 2, 5.65f, 5e6f}, {}, {}, {}};
		BfoPlan op;
		std::memset(&op, 0, sizeof(op));
		bfo_plan(&bp, shaders, slots, 5, BeamformerDataKind_Int16, ofs, &op);
		std::vector<int16_t> raw((size_t)S * T * C);
		for (auto &v : raw) v = (int16_t)pick(rng);
		const size_t chan = (size_t)2 * S * C * T;
		std::vector<float> b0(chan), b1(chan);
		std::vector<int32_t> H((size_t)T * T);
		bfo_hadamard_transpose((int32_t)T, H.data());
		std::vector<int16_t> map(256);
		for (int i = 0; i < 256; i++) map[i] = (int16_t)i;
		bfo_decode(&op.decode, op.shaders[0], 1, BeamformerDataKind_Int16, raw.data(), raw.size() * 2, b0.data(),
		           b0.size() * 4, H.data(), (int32_t)T, map.data(), op.decode_dispatch, 2);
		std::vector<float> taps(16);
		bfo_kaiser_low_pass(5e6f, bp.sampling_frequency / 2, 5.65f, 16, taps.data());
		bfo_filter(&op.demod, op.shaders[1], b0.data(), b0.size() * 4, b1.data(), b1.size() * 4, taps.data(), 16,
		           map.data(), op.demod_dispatch, 2);
		float M[16];
		bfo_voxel_transform(&op.das, M);
		const int32_t dims[3] = {(int32_t)op.das.output_points[0], (int32_t)op.das.output_points[1],
		                         (int32_t)op.das.output_points[2]};
		const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
		std::vector<float> frame(2 * nv), frame2(2 * nv), avg(2 * nv), focal(512, 0.0f);
		for (int i = 1; i < 512; i += 2) focal[i] = INFINITY;
		std::vector<int16_t> sparse(256);
		for (int i = 0; i < 256; i++) sparse[i] = (int16_t)i;
		for (int interp = 0; interp < 3; interp++) {
			bfo_das(&op.das, 1, b1.data(), op.rf_size / 4, sparse.data(), focal.data(), M, frame.data(), dims, 0,
			        (int64_t)nv, interp, 2);
			bfo_das(&op.das, 0, b1.data(), op.rf_size / 4, sparse.data(), focal.data(), M, frame2.data(), dims, 0,
			        (int64_t)nv, interp, 2);
			bool finite = true;
			for (size_t i = 0; i < 2 * nv; i++) finite = finite && std::isfinite(frame[i]) && std::isfinite(frame2[i]);
			check(finite, "das finite", rep, interp);
		}
		const float *ins[2] = {frame.data(), frame2.data()};
		bfo_sum(avg.data(), ins, 2, 0.5f, dims, 2);
		std::vector<float> levels(bfo_min_max_levels_floats(dims) + 2);
		bfo_min_max(frame.data(), dims, levels.data(), 2);
	}
}

int main()
{
	std::mt19937 rng(12345);
	check_planning(rng);
	check_matrices_and_filters(rng);
	run_oracle_stages(rng);
	std::printf("%d checks, %d mismatches\n", g_checks, g_fail);
	return g_fail ? 1 : 0;
}
