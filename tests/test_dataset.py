"""The reference's captured-dataset format (zemp_bp_v1 parameter block + zstd
int16 frames, tests/throughput.c) and its throughput driver's configuration."""
import ctypes
import json
import os

import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi, dataset
from bf_cases import small_params, small_raw, run_both, check_volume

HERE = os.path.dirname(os.path.abspath(__file__))
SH = abi.SHADER


def _zstd_or_skip():
    try:
        dataset._zstd_lib()
    except RuntimeError as e:
        pytest.skip(str(e))


def _study(tmp_path, bp, frames, **kw):
    focal = np.zeros(512, np.float32)
    focal[1::2] = np.inf
    focal[0::2] = np.linspace(-5, 5, 256)
    sparse = np.full(256, -1, np.int16)
    return dataset.write_study(str(tmp_path), "study", bp, frames, focal=kw.get("focal", focal),
                               sparse=kw.get("sparse", sparse), channel_mapping=kw.get("chmap"))


def test_layout_matches_reference_typedef():
    """Field offsets and size against those printed by a probe compiled from the
    reference's own zemp_bp_v1 typedef (tests/golden/make_zemp_layout.py)."""
    ref = json.load(open(os.path.join(HERE, "golden", "zemp_bp_v1_layout.json")))
    assert ctypes.sizeof(dataset.ZempBpV1) == ref.pop("sizeof")
    for name, off in ref.items():
        assert getattr(dataset.ZempBpV1, name).offset == off, name


def test_round_trip(tmp_path):
    _zstd_or_skip()
    bp = small_params(S=256, C=16, T=16)
    rng = np.random.default_rng(1)
    frames = [rng.integers(-2 ** 15, 2 ** 15, 256 * 16 * 16, dtype=np.int16) for _ in range(3)]
    chmap = rng.permutation(256).astype(np.int16)
    _study(tmp_path, bp, frames, chmap=chmap)
    st = dataset.Study(str(tmp_path), "study")
    assert st.frame_count() == 3
    for i, fr in enumerate(frames):
        assert np.array_equal(st.frame(i), fr)
    z = st.zbp
    assert z.magic == dataset.ZEMP_BP_MAGIC and z.version == 1
    assert np.array_equal(np.asarray(z.channel_mapping[:], np.int16), chmap)
    back = dataset.to_beamformer_parameters(z)
    for f in ("xdc_transform", "dec_data_dim", "xdc_element_pitch", "rf_raw_dim"):
        assert list(getattr(back, f)) == list(getattr(bp, f)), f
    for f in ("transmit_mode", "decode", "das_shader_id", "time_offset", "sampling_frequency", "center_frequency",
              "speed_of_sound"):
        assert getattr(back, f) == getattr(bp, f), f
    # fields the block does not carry stay as they were
    assert list(back.output_points) == [0, 0, 0, 0] and back.decimation_rate == 0


def test_bad_blocks_are_rejected(tmp_path):
    bp = small_params(S=256, C=16, T=16)
    _zstd_or_skip()
    path = os.path.join(_study(tmp_path, bp, []), "study.bp")
    raw = bytearray(open(path, "rb").read())
    for bad in (raw[:-1], raw + b"\0", bytes([raw[0] ^ 1]) + raw[1:], raw[:8] + b"\2" + raw[9:]):
        open(path, "wb").write(bytes(bad))
        with pytest.raises(ValueError):
            dataset.read_parameters(path)


def test_compress_round_trip_and_corrupt_frame():
    _zstd_or_skip()
    data = np.arange(10000, dtype=np.int16).tobytes()
    blob = dataset.compress(data)
    assert len(blob) < len(data) and dataset.decompress(blob) == data
    with pytest.raises(RuntimeError):
        dataset.decompress(blob[:len(blob) // 2])


def test_driver_setup_follows_reference_driver():
    bp = small_params(S=256, C=16, T=16)
    z = dataset.ZempBpV1()
    z.magic, z.version = dataset.ZEMP_BP_MAGIC, 1
    z.sampling_frequency, z.center_frequency = 40e6, 5e6
    z.raw_data_dim[:] = [bp.rf_raw_dim[0], bp.rf_raw_dim[1], 0, 0]
    z.sparse_elements[0] = -1
    z.transmit_angles[3], z.focal_depths[3] = 12.5, 0.04
    cfg = dataset.driver_setup(z)
    b = cfg["bp"]
    assert b.decimation_rate == 1 and b.center_frequency == 10e6 and b.interpolate == 0 and b.f_number == 0.5
    assert list(b.output_points) == [512, 1, 1024, 1]
    assert np.allclose(list(b.output_min_coordinate), [-60e-3, 0, 10e-3, 0])
    assert np.allclose(list(b.output_max_coordinate), [60e-3, 0, 165e-3, 0])
    assert cfg["pipeline"] == [SH["Demodulate"], SH["Decode"], SH["Filter"], SH["DAS"]]
    assert cfg["kaiser"] == (5.65, 1.2e6, 20e6, 36)
    # matched filter: transducer frequency, demodulation frequency, 4 x fs / 2, ceil(4 x 2 x fs / 2 / fc) taps
    assert cfg["matched"] == (5e6, 10e6, 80e6, 16, 1) and cfg["stage_slots"] == {0: 0, 2: 1}
    assert np.array_equal(cfg["sparse_elements"], np.arange(256))
    assert cfg["focal_vectors"][6] == 12.5 and np.isclose(cfg["focal_vectors"][7], 0.04)
    z.sparse_elements[0] = 3
    assert dataset.driver_setup(z)["sparse_elements"][0] == 3


@pytest.mark.gpu
def test_study_beamforms_like_the_oracle(tmp_path):
    """A study written in the reference's layout, read back and beamformed with
    the reference driver's pipeline (Demodulate -> Decode -> matched Filter ->
    DAS), against the oracle."""
    _zstd_or_skip()
    bp = small_params(S=512, C=16, T=16, points=(24, 1, 20))
    raw = small_raw(bp)
    _study(tmp_path, bp, [raw, raw[::-1].copy()])
    st = dataset.Study(str(tmp_path), "study")
    cfg = dataset.driver_setup(st.zbp, output_points=(24, 1, 20), lateral=(-1.5e-3, 1.5e-3), axial=(1.0e-3, 3.5e-3))
    for i in range(st.frame_count()):
        bf, ref = run_both(cfg["bp"], cfg["pipeline"], st.frame(i), kaiser=cfg["kaiser"], matched=cfg["matched"],
                           chmap=cfg["channel_mapping"], focal=cfg["focal_vectors"], sparse=cfg["sparse_elements"],
                           slots=cfg["stage_slots"])
        check_volume(bf.frame(0)[0], ref["frame"], f"study frame {i}")


@pytest.mark.gpu
def test_throughput_driver(tmp_path):
    _zstd_or_skip()
    bp = small_params(S=512, C=16, T=16)
    _study(tmp_path, bp, [small_raw(bp)])
    r = dataset.throughput(str(tmp_path), "study", loops=4, output_points=(64, 1, 64))
    assert r["frames"] == 4 and r["ms_per_frame"] > 0 and r["rf_gb_per_s"] > 0
