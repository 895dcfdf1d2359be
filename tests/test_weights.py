"""The learned variant's weight file: a plain versioned little-endian binary
(ogl_beamforming_cuda_gb300.learned.save_weights / load_weights)."""
import numpy as np
import pytest

def test_weight_file_round_trip_and_checks(tmp_path):
    """The versioned weight file (CPU only: plain arrays)."""
    from ogl_beamforming_cuda_gb300 import learned as Lm
    rng = np.random.default_rng(4)
    state = {n: (rng.standard_normal(cout * cin * 27).astype(np.float32), rng.standard_normal(cout).astype(np.float32))
             for n, cin, cout, _ in Lm.LAYERS}
    path = str(tmp_path / "w.bin")
    Lm.save_weights(path, state)
    back = Lm.load_weights(path)
    for n in state:
        assert np.array_equal(back[n][0], state[n][0]) and np.array_equal(back[n][1], state[n][1])
    raw = open(path, "rb").read()
    assert raw[:8] == Lm.WEIGHTS_MAGIC
    for bad in (raw[:-4], raw + b"\0\0\0\0", raw[:8] + b"\x02" + raw[9:], b"X" + raw[1:]):
        open(path, "wb").write(bad)
        with pytest.raises(ValueError):
            Lm.load_weights(path)
    state["m1"] = (state["m1"][0][:-1], state["m1"][1])
    with pytest.raises(ValueError):
        Lm.save_weights(path, state)


def test_learning_rate_schedule():
    """Linear warm-up over the first tenth of the steps to the peak, then a cosine
    decay to 5 % of it; never above the peak, monotone after the warm-up."""
    from ogl_beamforming_cuda_gb300 import learned as Lm
    steps, lr = 4000, 5e-4
    v = np.array([Lm.lr_schedule(s, steps, lr) for s in range(steps)])
    warm = steps // 10
    assert v[0] == pytest.approx(lr / warm)
    assert np.all(np.diff(v[:warm]) > 0) and v[warm - 1] == pytest.approx(lr)
    assert np.all(v <= lr * (1 + 1e-12))
    assert np.all(np.diff(v[warm:]) <= 1e-18)
    assert v[-1] == pytest.approx(0.05 * lr, rel=1e-3)


def test_bench_support_fraction_matches_direct_count():
    """bench.py's share of (transmit, receive) pairs inside the apodization support
    agrees with a direct count on a coarse voxel subset."""
    import bench
    from ogl_beamforming_cuda_gb300 import synth
    got = bench.support_fraction(step=32)
    lo, hi = np.asarray(bench.WORKLOAD_EXTENT[0]), np.asarray(bench.WORKLOAD_EXTENT[1])
    axes = [np.linspace(lo[k], hi[k], bench.POINTS[k])[::32] for k in range(3)]
    e = (np.arange(bench.C) - (bench.C - 1) / 2) * synth.PITCH
    inside = total = 0
    for x in axes[0]:
        for y in axes[1]:
            for z in axes[2]:
                d2 = (x - e)[:, None] ** 2 + (y - e)[None, :] ** 2
                inside += int(np.sum(d2 < (z / 2) ** 2))
                total += d2.size
    assert got == pytest.approx(inside / total, abs=2e-3)
