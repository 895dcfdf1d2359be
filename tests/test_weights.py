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
