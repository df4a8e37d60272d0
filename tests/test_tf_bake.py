"""TransFunc1DKeys bake: the library's host bake equals the oracle's
restatement on seeded key sets (split keys, gamma, thresholds). CPU only."""
import numpy as np
import pytest

import voreen_gb300 as v


def random_keys(rng, n):
    xs = np.sort(rng.uniform(0, 1, n)).astype(np.float32)
    keys = []
    for x in xs:
        cl = tuple(int(c) for c in rng.integers(0, 256, 4))
        cr = cl if rng.random() < 0.6 else tuple(int(c) for c in rng.integers(0, 256, 4))
        keys.append((float(x), cl, cr))
    return keys


@pytest.mark.parametrize("seed", range(12))
def test_bake_matches_oracle(vrc_lib, orc, seed):
    rng = np.random.default_rng(seed)
    keys = random_keys(rng, int(rng.integers(1, 12)))
    width = int(rng.choice([2, 256, 1000, 4096]))
    gamma = 1.0 if seed % 3 else float(rng.uniform(0.3, 3.0))
    thr = (0.0, 1.0) if seed % 4 else (float(rng.uniform(0, 0.3)), float(rng.uniform(0.6, 1.0)))
    a = v.TransferFunction.bake(keys, width, gamma, thr)
    b = orc.bake_tf(keys, width, gamma, thr)
    np.testing.assert_array_equal(a, b)


def test_bake_ramp_values(vrc_lib):
    # alpha 0 at intensity <= 40/255, linear to 153 at 1 (truncating lerp)
    from voreen_gb300 import synth
    t = v.TransferFunction.bake(synth.tf_keys_c1(), 256)
    assert (t[:41, 3] == 0).all() and t[255, 3] == 153
    assert (np.diff(t[41:, 3].astype(int)) >= 0).all()
    assert tuple(t[255, :3]) == (255, 0, 0) and tuple(t[0, :3]) == (0, 0, 255)


def test_bake_rejects_unsorted(vrc_lib):
    with pytest.raises(v.VrcError):
        v.TransferFunction.bake([(0.5, (0, 0, 0, 0)), (0.2, (1, 1, 1, 1))], 256)
