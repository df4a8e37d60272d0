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


def _golden_cases():
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tf_bake.npz"))
    for i in range(int(g["n"])):
        inten, cols = g[f"c{i}_intensity"], g[f"c{i}_colors"]
        width, gamma, lo, hi = g[f"c{i}_params"]
        keys = [(float(inten[k]), tuple(int(c) for c in cols[k, :4]), tuple(int(c) for c in cols[k, 4:]))
                for k in range(len(inten))]
        yield i, keys, int(width), float(gamma), (float(lo), float(hi)), g[f"c{i}_table"]


def test_bake_matches_reference_code(vrc_lib, orc):
    """Pinned: the library's bake (vrc_tf_bake_keys) and the oracle's equal
    the tables the reference's own TransFunc1DKeys::getMappingForValueUByte and
    applyGammaToIntensity produce (tests/golden/tf_bake.npz, made by
    tests/golden/make_golden.py from the Voreen sources), byte for byte; the
    cases include split and coincident keys, keys on texel values, gamma,
    thresholds and the keys of the sample transfer functions nucleon.tfi and
    walnut.tfi."""
    n = 0
    for i, keys, width, gamma, thr, table in _golden_cases():
        np.testing.assert_array_equal(orc.bake_tf(keys, width, gamma, thr), table, err_msg=f"oracle, case {i}")
        if keys:  # the library's C ABI takes at least one key
            np.testing.assert_array_equal(v.TransferFunction.bake(keys, width, gamma, thr), table,
                                          err_msg=f"library, case {i}")
        n += 1
    assert n >= 49
