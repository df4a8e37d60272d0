"""The oracle against the golden vectors made from the reference's own code
(tests/golden/make_golden.py over oracle/_ref), and the library's host math
against the same vectors. CPU only."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_trilinear_matches_reference_volumeram(orc):
    g = np.load(os.path.join(GOLD, "trilinear.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in g.files})
    assert len(keys) == 15
    for k in keys:
        vox, pos, val = g[k + "_vox"], g[k + "_pos"], g[k + "_val"]
        vol = orc.make_volume(np.ascontiguousarray(vox))
        got = orc.trilinear(vol, pos)
        # bit-exact: same operations in the same order as VolumeRAM
        np.testing.assert_array_equal(got.view(np.uint32), val.view(np.uint32), err_msg=k)


def test_iround_matches_tgt(orc):
    g = np.load(os.path.join(GOLD, "iround.npz"))
    x = g["x"].astype(np.float32)
    ours = np.floor(x + np.float32(0.5)).astype(np.int32)  # tgt::round = floor(x + 0.5f) in float
    np.testing.assert_array_equal(ours, g["iround"])


def test_camera_matrices_match_tgt(vrc_lib):
    import voreen_gb300 as v
    g = np.load(os.path.join(GOLD, "camera.npz"))
    desc = v.make_desc(v.U8, (8, 8, 8))
    for i in range(len(g["eye"])):
        cam = v.make_camera(g["eye"][i], g["focus"][i], g["up"][i])
        view, _, _ = v.camera_matrices(cam, desc, 64, 64)
        np.testing.assert_allclose(view.reshape(-1), g["lookat"][i].astype(np.float64), rtol=2e-5, atol=2e-4)
    # createPerspective: the library's projection for fov / aspect / near / far
    for i in range(len(g["persp"])):
        fov, asp, n, f = [float(x) for x in g["persp_params"][i]]
        W, H = 1000, max(1, int(round(1000 / asp)))
        asp_eff = W / H
        cam = v.make_camera((0, 0, 1), (0, 0, 0), fovy=np.degrees(fov), near=n, far=f)
        _, proj, _ = v.camera_matrices(cam, desc, W, H)
        ref = g["persp"][i].astype(np.float64).reshape(4, 4)
        if asp_eff >= 1.0:
            ref[0, 0] *= asp / asp_eff  # f / aspect with the window aspect the library was given
            np.testing.assert_allclose(proj, ref, rtol=1e-5, atol=1e-6)


def test_oracle_camera_matches_tgt(orc):
    """The oracle's own camera chain (used by the benchmark's CPU arm) against
    the reference's createLookAt / createPerspective outputs."""
    from oracle import camera as ocam
    g = np.load(os.path.join(GOLD, "camera.npz"))
    for i in range(len(g["eye"])):
        m = ocam.look_at(g["eye"][i].astype(np.float64), g["focus"][i].astype(np.float64),
                         g["up"][i].astype(np.float64))
        np.testing.assert_allclose(m.reshape(-1), g["lookat"][i].astype(np.float64), rtol=2e-5, atol=2e-4)
    for i in range(len(g["persp"])):
        fov, asp, n, f = [float(x) for x in g["persp_params"][i]]
        if asp < 1.0:
            continue  # the camera widens fovy for tall windows; createPerspective alone does not
        m = ocam.perspective(np.degrees(fov), n, f, asp)
        np.testing.assert_allclose(m, g["persp"][i].astype(np.float64).reshape(4, 4), rtol=1e-5, atol=1e-6)


def test_oracle_camera_equals_library(vrc_lib):
    import voreen_gb300 as v
    from oracle import camera as ocam
    rng = np.random.default_rng(7)
    for _ in range(20):
        dims = tuple(int(d) for d in rng.integers(1, 600, 3))
        spacing = tuple(float(s) for s in rng.uniform(0.3, 2.0, 3))
        pos = rng.uniform(-900, 900, 3)
        focus = rng.uniform(0, 300, 3)
        W, H = int(rng.integers(16, 2000)), int(rng.integers(16, 2000))
        fovy, near, far = float(rng.uniform(10, 90)), float(rng.uniform(0.1, 5)), float(rng.uniform(2000, 5000))
        cam = v.make_camera(pos, focus, fovy=fovy, near=near, far=far)
        _, _, inv = v.camera_matrices(cam, v.make_desc(v.U8, dims, spacing), W, H)
        ours = ocam.inverse_mvp(pos, focus, (0, 1, 0), fovy, near, far, W, H, dims, spacing)
        np.testing.assert_allclose(ours, inv, rtol=1e-9, atol=1e-12 * np.abs(inv).max())


def test_oracle_generator_equals_library(vrc_lib):
    """The benchmark's CPU arm builds its inputs with oracle.synth_volume: the
    same volumes as the library's generator."""
    import oracle
    import voreen_gb300 as v
    for kind, dt, dims, seed in [(0, v.U8, (40, 33, 27), 5), (1, v.U16, (64, 48, 40), 2002), (0, v.F32, (17, 9, 31), 9)]:
        np.testing.assert_array_equal(oracle.synth_volume(kind, dt, dims, seed), v.synth_volume(kind, dt, dims, seed))
