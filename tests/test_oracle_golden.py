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
