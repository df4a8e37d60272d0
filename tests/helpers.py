"""Shared helpers for the parity tests: run one case through the C ABI and
through the oracle on identical inputs."""
from __future__ import annotations

import numpy as np

import oracle
from oracle import parity
import voreen_gb300 as v

TOL = 1.0 / 255.0  # spec bound per RGBA channel against the FP64 oracle

# Parity reports of this session (printed by conftest's terminal summary).
REPORTS: list = []


def oracle_params(w_params, light=None, cam=None, preint_table=None):
    p = w_params
    return oracle.make_params(sampling_rate=p.sampling_rate, compositing=p.compositing, shading=p.shading,
                              mida_gamma=p.mida_gamma, preint_table=preint_table,
                              iso_value=p.iso_value, ert=p.ert_threshold,
                              light_pos=list(p.light_position)[:3] if light is None else light,
                              camera_pos=list(p.camera.position) if cam is None else cam,
                              ambient=list(p.light_ambient), diffuse=list(p.light_diffuse),
                              specular=list(p.light_specular), shininess=p.material_shininess,
                              attenuation=list(p.light_attenuation) if p.apply_attenuation else None)


def oracle_entry_exit(desc, params, quantize=False):
    _, _, inv = v.camera_matrices(params.camera, desc, params.width, params.height)
    return oracle.entry_exit(inv, params.width, params.height, quantize)


class Case:
    """One render on both sides. vox is (Z, Y, X)."""

    def __init__(self, ctx, vox, tf_rgba, domain, params, spacing=(1, 1, 1), offset=(0, 0, 0), rwm=(1.0, 0.0),
                 brick=0, entry=None, exit_pts=None):
        self.ctx = ctx
        self.vox = np.ascontiguousarray(vox)
        self.tf_rgba = tf_rgba
        self.domain = domain
        self.params = params
        self.spacing, self.offset, self.rwm = spacing, offset, rwm
        self.vol = v.Volume(ctx, self.vox, spacing, offset, rwm, brick)
        self.tf = v.TransferFunction(ctx, tf_rgba, domain)
        if entry is None and params.entry_exit_mode == v.EE_BUFFERS:
            entry, exit_pts = oracle_entry_exit(self.vol.desc, params)
        self.entry, self.exit = entry, exit_pts
        self.ovol = oracle.make_volume(self.vox, spacing, offset, rwm)
        self.sig = {}  # precision -> the last oracle render's decision signatures

    def gpu(self, out_format=v.OUT_RGBA32F, **over):
        p = self.params
        for k, val in over.items():
            setattr(p, k, val)
        return v.render(self.ctx, self.vol, self.tf, p, self.entry, self.exit, out_format)

    @property
    def step(self):
        return 1.0 / (max(self.vol.dims) * self.params.sampling_rate)

    def oracle(self, precision=32, rows=None, entry=None, exit_pts=None, preint_table=None):
        e = self.entry if entry is None else entry
        x = self.exit if exit_pts is None else exit_pts
        sig = np.zeros(e.shape[:2], np.uint32)
        r = oracle.render(self.ovol, self.tf_rgba, self.domain, oracle_params(self.params, preint_table=preint_table),
                          e, x, precision, rows, signature=sig)
        self.sig[precision] = sig
        return r

    @property
    def sigs(self):
        """(FP32, FP64) decision signatures of the last oracle renders."""
        return self.sig.get(32), self.sig.get(64)


sample_index = parity.sample_index
decision_divergent = parity.decision_divergent


def assert_fp64_parity(gpu_img, o32, s32, fh32, o64, s64, fh64, comp, step, shaded=False, max_div_frac=2e-3,
                       tol=TOL, label=None, sigs=(None, None)):
    """max |d| <= tol on every ray where FP32 and FP64 make the same discrete
    decisions. A ray above tol is waived only if its decisions diverge, and
    the waived rays (counted, with their max |d| reported) must be a tiny
    fraction of the hit rays. Returns the parity report."""
    r = parity.report(gpu_img, o32, s32, fh32, o64, s64, fh64, comp, step, shaded, tol, sigs[0], sigs[1])
    if label is not None:
        REPORTS.append((label, r))
    hits = max(1, r["hit_rays"])
    assert r["waived_rays"] <= max(2, max_div_frac * hits), \
        f"{r['waived_rays']} decision-divergent rays above the bound of {hits} hit rays " \
        f"(their max |d| {r['divergent_max_abs_vs_fp64'] * 255:.3f}/255)"
    assert r["max_abs_vs_fp64"] <= tol, f"max |d| on agreeing rays = {r['max_abs_vs_fp64'] * 255:.3f}/255"
    return r
