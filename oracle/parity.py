"""Parity measures between a GPU frame and the oracle -- TEST INFRASTRUCTURE ONLY.

The bar is max |d| <= 1/255 per RGBA channel against the FP64 oracle. The
reference's CPU path is itself FP32, so on a few rays FP32 and FP64 take a
different discrete decision -- a different number of samples (accumulated
alpha lands within rounding of the 0.95 termination threshold, or t of the
t <= tend stop), a different selected sample (first hit, MIP maximum, ISO
hit) or, for MIP / ISO, a different TF entry for the selected sample. Those
rays are counted and their max |d| is reported beside the bound, which is
checked on every other ray. A different TF entry at any sample (an index
rounding tie, detected through the oracle's per-ray decision signatures)
counts as a different decision in every compositing mode.
"""
from __future__ import annotations

import numpy as np

DVR, MIP, ISO = 0, 1, 2


def sample_index(first_hit, step):
    """Loop index of the selected sample from its ray parameter (-1: none)."""
    fh = np.asarray(first_hit, np.float64)
    return np.where(fh >= 0, np.rint(fh / step), -1).astype(np.int64)


def decision_divergent(o32, s32, fh32, o64, s64, fh64, comp, step, shaded=False, sig32=None, sig64=None):
    """Boolean (H, W): rays where FP32 and FP64 take a different discrete
    decision. sig32 / sig64: the oracle's per-ray decision signatures (the TF
    entries with alpha > 0 picked, by sample); with them a different TF entry
    at any sample counts too."""
    div = s32 != s64
    div |= sample_index(fh32, step) != sample_index(fh64, step)
    if sig32 is not None and sig64 is not None:
        div |= sig32 != sig64
    if comp in (MIP, ISO):
        d = np.abs(o32.astype(np.float64) - o64)
        div |= d[..., 3] > 1e-6
        if not shaded:
            div |= d.max(axis=-1) > 1e-5
    return div


def report(gpu_img, o32, s32, fh32, o64, s64, fh64, comp, step, shaded=False, tol=1.0 / 255.0, sig32=None,
           sig64=None) -> dict:
    """Parity of one frame: max |d| against the FP32 oracle; against the FP64
    oracle on all rays and on agreeing rays; the decision-divergent rays
    (count, max |d|) and, of them, the waived ones -- those above `tol` --
    with their max |d|; the hit rays and the channels above 0.5/255."""
    g = np.asarray(gpu_img, np.float64)
    d32 = np.abs(g - o32.astype(np.float64)).max(axis=-1)
    d64 = np.abs(g - o64).max(axis=-1)
    div = decision_divergent(o32, s32, fh32, o64, s64, fh64, comp, step, shaded, sig32, sig64)
    waived = div & (d64 > tol)
    hits = int((s32 > 0).sum())
    ok = ~div
    return {
        "max_abs_vs_fp32": float(d32.max(initial=0.0)),
        "max_abs_vs_fp64_all_rays": float(d64.max(initial=0.0)),
        "max_abs_vs_fp64": float(d64[ok].max(initial=0.0)),
        "divergent_rays": int(div.sum()),
        "divergent_max_abs_vs_fp64": float(d64[div].max(initial=0.0)),
        "waived_rays": int(waived.sum()),
        "hit_rays": hits,
        "rays": int(d64.size),
        "channels_over_half_lsb_vs_fp64": int((np.abs(g - o64) > 0.5 / 255.0)[ok].sum()),
    }
