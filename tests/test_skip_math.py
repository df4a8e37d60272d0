"""The closed-form jump over empty runs (march.cu: jump_empty_run) restated
in float32 numpy: n steps of the FP32 accumulation t += step inside one
binade equal t + n * round(step / ulp(t)) * ulp(t), so the jump lands on the
exact t and sample count of the one-at-a-time loop. CPU only."""
import struct

import numpy as np

f32 = np.float32
CAP = 255 * 255


def _bits(x):
    return struct.unpack("<i", struct.pack("<f", float(x)))[0]


def _float(b):
    return f32(struct.unpack("<f", struct.pack("<i", b))[0])


def jump(t, loop, step, lim):
    ex = (_bits(t) >> 23) & 0xFF
    if ex < 24 or ex > 250:
        return t, loop
    u, top = _float((ex - 23) << 23), _float((ex + 1) << 23)
    k = f32(step * _float((277 - ex) << 23))
    if f32(k - np.floor(k)) == f32(0.5):
        return t, loop
    q = f32(np.rint(k) * u)
    if q <= 0:
        return t, loop
    nf = min(f32(np.floor(f32(f32(lim - t) / q)) + 1), f32(np.floor(f32(f32(top - t) / q))), f32(CAP - loop))
    n = int(nf) if nf > 0 else 0
    while n > 0 and (f32(t + f32(f32(n - 1) * q)) > lim or f32(t + f32(f32(n) * q)) >= top):
        n -= 1
    return f32(t + f32(f32(n) * q)), loop + n


def exact(t, loop, step, lim, tend):
    while not (t > tend) and loop < CAP and t <= lim:
        t = f32(t + step)
        loop += 1
    return t, loop


def skip(t, loop, step, lim):
    """The march's skip loop: jump inside a binade, single-step across its edge."""
    while t <= lim and loop < CAP:
        t, loop = jump(t, loop, step, lim)
        if t <= lim and loop < CAP:
            t = f32(t + step)
            loop += 1
    return t, loop


def test_skip_loop_across_binades():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        step = f32(1.0 / (f32(rng.choice([100, 256, 333, 1024, 3072])) * f32(rng.choice([1, 1.5, 2, 3.7]))))
        t = f32(rng.uniform(0.05, 1.2))
        lim = f32(t + rng.uniform(0, 0.9))   # runs that cross binade edges (0.125, 0.25, 0.5, 1)
        tend = f32(rng.uniform(float(t), 1.74))
        L = min(lim, tend)
        assert skip(t, 0, step, L) == exact(t, 0, step, L, tend)


def test_jump_equals_accumulation():
    rng = np.random.default_rng(0)
    for _ in range(5000):
        step = f32(1.0 / (f32(rng.choice([64, 128, 255, 512, 1024, 2048, 3000, 4096])) *
                          f32(rng.choice([0.5, 1, 1.5, 2, 3, 7.3, 20]))))
        t = max(f32(rng.uniform(0, 1.7)), step)
        loop = int(rng.integers(0, 2000))
        lim = f32(t + rng.uniform(0, 0.2))
        tend = f32(rng.uniform(float(t), 1.74))
        L = min(lim, tend)
        tj, lj = jump(t, loop, step, L) if t <= L else (t, loop)
        assert exact(tj, lj, step, L, tend) == exact(t, loop, step, L, tend)
