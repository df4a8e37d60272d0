"""The march normalises voxels (VolumeRAM::getVoxelNormalized, v / 255 and
v / 65535 as float divisions) as fma(v, A, v * B) with the constants of
Vox<VRC_U8>/Vox<VRC_U16>::norm (march_core.cuh). This checks, with exact
rational arithmetic, that the fused form rounds to the correctly rounded
quotient for every voxel value, and that the shorter u8 form (one tail term
fewer) does not, so the extra term is needed."""
from fractions import Fraction as F
import struct

import numpy as np


def _bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def _f(bits: int) -> float:
    return struct.unpack("<f", struct.pack("<I", bits))[0]


def _rn32(q: F) -> float:
    """Correctly rounded (ties to even) binary32 value of a non-negative rational."""
    if q == 0:
        return 0.0
    c = _bits(float(np.float32(float(q))))
    best = None
    for b in (c - 1, c, c + 1):
        d = abs(F(_f(b)) - q)
        key = (d, b & 1)
        if best is None or key < best[0]:
            best = (key, b)
    return _f(best[1])


def _exact(c: F) -> F:
    assert F(float(np.float32(float(c)))) == c, "constant is not a float"
    return c


def _mismatches(D: int, A: F, B: F) -> list[int]:
    bad = []
    for v in range(D + 1):
        assert F(float(np.float32(float(v * B)))) == v * B  # v * B is exact
        if _rn32(v * A + v * B) != _rn32(F(v, D)):
            bad.append(v)
    return bad


A8 = _exact(F(1, 2**8) + F(1, 2**16))
B8 = _exact(F(1, 2**24) + F(1, 2**32) + F(1, 2**40))
A16 = _exact(F(1, 2**16) + F(1, 2**32))
B16 = _exact(F(1, 2**48))


def test_u8_norm_is_correctly_rounded():
    assert _mismatches(255, A8, B8) == []


def test_u8_short_form_fails_at_powers_of_two():
    assert _mismatches(255, A8, F(1, 2**24) + F(1, 2**32)) == [1, 2, 4, 8, 16, 32, 64, 128]


def test_u16_norm_is_correctly_rounded():
    assert _mismatches(65535, A16, B16) == []


def test_constants_match_the_kernel_literals():
    # 0x1.01p-8f, 0x1.0101p-24f, 0x1.0001p-16f, 0x1p-48f
    assert float(A8) == float.fromhex("0x1.01p-8")
    assert float(B8) == float.fromhex("0x1.0101p-24")
    assert float(A16) == float.fromhex("0x1.0001p-16")
    assert float(B16) == float.fromhex("0x1p-48")
