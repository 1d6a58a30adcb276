"""The kernels' exact FP32 -> FP64 conversion (lmg::f2d: bit moves for normal
numbers, used for every K and F entry the insertions write)
against the hardware conversion (numpy float32 -> float64), bit for bit, on a
million random bit patterns, every subnormal significand bit, signed zeros,
infinities and the extremes of the range."""
import numpy as np
import pytest

import libmesh_gb300 as lm

pytestmark = pytest.mark.gpu


def test_f2d_matches_the_hardware_conversion():
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2 ** 32, 1 << 20, dtype=np.uint64).astype(np.uint32)
    special = np.array([0x00000000, 0x80000000, 0x00000001, 0x80000001, 0x007fffff, 0x807fffff, 0x00400000,
                        0x00800000, 0x80800000, 0x7f7fffff, 0xff7fffff, 0x7f800000, 0xff800000, 0x3f800000,
                        0x33800000, 0x4b800000], np.uint32)
    sub = np.uint32(1) << np.arange(23, dtype=np.uint32)
    x = np.concatenate([bits, special, sub, sub | np.uint32(0x80000000), sub | np.uint32(0x00000001)])
    x = x.view(np.float32)
    x = x[~np.isnan(x)]  # NaN payloads are not part of the contract
    out = lm.probe_f2d(x)
    assert np.array_equal(out.view(np.uint64), x.astype(np.float64).view(np.uint64))
    assert np.isnan(lm.probe_f2d(np.array([np.nan], np.float32))[0])
