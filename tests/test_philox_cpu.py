"""Philox4x32-10 against the known-answer vectors published with Random123
(Salmon et al., SC'11): numpy and C++ oracle implementations."""
import numpy as np

import philox_np
from oracle import oracle_api as orc

KAT = [((0, 0, 0, 0, 0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
       ((0xffffffff,) * 6, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
       ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344, 0xa4093822, 0x299f31d0),
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]


def test_numpy_kat():
    for a, e in KAT:
        o = philox_np.philox4x32_10(*[np.array([x], np.uint32) for x in a[:4]], a[4], a[5])
        assert tuple(int(x[0]) for x in o) == e


def test_oracle_matches_numpy():
    a = orc.uniforms(123456789012345, 1000, 8, first=(1 << 33) + 5, stream=9)
    b = philox_np.uniforms(123456789012345, 1000, 8, first=(1 << 33) + 5, stream=9)
    assert np.array_equal(a, b)
    assert a.min() >= 0.0 and a.max() < 1.0
