"""The host restatement of Philox4x32-10 used to check the on-device sampler
(CPU test): it reproduces the generator's published known-answer vectors."""
import numpy as np

from philox_ref import philox4x32_10

# (counter, key) -> output words, the published known answers of Philox4x32-10
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_philox_known_answers():
    for ctr, key, expect in KAT:
        out = philox4x32_10([np.array([c], dtype=np.uint64) for c in ctr], key)
        assert tuple(int(w[0]) for w in out) == expect
