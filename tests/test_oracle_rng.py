"""Philox4x32-10 known-answer vectors (Salmon et al., SC'11; Random123
kat_vectors) and the engine's counter layout."""
import numpy as np

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers(oracle):
    for ctr, key, expected in KAT:
        out = np.zeros(4, np.uint32)
        oracle.lib().orc_philox4x32(*ctr, *key, out)
        assert tuple(int(x) for x in out) == expected


def test_uniform_and_start_ranges(oracle):
    lib = oracle.lib()
    key = lib.orc_colony_key(17, 1234)
    u = [lib.orc_uniform(key, b, a, s) for b in range(3) for a in range(5) for s in range(1, 50)]
    assert all(0.0 <= x < 1.0 for x in u) and len(set(u)) == len(u)
    assert abs(np.mean(u) - 0.5) < 0.05
    starts = [lib.orc_start_node(key, b, a, 7) for b in range(50) for a in range(20)]
    assert set(starts) == set(range(7))
    assert 0.0 <= lib.orc_source_uniform(key, 3) < 1.0
