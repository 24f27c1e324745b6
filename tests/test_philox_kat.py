"""Philox4x32-10 pinned to the known-answer vectors published with the
generator (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
1, 2, 3", SC'11; the kat_vectors file of the Random123 distribution): the
numpy restatement the noise test uses (CPU) and the device generator behind
cageo_noise_philox (GPU, through the C ABI) must both reproduce them."""
import numpy as np
import pytest

from cases import philox_np

# (counter c0..c3, key k0 k1) -> output words, Philox4x32 with 10 rounds.
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_numpy_restatement_matches_published_vectors(ctr, key, want):
    got = philox_np([np.array([c], np.uint64) for c in ctr], key)
    assert tuple(int(w[0]) for w in got) == want


@pytest.mark.gpu
@pytest.mark.parametrize("ctr,key,want", KAT)
def test_device_generator_matches_published_vectors(cuda, ctr, key, want):
    from cageo_gb300 import api
    got = api.philox4x32_10(ctr, key, n=1)
    assert tuple(int(w) for w in got[0]) == want


@pytest.mark.gpu
def test_device_generator_counter_stream(cuda):
    """Consecutive blocks advance the first counter word (the layout the
    noise kernel uses for cells), equal to the pinned restatement."""
    from cageo_gb300 import api
    ctr, key, n = (0xfffffff0, 7, 0x63616765, 0), (0x12345678, 0x9abc), 40
    got = api.philox4x32_10(ctr, key, n=n)
    c0 = (np.arange(n, dtype=np.uint64) + ctr[0]) & np.uint64(0xFFFFFFFF)
    ref = philox_np([c0, np.full(n, ctr[1], np.uint64), np.full(n, ctr[2], np.uint64),
                     np.full(n, ctr[3], np.uint64)], key)
    assert np.array_equal(got, np.stack([r.astype(np.uint32) for r in ref], axis=1))
