"""Source encoding (wave_encode_sources, host only) against the restatement of
Sources.cpp:569-660 in oracle/encode.py, and the super-shot invariants."""
import numpy as np
import pytest


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("n,domains,seed", [(10, 3, 7), (24, 4, 12345), (5, 5, 1), (17, 2, 2024)])
def test_encoding_matches_restatement(mode, n, domains, seed, wave):
    from oracle import encode
    amp = np.linspace(1.0, 2.0, n).astype(np.float32)
    no, a = wave.encode_sources(mode, domains, seed, np.arange(1, n + 1), amp)
    want_no, want_a = encode.encode(mode, domains, seed, amp)
    np.testing.assert_array_equal(no, want_no)
    np.testing.assert_array_equal(a, want_a)
    # every super-shot gets at most ceil(n / domains) shots, every one at least one
    per = int(np.ceil(n / domains))
    ids, counts = np.unique(no, return_counts=True)
    assert len(ids) == domains and counts.max() <= per
    assert np.all(ids == domains * 10000 + 1 + np.arange(domains))
    assert np.all(np.abs(a) == amp)
    if mode != 1:
        np.testing.assert_array_equal(a, amp)


def test_encoding_rejects_more_domains_than_shots(wave):
    with pytest.raises(wave.WaveError):
        wave.encode_sources(2, 5, 0, np.arange(3), np.ones(3, np.float32))
