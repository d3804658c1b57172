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


@pytest.mark.parametrize("encoded", [True, False])
@pytest.mark.parametrize("fc1,fc2,T,DT,cpml", [(2.0, 10.0, 1.0, 1e-3, 5.0), (0.0, 0.0, 2.4, 2e-4, 8.0), (3.3, 7.1, 0.6, 5e-4, 6.0)])
def test_frequency_list_matches_restatement(encoded, fc1, fc2, T, DT, cpml, wave):
    from oracle import encode
    got = wave.encode_frequencies(encoded, fc1, fc2, T, DT, cpml)
    want = encode.frequencies(encoded, fc1, fc2, T, DT, cpml)
    np.testing.assert_array_equal(got, want)
    assert got.size > 0 and np.all(np.diff(got) > 0)


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("n,domains,seed", [(10, 3, 7), (24, 4, 12345), (9, 9, 1)])
def test_frequency_encoding_matches_restatement(mode, n, domains, seed, wave):
    """Every shot of a super-shot gets its own frequency of the encoded list;
    the assignment and the signs equal the time-domain encoding's."""
    from oracle import encode
    amp = np.linspace(1.0, 2.0, n).astype(np.float32)
    args = (2.0, 30.0, 1.2, 2.5e-4, 10.0)
    no, a, fc = wave.encode_sources_frequency(mode, domains, seed, amp, *args)
    want_no, want_a, want_fc = encode.encode_frequency(mode, domains, seed, amp, *args)
    np.testing.assert_array_equal(no, want_no)
    np.testing.assert_array_equal(a, want_a)
    np.testing.assert_array_equal(fc, want_fc)
    td_no, td_a = wave.encode_sources(mode, domains, seed, np.arange(1, n + 1), amp)
    np.testing.assert_array_equal(no, td_no)
    np.testing.assert_array_equal(a, td_a)
    flist = wave.encode_frequencies(True, *args)
    assert np.all(np.isin(fc, flist))
    for s in np.unique(no):
        assert len(set(fc[no == s].tolist())) == int(np.sum(no == s))


def test_frequency_encoding_needs_enough_frequencies(wave):
    # a narrow band (two encoded frequencies) for three shots per super-shot
    with pytest.raises(wave.WaveError):
        wave.encode_sources_frequency(3, 2, 0, np.ones(6, np.float32), 10.0, 12.0, 0.5, 1e-3, 5.0)
