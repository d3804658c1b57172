"""The reference's own known-answer unit tests for the source time functions
and the coordinate mapping, replayed against the library's C ABI (no GPU).

Wavelets: src/Tests/UnitTest/RickerUnitTest.cpp, SinWUnitTest.cpp,
FGaussianUnitTest.cpp, SinThreeUnitTest.cpp, IntgSinThreeUnitTest.cpp and
SpikeUnitTest.cpp each build a "sample result" from the formula and assert
that sample 3 of an NT = 4 trace equals the library's, and that negative NT,
DT or FC throw. The sample results are restated here in float64 numpy
(following each test's own loop); the library computes in single precision
like the reference's float instantiation, so equality is up to float32
rounding. The same formulas are also compared over whole traces with pulses
that span many samples, where a four-sample trace says little.

Coordinates: src/Tests/UnitTest/CoordinatesUnitTest.cpp:11-129
(locatedOnSurface, index2coordinate, coordinate2index and its range checks).
"""
import math

import numpy as np
import pytest


def ricker_kat(nt, dt, fc, amp, ts):          # RickerUnitTest.cpp:20-31
    t = np.arange(nt) * dt
    tau = (t - (1.5 / fc + ts)) * math.pi * fc
    h = tau * tau
    return amp * (1.0 - 2.0 * h) * np.exp(-h)


def fgaussian_kat(nt, dt, fc, amp, ts):       # FGaussianUnitTest.cpp:20-30
    t = np.arange(nt) * dt
    tau = (t - (1.2 / fc + ts)) * math.pi * fc
    return amp * (-2.0 * tau) * np.exp(-tau * tau)


def _pulse_span(nt, dt, fc, ts):
    i1 = math.floor(ts / dt)
    return i1, i1 + math.floor(1.0 / fc / dt)


def sinw_kat(nt, dt, fc, amp, ts):            # SinWUnitTest.cpp:20-40
    zero, help_ = np.zeros(nt), np.zeros(nt)
    i1, i2 = _pulse_span(nt, dt, fc, ts)
    for count, i in enumerate(range(i1, i2 + 1)):
        if i >= nt:
            break
        a = 2.0 * count * dt * math.pi * fc
        help_[i] = math.sin(a)
        zero[i] = math.sin(2.0 * a)
    return amp * (help_ - zero / 2.0)


def sinthree_kat(nt, dt, fc, amp, ts):        # SinThreeUnitTest.cpp:20-34
    zero = np.zeros(nt)
    i1, i2 = _pulse_span(nt, dt, fc, ts)
    for count, i in enumerate(range(i1, i2 + 1)):
        if i >= nt:
            break
        zero[i] = math.sin(count * dt * math.pi * fc) ** 3
    return amp * zero


def intgsinthree_kat(nt, dt, fc, amp, ts):    # IntgSinThreeUnitTest.cpp:20-44
    zero, help_ = np.zeros(nt), np.zeros(nt)
    i1, i2 = _pulse_span(nt, dt, fc, ts)
    for count, i in enumerate(range(i1, i2 + 1)):
        if i >= nt:
            break
        c = math.cos(count * dt * math.pi * fc)
        help_[i] = c
        zero[i] = c ** 3
    z = 0.5 + (0.25 * zero - 0.75 * help_)       # the 0.5 ("half") spans the whole trace
    return amp * (z / fc / math.pi / 0.75)


def spike_kat(nt, dt, fc, amp, ts):           # SpikeUnitTest.cpp:20-27 (the formula; the test then calls SinW)
    h = np.zeros(nt)
    h[math.floor(ts / dt)] = 1.0
    return amp * h


KATS = {1: ricker_kat, 2: sinw_kat, 3: sinthree_kat, 4: fgaussian_kat, 5: spike_kat, 6: intgsinthree_kat}
# (NT, DT, FC, AMP, Tshift) of each unit test's TestConstructor
UNIT_ARGS = {1: (4, 1.0, 1.0, 1.0, 0.0), 2: (4, 1.0, 1.0, 1.0, 0.0), 3: (4, 1.0, 1.0, 1.0, 0.0),
             4: (4, 10.0, 1.0, 1.0, 0.0), 5: (4, 1.0, 1.0, 1.0, 0.0), 6: (4, 1.0, 1.0, 1.0, 0.0)}


def _close(got, want, amp):
    return np.allclose(got, want, rtol=2e-6, atol=2e-6 * abs(amp))


@pytest.mark.parametrize("shape", sorted(KATS))
def test_wavelet_unit_test_sample_three(wave, shape):
    nt, dt, fc, amp, ts = UNIT_ARGS[shape]
    want = KATS[shape](nt, dt, fc, amp, ts)
    got = wave.wavelet(shape, nt, dt, fc, amp, ts)
    assert _close(got[3], want[3], amp), (shape, got, want)
    assert _close(got, want, amp)
    if shape == 5:
        # SpikeUnitTest.cpp:29-37 asserts SinW's sample 3 against the spike formula
        assert _close(wave.wavelet(2, nt, dt, fc, amp, ts)[3], want[3], amp)


@pytest.mark.parametrize("shape", sorted(KATS))
@pytest.mark.parametrize("args", [(400, 1e-3, 10.0, 2.0, 0.0505), (1200, 2e-4, 15.0, 1.0, 0.0131), (300, 7e-11, 2e8, 1.0, 0.0)])
def test_wavelet_formulas_over_whole_traces(wave, shape, args):
    # Tshift/DT stays half a sample away from an integer: floor(Tshift/DT) in
    # float32 (the library, like the reference's float build) and in float64
    # (this restatement) may differ by one sample when the quotient is whole
    nt, dt, fc, amp, ts = args
    # the reference's float build receives DT, FC, Tshift rounded to float32; the
    # pulse's sample span (floor(1/FC/DT)) depends on that rounding
    r = lambda v: float(np.float32(v))
    want = KATS[shape](nt, r(dt), r(fc), r(amp), r(ts))
    got = wave.wavelet(shape, nt, dt, fc, amp, ts)
    assert np.abs(want).max() > 0
    # the time argument is formed in float32 (t = k*DT), so the phase error grows with t
    assert np.allclose(got, want, rtol=1e-4, atol=1e-4 * abs(amp) * np.abs(want).max()), shape


@pytest.mark.parametrize("shape", [1, 2, 3, 4, 6])
def test_wavelet_argument_asserts(wave, shape):
    """TestAsserts of each unit test: negative NT, DT or FC are errors."""
    import ctypes
    out = np.zeros(4, np.float32)
    ptr = out.ctypes.data_as(ctypes.c_void_p)
    for nt, dt, fc in ((-4, 10.0, 1.0), (4, -10.0, 1.0), (4, 10.0, -1.0)):
        assert wave.lib().wave_wavelet(shape, nt, dt, fc, 1.0, 0.0, ptr) == wave.WAVE_ERR_ARG, (nt, dt, fc)


def _cfg(wave, NX, NY, NZ):
    return wave.WaveConfig.make(dimension=3, equation="acoustic", NX=NX, NY=NY, NZ=NZ, DH=1.0, DT=1e-3, T=0.01,
                                spatialFDorder=2)


def test_coordinates_located_on_surface(wave):
    """CoordinatesUnitTest.cpp:11-27: indices 2 and 52 of a 5 x 10 x 15 grid lie
    on the surface (y = 0), index 80 does not."""
    x, y, z, _ = wave.grid_coordinates(_cfg(wave, 5, 10, 15))
    assert y[2] == 0 and y[52] == 0 and y[80] != 0


def test_coordinates_index2coordinate(wave):
    """CoordinatesUnitTest.cpp:29-61: index 112 of a 5 x 15 x 10 grid is (2, 2, 2)."""
    x, y, z, _ = wave.grid_coordinates(_cfg(wave, 5, 15, 10))
    assert (x[112], y[112], z[112]) == (2, 2, 2)
    n = 5 * 15 * 10
    i = np.arange(n)
    assert np.array_equal(i, x + 5 * z + 5 * 10 * y)


def test_coordinates_coordinate2index_and_range_checks(wave):
    """CoordinatesUnitTest.cpp:63-98: (4, 2, 3) maps to 119 on a 5 x 15 x 10
    grid; coordinates outside the grid are errors."""
    cfg = _cfg(wave, 5, 15, 10)
    assert wave.grid_index(cfg, 4, 2, 3) == 119
    for bad in ((4, 2, 30), (4, 16, 3), (8, 2, 3), (-4, 2, 3), (4, -2, 3), (4, 2, -3)):
        with pytest.raises(wave.WaveError):
            wave.grid_index(cfg, *bad)
