"""File formats around the time step (host code, no GPU): MatrixMarket
reading/writing (IO.hpp:21-145) against the reference's own golden files and
the oracle's reader, and the SeismicUnix trace headers of SUIO::writeSU
(SUIO.hpp:156-262)."""
import glob
import os
import struct

import numpy as np
import pytest

from oracle import refcpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ci")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "seismogram.*.mtx")))[:6])
def test_read_mtx_matches_the_oracle_reader_on_reference_goldens(wave, path):
    a = wave.read_mtx(path)
    b = refcpu.read_mtx_array(path)
    assert a.shape == b.shape
    assert np.array_equal(a, b.astype(np.float32))


def test_write_read_mtx_round_trip(wave, tmp_path):
    rng = np.random.default_rng(5)
    m = (rng.standard_normal((7, 33)) * 10 ** rng.uniform(-20, 20, (7, 33))).astype(np.float32)
    p = str(tmp_path / "m.mtx")
    wave.write_mtx(p, m)
    assert np.array_equal(wave.read_mtx(p), m)
    assert np.array_equal(refcpu.read_mtx_array(p).astype(np.float32), m)
    v = rng.standard_normal(50).astype(np.float32)
    wave.write_mtx(p, v)
    assert np.array_equal(wave.read_mtx(p)[:, 0], v)


def test_read_mtx_coordinate_format(wave, tmp_path):
    p = tmp_path / "c.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% comment\n3 2 3\n1 1 1.5\n3 2 -2\n2 1 4e-3\n")
    a = wave.read_mtx(str(p))
    assert np.array_equal(a, np.array([[1.5, 0], [4e-3, 0], [0, -2]], np.float32))


def test_read_mtx_errors(wave, tmp_path):
    with pytest.raises(wave.WaveError):
        wave.read_mtx(str(tmp_path / "missing.mtx"))
    p = tmp_path / "bad.mtx"
    p.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n")
    with pytest.raises(wave.WaveError):
        wave.read_mtx(str(p))


def test_write_su_headers_and_samples(wave, tmp_path):
    NX, NY, NZ, DH = 50, 40, 1, 2.5
    ntr, ns, dt = 3, 17, 2e-4
    data = np.arange(ntr * ns, dtype=np.float32).reshape(ntr, ns)
    rec = np.array([4 + NX * 3, 20 + NX * 3, 40 + NX * 10], np.int64)
    src = 10 + NX * 5
    p = str(tmp_path / "s.su")
    wave.write_su(p, data, dt, rec, src, (NX, NY, NZ), DH)
    raw = open(p, "rb").read()
    assert len(raw) == ntr * (240 + 4 * ns)
    xs, ys = 10 * DH, 5 * DH
    for t in range(ntr):
        h = raw[t * (240 + 4 * ns):t * (240 + 4 * ns) + 240]
        xr, yr = (rec[t] % NX) * DH, (rec[t] // NX) * DH
        assert struct.unpack_from("<i", h, 0)[0] == t + 1                       # tracl
        assert struct.unpack_from("<i", h, 20)[0] == ntr                        # cdp
        assert struct.unpack_from("<i", h, 36)[0] == round(np.hypot(xs - xr, ys - yr) * 1000)   # offset (mm)
        assert struct.unpack_from("<i", h, 40)[0] == round(yr * 1000)           # gelev
        assert struct.unpack_from("<hh", h, 68) == (-3, -3)                     # scalel, scalco
        assert struct.unpack_from("<i", h, 72)[0] == round(xs * 1000)           # sx
        assert struct.unpack_from("<i", h, 80)[0] == round(xr * 1000)           # gx
        assert struct.unpack_from("<HH", h, 114) == (ns, round(dt * 1e6))       # ns, dt (us)
        assert abs(struct.unpack_from("<f", h, 180)[0] - dt) < 1e-9             # d1
        assert struct.unpack_from("<i", h, 204)[0] == ntr                       # ntr
        samples = np.frombuffer(raw, dtype="<f4", count=ns, offset=t * (240 + 4 * ns) + 240)
        assert np.array_equal(samples, data[t])
