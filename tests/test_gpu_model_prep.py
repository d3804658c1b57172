"""Device model preparation helpers against a numpy restatement of the
reference's harmonic S-modulus average (ModelparameterSeismic.cpp:421-432 with
the averaging-matrix edge fallbacks of Modelparameter.cpp:336-527)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def harmonic_reference(mu, NX, NY, NZ, mode):
    m = np.where(mu < 1.0, 1.0, mu).astype(np.float32).reshape(NY, NZ, NX)
    inv = (np.float32(1.0) / m).astype(np.float32)
    out = np.zeros_like(inv)
    for y in range(NY):
        for z in range(NZ):
            for x in range(NX):
                if mode >= 3:
                    nx, ny = (x + 1, y) if mode == 3 else (x, y + 1)
                    inn = nx < NX and ny < NY
                    s = np.float32(0.5) * inv[y, z, x] + np.float32(0.5) * inv[ny, z, nx] if inn else inv[y, z, x]
                else:
                    p2, p3, p4 = {0: ((x + 1, y, z), (x, y + 1, z), (x + 1, y + 1, z)),
                                  1: ((x + 1, y, z), (x, y, z + 1), (x + 1, y, z + 1)),
                                  2: ((x, y + 1, z), (x, y, z + 1), (x, y + 1, z + 1))}[mode]
                    mx, my, mz = max(x, p2[0], p3[0], p4[0]), max(y, p2[1], p3[1], p4[1]), max(z, p2[2], p3[2], p4[2])
                    ix, iy, iz = mx < NX, my < NY, mz < NZ
                    v = lambda p: inv[p[1], p[2], p[0]]
                    if ix and iy and iz:
                        s = np.float32(0.25) * inv[y, z, x] + np.float32(0.25) * v(p2) + np.float32(0.25) * v(p3) + np.float32(0.25) * v(p4)
                    elif ix and not iy and iz:      # bottom side: (maxX, y, maxZ)
                        s = np.float32(0.5) * inv[y, mz, mx] + np.float32(0.5) * inv[y, z, x]
                    elif not ix and iy and iz:      # right side: (x, maxY, maxZ)
                        s = np.float32(0.5) * inv[my, mz, x] + np.float32(0.5) * inv[y, z, x]
                    elif ix and iy and not iz:      # back side: (maxX, maxY, z)
                        s = np.float32(0.5) * inv[my, z, mx] + np.float32(0.5) * inv[y, z, x]
                    else:
                        s = inv[y, z, x]
                r = np.float32(1.0) / np.float32(s)
                out[y, z, x] = 0.0 if r < 4.0 else r
    return out.reshape(-1)


@pytest.mark.parametrize("mode,dims", [(0, (9, 7, 5)), (1, (8, 6, 7)), (2, (7, 9, 6)), (3, (11, 8, 1)), (4, (10, 9, 1)), (0, (12, 10, 1))])
def test_average_shear_modulus_matches_reference_rules(wave, mode, dims):
    rng = np.random.default_rng(mode)
    n = int(np.prod(dims))
    mu = rng.uniform(0.0, 3e9, n).astype(np.float32)
    mu[rng.integers(0, n, n // 5)] = 0.0          # vacuum / fluid cells
    mu[rng.integers(0, n, n // 10)] = 3.0         # below the 4.0 threshold after averaging
    got = wave.average_shear_modulus(mu, dims, mode)
    ref = harmonic_reference(mu, *dims, mode)
    assert np.allclose(got, ref, rtol=1e-6, atol=0.0)


def test_average_shear_modulus_device_pointers(wave):
    torch = pytest.importorskip("torch")
    dims = (16, 12, 10)
    mu = np.random.default_rng(3).uniform(1e8, 3e9, int(np.prod(dims))).astype(np.float32)
    host = wave.average_shear_modulus(mu, dims, 1)
    dev = wave.average_shear_modulus(torch.from_numpy(mu).cuda(), dims, 1).cpu().numpy()
    assert np.array_equal(host, dev)
