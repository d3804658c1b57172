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


def test_device_bytes_cover_the_state_and_grow_with_the_acquisition(wave):
    """wave_device_bytes (ForwardSolver::estimateMemory): at least the nine
    wavefields, the three base materials and the CPML slabs of a 3-D elastic
    handle; receivers add their seismogram buffer."""
    NX = NY = NZ = 48
    cfg = wave.WaveConfig.make(dimension=3, equation="elastic", NX=NX, NY=NY, NZ=NZ, DH=5.0, DT=4e-4, T=0.04,
                               spatialFDorder=4, DampingBoundary=2, BoundaryWidth=8, NPower=4.0,
                               CenterFrequencyCPML=10.0, VMaxCPML=3500.0)
    s = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
    n = NX * NY * NZ
    b0 = s.estimateMemory()
    assert b0 >= (9 + 3) * n * 4
    s.prepareForModelling(dict(rho=np.full(n, 2000.0, np.float32), vp=np.full(n, 3000.0, np.float32),
                               vs=np.full(n, 1700.0, np.float32)))
    s.setReceivers(np.arange(1000, dtype=np.int64), np.full(1000, 2, np.int32))
    assert s.estimateMemory() >= b0 + 1000 * s.nt * 4
    s.close()
