"""The allocation-free shear-modulus average (wave_average_shear_modulus_noalloc)
against the allocating entry point (wave_average_shear_modulus), both through
the C ABI with device pointers. The reference has no counterpart of the
allocation-free form; the averaging rules are ModelparameterSeismic.cpp:421-432
with the edge fallbacks of Modelparameter.cpp:336-527."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6   # same kernels on both paths: the results agree to the last bit in practice


def _mu(rng, n):
    mu = rng.uniform(5e8, 3e10, n).astype(np.float32)
    mu[rng.random(n) < 0.05] = 0.0     # vacuum cells: clamped to 1 before inversion
    mu[rng.random(n) < 0.02] = 0.5
    return mu


@pytest.mark.parametrize("mode", range(5))
def test_noalloc_matches_allocating_entry_point_on_two_calls(wave, mode):
    torch = pytest.importorskip("torch")
    dims = (40, 30, 20)
    n = int(np.prod(dims))
    rng = np.random.default_rng(100 + mode)
    for call in range(2):
        mu = torch.from_numpy(_mu(rng, n)).cuda()
        ref = wave.average_shear_modulus(mu, dims, mode)
        out = torch.full_like(mu, float("nan"))
        wave.average_shear_modulus_noalloc(mu, out, dims, mode)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=RTOL, atol=0,
                                   err_msg=f"call {call}, mode {mode}")


def test_noalloc_on_a_side_stream_and_in_place(wave):
    torch = pytest.importorskip("torch")
    dims = (64, 33, 17)
    n = int(np.prod(dims))
    mu = torch.from_numpy(_mu(np.random.default_rng(7), n)).cuda()
    ref = wave.average_shear_modulus(mu, dims, 1)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    work = mu.clone()
    side.wait_stream(torch.cuda.current_stream())
    wave.average_shear_modulus_noalloc(work, work, dims, 1, stream=side.cuda_stream)
    side.synchronize()
    np.testing.assert_allclose(work.cpu().numpy(), ref.cpu().numpy(), rtol=RTOL, atol=0)


def test_noalloc_rejects_models_above_its_scratch_and_host_memory(wave):
    torch = pytest.importorskip("torch")
    small = torch.ones(16, device="cuda")
    ptr = ctypes.c_void_p(small.data_ptr())
    # 4,227,072 > 2^22 points: the C ABI refuses before it touches the pointers
    rc = wave.lib().wave_average_shear_modulus_noalloc(ptr, ptr, 256, 128, 129, 0, None)
    assert rc == wave.WAVE_ERR_ARG
    assert b"exceeds the fixed scratch" in wave.lib().wave_last_error(None)
    host = np.ones(16, dtype=np.float32)
    rc = wave.lib().wave_average_shear_modulus_noalloc(host.ctypes.data_as(ctypes.c_void_p), host.ctypes.data_as(ctypes.c_void_p),
                                                       4, 2, 2, 0, None)
    assert rc == wave.WAVE_ERR_ARG
    assert b"device memory" in wave.lib().wave_last_error(None)


def test_noalloc_wrapper_rejects_short_or_mistyped_tensors_before_any_launch(wave):
    """A tensor shorter than NX*NY*NZ would be read or written past its end by
    the kernels (the C ABI cannot see its length): the wrapper refuses it, and
    the output tensor stays untouched."""
    torch = pytest.importorskip("torch")
    small = torch.ones(16, device="cuda")
    big = torch.full((100 * 100 * 100,), 7.0, device="cuda")
    for mu, out in ((small, big), (big, small)):
        with pytest.raises(wave.WaveError) as e:
            wave.average_shear_modulus_noalloc(mu, out, (100, 100, 100), 0)
        assert "fewer than NX*NY*NZ" in str(e.value)
    with pytest.raises(wave.WaveError):
        wave.average_shear_modulus_noalloc(big.double(), big, (100, 100, 100), 0)
    with pytest.raises(wave.WaveError):
        wave.average_shear_modulus_noalloc(big.view(100, 10000)[:, :100], big, (10, 10, 100), 0)
    torch.cuda.synchronize()
    assert bool((big == 7.0).all())
