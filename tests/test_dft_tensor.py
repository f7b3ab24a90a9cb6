"""Tensor-core DFT accumulation (tcgen05, 3xTF32) against float64 sums and against the
step-by-step path.

The contraction adds sum_k phase[f][k] * sample[k][n] to every accumulator; its phases
are the float32 words the step-by-step path forms (float64 sincos, rounded once), so
the float64 reference below uses those same words and the only differences are the
3xTF32 products and the summation order: the bar is a relative error of 2e-6 of the
largest contribution. A monitor accumulated either way must give the same spectrum to
float32 rounding (1e-5 of its peak) and the same float64-oracle flux error.
"""

import ctypes

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility, _lib

pytestmark = pytest.mark.gpu


def phase_words(omega, nfreq, first, stride, dt, half_back, scale, nsamples):
    k = np.arange(nsamples)
    t = (first + k * stride).astype(np.float64) * dt
    if half_back:
        t = t - 0.5 * dt
    arg = t[None, :] * omega[:nfreq, None]
    cos = (np.cos(arg) * scale).astype(np.float32).astype(np.float64)
    sin = (np.sin(arg) * scale).astype(np.float32).astype(np.float64)
    table = np.empty((2 * nfreq, nsamples))
    table[0::2] = cos
    table[1::2] = sin
    return table


def contract(torch, samples, ld, ncols, nsamples, omega, nfreq, first, stride, dt, half_back, scale, acc):
    lib = _lib.load()
    scratch = torch.empty(lib.mgb_dft_scratch_bytes(nfreq) // 4, dtype=torch.float32, device="cuda")
    _lib.check(lib, lib.mgb_dft_contract(samples.data_ptr(), ld, ncols, nsamples, omega.data_ptr(), nfreq,
                                         first, stride, dt, half_back, scale, acc.data_ptr(),
                                         scratch.data_ptr(), scratch.numel() * 4,
                                         torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()


@pytest.mark.parametrize("nfreq,ncols,nsamples", [(1, 1, 1), (50, 257, 32), (64, 256, 7),
                                                  (100, 1000, 32), (200, 513, 19), (512, 300, 32)])
def test_contraction_matches_float64_sums(gpu, nfreq, ncols, nsamples):
    import torch

    rng = np.random.default_rng(nfreq * 1000 + ncols)
    ld = ncols + 3
    samples = rng.standard_normal((32, ld)).astype(np.float32)
    omega = np.sort(rng.uniform(0.5, 8.0, nfreq))
    acc0 = rng.standard_normal((2 * nfreq, ncols)).astype(np.float32)
    first, stride, dt, half_back, scale = 49, 49, 0.05, 1, 0.05 * 49 / np.sqrt(2 * np.pi)
    d_samples = torch.from_numpy(samples).cuda()
    d_omega = torch.from_numpy(omega).cuda()
    d_acc = torch.from_numpy(acc0.copy()).cuda()
    contract(torch, d_samples, ld, ncols, nsamples, d_omega, nfreq, first, stride, dt, half_back, scale, d_acc)
    got = d_acc.cpu().numpy().astype(np.float64)
    table = phase_words(omega, nfreq, first, stride, dt, half_back, scale, nsamples)
    update = table @ samples[:nsamples, :ncols].astype(np.float64)
    expected = acc0.astype(np.float64) + update
    # each accumulator word is rounded to float32 once after the add
    bound = 2e-6 * np.max(np.abs(table)) * np.max(np.abs(samples[:nsamples, :ncols])) * nsamples
    err = np.max(np.abs(got - expected) - 1.2e-7 * np.abs(expected))
    assert err <= bound, (err, bound)


def test_contraction_of_no_samples_leaves_the_accumulators(gpu):
    import torch

    acc = torch.ones((2 * 4, 10), dtype=torch.float32, device="cuda")
    samples = torch.ones((32, 10), dtype=torch.float32, device="cuda")
    omega = torch.ones(4, dtype=torch.float64, device="cuda")
    contract(torch, samples, 10, 10, 0, omega, 4, 1, 1, 0.1, 0, 1.0, acc)
    assert torch.all(acc == 1)


def test_contraction_refuses_bad_sizes(gpu):
    import torch

    lib = _lib.load()
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    ptr = buf.data_ptr()
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.mgb_dft_contract(ptr, 4, 4, 33, ptr, 1, 0, 1, 0.1, 0, 1.0, ptr, ptr, 4096, stream) == -1
    assert lib.mgb_dft_contract(ptr, 4, 4, 1, ptr, 513, 0, 1, 0.1, 0, 1.0, ptr, ptr, 1 << 30, stream) == -1
    assert lib.mgb_dft_contract(ptr, 4, 4, 1, ptr, 8, 0, 1, 0.1, 0, 1.0, ptr, ptr, 16, stream) == -1
    # one 128-row tile of 32 samples, each phase as its two TF32 parts
    assert lib.mgb_dft_scratch_bytes(0) == 0 and lib.mgb_dft_scratch_bytes(64) == 128 * 32 * 4 * 2
    assert lib.mgb_dft_scratch_bytes(65) == 2 * 128 * 32 * 4 * 2
    # a scratch that is not 16-byte aligned is refused before the device is touched
    assert lib.mgb_dft_contract(ptr, 4, 4, 1, ptr, 8, 0, 1, 0.1, 0, 1.0, ptr, ptr + 4, 1 << 20, stream) == -1


def sphere(dft_accumulation, steps):
    d = FdtdDriver((3.2, 3.2, 3.2), 10, force_complex_fields=False, boundaries="metallic",
                   kernels=(0, 32, 4, 4), dft_accumulation=dft_accumulation)
    d.setup_pml(6)
    x, y, z = d.grid.meshgrid()
    d.set_epsilon(np.where(x * x + y * y + z * z < 0.7 ** 2, 6.0, 1.0).astype(np.float32))
    d.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05),
                         np.where(np.abs(x) < 0.3, 0.5, 0.0).astype(np.float32))
    d.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.8, 0.1, 0.0),
                  "size": (0, 0, 0), "frequency": 0.3, "fwidth": 0.3})
    flux = d.add_flux_monitor(fcen=0.3, df=0.3, nfreq=70, center=(0.8, 0, 0), size=(0, 1.8, 1.8),
                              decimation_factor=3)
    vol = d.add_dft_monitor(fcen=0.3, df=0.2, nfreq=40, components=("Ex", "Hy", "Ez"),
                            center=(0.1, 0, 0), size=(0.8, 0.6, 0.5), decimation_factor=2)
    d.step_many(steps)
    return d, flux, vol


@pytest.mark.parametrize("steps", [200, 61])  # a full buffer count, and one left pending
def test_monitor_tensor_mode_equals_direct_mode(gpu, steps):
    a, fa, va = sphere("tensor", steps)
    b, fb, vb = sphere("direct", steps)
    assert a.engine.dft_accumulation == "tensor" and b.engine.dft_accumulation == "direct"
    lib = _lib.load()
    assert lib.mgb_dft_pending(a.engine.handle, 0) == (steps // 3) % 32
    sa, sb = fa.get_flux_spectrum(), fb.get_flux_spectrum()
    assert np.max(np.abs(sa - sb)) <= 1e-5 * np.max(np.abs(sb))
    assert lib.mgb_dft_pending(a.engine.handle, 0) == 0
    for c in ("Ex", "Hy", "Ez"):
        ra, rb = va.raw(c), vb.raw(c)
        assert np.max(np.abs(ra - rb)) <= 1e-5 * np.max(np.abs(rb)), c
    assert int(a.engine.status.item()) == 0
    # the fields are not touched by the accumulation mode
    assert np.array_equal(a.get_field("Ez", cell_centered=False), b.get_field("Ez", cell_centered=False))
    a.close()
    b.close()


def test_tensor_mode_flux_against_float64_oracle(gpu):
    from oracle.oracle import Oracle, problem_from_driver

    steps = 300
    d, flux, _ = sphere("tensor", steps)
    got = flux.get_flux_spectrum()
    ref = FdtdDriver((3.2, 3.2, 3.2), 10, force_complex_fields=False, boundaries="metallic")
    # same configuration, built again for the oracle (host arrays only)
    ref.setup_pml(6)
    x, y, z = ref.grid.meshgrid()
    ref.set_epsilon(np.where(x * x + y * y + z * z < 0.7 ** 2, 6.0, 1.0).astype(np.float32))
    ref.add_susceptibility(Susceptibility(frequency=1.1, gamma=0.05),
                           np.where(np.abs(x) < 0.3, 0.5, 0.0).astype(np.float32))
    ref.add_source({"source_type": "gaussian", "component": "Ez", "center": (-0.8, 0.1, 0.0),
                    "size": (0, 0, 0), "frequency": 0.3, "fwidth": 0.3})
    ref.add_flux_monitor(fcen=0.3, df=0.3, nfreq=70, center=(0.8, 0, 0), size=(0, 1.8, 1.8),
                         decimation_factor=3)
    ref.add_dft_monitor(fcen=0.3, df=0.2, nfreq=40, components=("Ex", "Hy", "Ez"),
                        center=(0.1, 0, 0), size=(0.8, 0.6, 0.5), decimation_factor=2)
    oracle = Oracle(problem_from_driver(ref), "f64")
    oracle.run(steps)
    expected = oracle.flux_spectrum(0)
    rel = np.max(np.abs(got - expected)) / np.max(np.abs(expected))
    assert rel <= 1e-4, rel
    d.close()
