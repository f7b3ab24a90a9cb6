"""Bounded device waits made to run out, with no GPU fault and no hang.

The library's test hook (``mgb_set_test_wait_limit``) makes the FIRST bounded wait of a
kernel give up at once; every later wait, including the one that lets the kernel's own
bulk copies or tensor-core MMAs land before it leaves or frees tensor memory, keeps its
normal bound, so nothing the kernel issued is left in flight. The status bit reaches the
host (bit 2: a tile kernel's staged planes; bit 4: a contraction's MMAs), the results of
that launch are not taken, and the context stays usable.
"""

import numpy as np
import pytest

from meep_gpu_gb300 import FdtdDriver, Susceptibility, _lib
from tests import golden_io
from tests.golden.cases import CASES, build_case

TILES = (1, 64, 8, 8)


@pytest.fixture
def lib():
    lib = _lib.load()
    yield lib
    lib.mgb_set_test_wait_limit(0, -1)
    lib.mgb_set_test_wait_limit(1, -1)


def test_hook_refuses_an_unknown_wait_without_a_gpu(lib):
    assert lib.mgb_set_test_wait_limit(2, 0) == -1
    assert "which" in _lib.last_error(lib)
    assert lib.mgb_set_test_wait_limit(0, -5) == 0


@pytest.mark.gpu
def test_contraction_wait_that_runs_out_sets_bit_4_and_leaves_the_accumulators(gpu, lib):
    import torch

    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(3)
    nfreq, ncols, nsamples = 16, 1000, 8  # one 128-row phase tile
    samples = torch.from_numpy(rng.standard_normal((32, ncols)).astype(np.float32)).cuda()
    omega = torch.from_numpy(np.linspace(0.5, 3.0, nfreq)).cuda()
    acc0 = torch.from_numpy(rng.standard_normal((2 * nfreq, ncols)).astype(np.float32)).cuda()
    scratch = torch.empty(lib.mgb_dft_scratch_bytes(nfreq) // 4, dtype=torch.float32, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    args = (ncols, ncols, nsamples, omega.data_ptr(), nfreq, 10, 3, 0.05, 0, 0.5)

    def contract(acc):
        _lib.check(lib, lib.mgb_dft_contract(samples.data_ptr(), *args, acc.data_ptr(), scratch.data_ptr(),
                                             scratch.numel() * 4, stream))

    _lib.check(lib, lib.mgb_dft_contract_status(status.data_ptr(), 1, stream))
    _lib.check(lib, lib.mgb_set_test_wait_limit(1, 0))
    timed_out = acc0.clone()
    contract(timed_out)
    _lib.check(lib, lib.mgb_dft_contract_status(status.data_ptr(), 1, stream))
    torch.cuda.synchronize()
    assert int(status.item()) & 4
    assert torch.equal(timed_out, acc0)
    _lib.check(lib, lib.mgb_set_test_wait_limit(1, -1))
    done = acc0.clone()
    contract(done)
    _lib.check(lib, lib.mgb_dft_contract_status(status.data_ptr(), 0, stream))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    # the same sums in float64 on the host
    t = (10 + 3 * np.arange(nsamples)) * 0.05
    phase = np.outer(omega.cpu().numpy(), t)
    table = np.empty((2 * nfreq, nsamples))
    table[0::2], table[1::2] = np.cos(phase) * 0.5, np.sin(phase) * 0.5
    expected = acc0.cpu().numpy().astype(np.float64) + table @ samples.cpu().numpy()[:nsamples].astype(np.float64)
    scale = np.max(np.abs(table @ samples.cpu().numpy()[:nsamples]))
    assert np.max(np.abs(done.cpu().numpy() - expected)) <= 2e-6 * scale + 1e-6 * np.max(np.abs(expected))


@pytest.mark.gpu
def test_tile_wait_that_runs_out_is_reported_by_the_run(gpu, lib):
    case = CASES["tile_lorentz"]
    driver, _, _ = build_case(FdtdDriver, Susceptibility, case)
    driver.kernels = TILES
    driver.run(num_steps=3)
    assert driver.engine.uses_tiles
    _lib.check(lib, lib.mgb_set_test_wait_limit(0, 0))
    driver.step_many(1)
    _lib.check(lib, lib.mgb_set_test_wait_limit(0, -1))
    with pytest.raises(RuntimeError, match="tile kernel"):
        driver.engine.nonfinite()
    driver.close()
    # the context is still usable: the same case from the start gives the reference's words
    gold = golden_io.fields("tile_lorentz")
    again, _, _ = build_case(FdtdDriver, Susceptibility, case)
    again.kernels = TILES
    again.run(num_steps=case["steps"])
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        assert np.array_equal(again.get_field(c, cell_centered=False), gold[c]), c
    again.close()
