"""The allocation-free contraction entry point (static phase-table scratch) against the
entry point that takes caller scratch: identical words, twice in a row, across sizes."""

import numpy as np
import pytest

from meep_gpu_gb300 import _lib


def test_noalloc_refuses_sizes_beyond_the_maximum_before_touching_the_device():
    lib = _lib.load()
    assert lib.mgb_dft_contract_noalloc(None, 4, 4, 1, None, _lib.MGB_DFT_MAX_FREQ + 1, 0, 1, 0.1, 0,
                                        1.0, None, None) == -1
    assert "nfreq" in _lib.last_error(lib)
    assert lib.mgb_dft_contract_noalloc(None, 4, 4, _lib.MGB_DFT_DEPTH + 1, None, 4, 0, 1, 0.1, 0,
                                        1.0, None, None) == -1
    assert "nsamples" in _lib.last_error(lib)


@pytest.mark.gpu
def test_noalloc_equals_the_scratch_entry_point_twice_in_a_row(gpu):
    import torch

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    for nfreq, ncols, nsamples in ((64, 700, 32), (512, 300, 17), (3, 1, 1)):
        ld = ncols + 5
        samples = torch.from_numpy(rng.standard_normal((32, ld)).astype(np.float32)).cuda()
        omega = torch.from_numpy(np.linspace(0.5, 3.0, nfreq)).cuda()
        acc0 = torch.from_numpy(rng.standard_normal((2 * nfreq, ncols)).astype(np.float32)).cuda()
        args = (ld, ncols, nsamples, omega.data_ptr(), nfreq, 98, 49, 0.05, 1, 0.3)
        scratch = torch.empty(lib.mgb_dft_scratch_bytes(nfreq) // 4, dtype=torch.float32, device="cuda")
        expected = acc0.clone()
        _lib.check(lib, lib.mgb_dft_contract(samples.data_ptr(), *args, expected.data_ptr(), scratch.data_ptr(),
                                             scratch.numel() * 4, stream))
        for _ in range(2):
            got = acc0.clone()
            _lib.check(lib, lib.mgb_dft_contract_noalloc(samples.data_ptr(), *args, got.data_ptr(), stream))
            torch.cuda.synchronize()
            assert torch.equal(got, expected), (nfreq, ncols, nsamples)
        assert not torch.equal(expected, acc0)
