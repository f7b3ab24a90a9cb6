"""The allocation-free contraction entry point (static phase-table scratch) against the
entry point that takes caller scratch: identical words, twice in a row, across sizes,
with no device memory taken by the calls."""

import gc
import re
from pathlib import Path

import numpy as np
import pytest

from meep_gpu_gb300 import _lib

SOURCE = Path(__file__).resolve().parent.parent / "meep_gpu_gb300" / "csrc" / "meepgb.cu"


def test_noalloc_refuses_bad_arguments_before_touching_the_device():
    lib = _lib.load()
    assert lib.mgb_dft_contract_noalloc(None, 4, 4, 1, None, _lib.MGB_DFT_MAX_FREQ + 1, 0, 1, 0.1, 0,
                                        1.0, None, None) == -1
    assert "nfreq" in _lib.last_error(lib)
    assert lib.mgb_dft_contract_noalloc(None, 4, 4, _lib.MGB_DFT_DEPTH + 1, None, 4, 0, 1, 0.1, 0,
                                        1.0, None, None) == -1
    assert "nsamples" in _lib.last_error(lib)
    assert lib.mgb_dft_contract_noalloc(None, 3, 4, 1, None, 4, 0, 1, 0.1, 0, 1.0, None, None) == -1
    assert "ld" in _lib.last_error(lib)
    assert lib.mgb_dft_contract_noalloc(None, 4, 4, 1, None, 4, 0, 1, 0.1, 0, 1.0, None, None) == -1
    assert "null" in _lib.last_error(lib)
    assert lib.mgb_dft_contract_status(None, 0, None) == -1


def _function_body(text: str, name: str) -> str:
    start = text.index(f"int {name}(")
    depth, i = 0, text.index("{", start)
    for j in range(i, len(text)):
        depth += {"{": 1, "}": -1}.get(text[j], 0)
        if depth == 0:
            return text[start:j + 1]
    raise AssertionError(f"no body for {name}")


def test_noalloc_path_names_no_allocating_call():
    """The entry point and the helpers it calls name no allocating CUDA routine."""
    text = SOURCE.read_text()
    body = "".join(_function_body(text, name) for name in
                   ("mgb_dft_contract_noalloc", "static_words", "check_contract", "contract_with_table",
                    "mgb_dft_contract_status"))
    assert not re.search(r"cuda(Malloc|Free|HostAlloc|MallocAsync|MallocManaged|MallocHost)\w*", body)
    assert "g_dft_table" in body and "cudaGetSymbolAddress" in body


@pytest.mark.gpu
def test_noalloc_equals_the_scratch_entry_point_twice_in_a_row(gpu):
    import torch

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _lib.check(lib, lib.mgb_dft_contract_status(status.data_ptr(), 1, stream))
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
        outputs = [acc0.clone(), acc0.clone()]
        # one call first (its device's table address is looked up), then two more with
        # the caching allocator's counters unchanged across them (the garbage collector
        # held off, so no tensor of an earlier test is freed in between)
        warm = acc0.clone()
        _lib.check(lib, lib.mgb_dft_contract_noalloc(samples.data_ptr(), *args, warm.data_ptr(), stream))
        torch.cuda.synchronize()
        pointers = [out.data_ptr() for out in outputs]
        gc.collect()
        gc.disable()
        try:
            allocated, reserved = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
            for ptr in pointers:
                _lib.check(lib, lib.mgb_dft_contract_noalloc(samples.data_ptr(), *args, ptr, stream))
            torch.cuda.synchronize()
            after = (torch.cuda.memory_allocated(), torch.cuda.memory_reserved())
        finally:
            gc.enable()
        assert after == (allocated, reserved)
        for out in outputs:
            assert torch.equal(out, expected), (nfreq, ncols, nsamples)
        assert not torch.equal(expected, acc0)
    _lib.check(lib, lib.mgb_dft_contract_status(status.data_ptr(), 0, stream))
    torch.cuda.synchronize()
    assert int(status.item()) == 0, "a contraction reported a tensor-core wait that ran out"
