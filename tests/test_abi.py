"""The C ABI: libmeepgb.so builds, loads, exports every declared symbol, and the
ctypes mirror of ``include/meepgb.h`` has the header's layout (no GPU needed)."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from meep_gpu_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "meepgb.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|size_t|int64_t|int32_t)\s+(mgb_\w+)\s*\(", text, re.M)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load()
    symbols = declared_symbols()
    assert symbols, "no entry points found in the header"
    for name in symbols:
        assert hasattr(lib, name), f"libmeepgb.so does not export {name}"
    assert set(symbols) == set(_lib.SIGNATURES), "binding and header disagree on the entry points"
    assert lib.mgb_abi_version() == _lib.MGB_ABI_VERSION


def test_build_compiles_every_translation_unit():
    """The GPU machine has only what build() compiles: every CUDA source and header of the
    package is in the recipe (a unit left out would leave its kernels unresolved there)."""
    from meep_gpu_gb300 import build

    csrc = ROOT / "meep_gpu_gb300" / "csrc"
    assert {p.name for p in csrc.glob("*.cu")} == {p.name for p in build.SOURCES}
    assert {p.name for p in csrc.glob("*.cuh")} == {p.name for p in build.HEADERS}


def test_create_refuses_bad_descriptors_without_a_gpu():
    lib = _lib.load()
    desc = _lib.MgbSimDesc()
    desc.abi_version = _lib.MGB_ABI_VERSION + 7
    handle = ctypes.c_void_p()
    code = lib.mgb_create(ctypes.byref(desc), ctypes.byref(handle))
    assert code == -1 and "ABI version" in _lib.last_error(lib)
    desc.abi_version = _lib.MGB_ABI_VERSION
    desc.nx, desc.ny, desc.nz = 0, 8, 8
    assert lib.mgb_create(ctypes.byref(desc), ctypes.byref(handle)) == -1
    assert "at least one cell" in _lib.last_error(lib)
    desc.nx = 1  # a one-cell axis must be periodic
    desc.metallic[0] = 1
    assert lib.mgb_create(ctypes.byref(desc), ctypes.byref(handle)) == -3
    assert "one cell must be periodic" in _lib.last_error(lib)
    desc.metallic[0] = 0
    desc.nx, desc.ny, desc.nz = 1300, 1300, 1300  # 2.2e9 cells: past 32-bit offsets
    assert lib.mgb_create(ctypes.byref(desc), ctypes.byref(handle)) == -3
    assert "2^31" in _lib.last_error(lib)


def test_batch_entry_points_refuse_bad_arguments_without_a_gpu():
    lib = _lib.load()
    small = lib.mgb_batch_bytes(1, 1, 1)
    big = lib.mgb_batch_bytes(64, 100000, 20000)
    assert small % 256 == 0 and big > small
    handle = ctypes.c_void_p()
    assert lib.mgb_batch_create(4, 16, 16, None, big, ctypes.byref(handle)) == -1
    assert "device buffer" in _lib.last_error(lib)
    # size and alignment are checked before any device call
    assert lib.mgb_batch_create(4, 16, 16, 256, 8, ctypes.byref(handle)) == -1
    assert "smaller than" in _lib.last_error(lib)
    assert lib.mgb_batch_create(4, 16, 16, 257, big, ctypes.byref(handle)) == -1
    assert "aligned" in _lib.last_error(lib)
    assert lib.mgb_batch_set_slot(None, 0, None, 10, None) == -1
    assert lib.mgb_batch_set_shape(None, 32, 4, 4) == -1
    assert lib.mgb_batch_set_family(None, 2) == -1
    assert lib.mgb_batch_items(None, 0) == -1
    lib.mgb_batch_destroy(None)


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "meepgb.h"
#define F(T, m) printf(#T "." #m " %zu\n", offsetof(T, m));
int main(void) {
  printf("sizeof.mgb_sim_desc %zu\n", sizeof(mgb_sim_desc));
  printf("sizeof.mgb_monitor %zu\n", sizeof(mgb_monitor));
  printf("sizeof.mgb_pole %zu\n", sizeof(mgb_pole));
  printf("sizeof.mgb_aux %zu\n", sizeof(mgb_aux));
  printf("sizeof.mgb_conductivity %zu\n", sizeof(mgb_conductivity));
  F(mgb_sim_desc, dtdx) F(mgb_sim_desc, kms) F(mgb_sim_desc, E) F(mgb_sim_desc, H) F(mgb_sim_desc, B)
  F(mgb_sim_desc, fuD) F(mgb_sim_desc, npoles) F(mgb_sim_desc, poles) F(mgb_sim_desc, nsrc)
  F(mgb_sim_desc, src_box) F(mgb_sim_desc, nmonitors) F(mgb_sim_desc, monitors)
  F(mgb_sim_desc, status) F(mgb_monitor, scale) F(mgb_monitor, omega) F(mgb_monitor, acc)
  F(mgb_pole, sigma) F(mgb_pole, p) F(mgb_sim_desc, conductivity)
  F(mgb_conductivity, condinv) F(mgb_conductivity, fcond) F(mgb_conductivity, chunk_of)
  F(mgb_conductivity, keeps) F(mgb_sim_desc, nsrc_magnetic) F(mgb_sim_desc, src_box_magnetic)
  F(mgb_sim_desc, bloch_axes) F(mgb_sim_desc, bloch_phase) F(mgb_sim_desc, partner_E)
  F(mgb_sim_desc, partner_H) F(mgb_sim_desc, mirror) F(mgb_sim_desc, full) F(mgb_sim_desc, fold)
  F(mgb_fold, ghost) F(mgb_fold, image) F(mgb_fold, code) F(mgb_fold, saved)
  printf("sizeof.mgb_fold %zu\n", sizeof(mgb_fold));
  return 0;
}
"""


def test_ctypes_layout_matches_the_header(tmp_path):
    source = tmp_path / "probe.c"
    source.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), "-o", str(exe), str(source)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = dict(line.split() for line in out.strip().splitlines())
    types = {"mgb_sim_desc": _lib.MgbSimDesc, "mgb_monitor": _lib.MgbMonitor,
             "mgb_pole": _lib.MgbPole, "mgb_aux": _lib.MgbAux,
             "mgb_conductivity": _lib.MgbConductivity, "mgb_fold": _lib.MgbFold}
    for key, value in layout.items():
        kind, member = key.split(".")
        if kind == "sizeof":
            assert ctypes.sizeof(types[member]) == int(value), key
        else:
            assert getattr(types[kind], member).offset == int(value), key
