"""ctypes binding of ``libmeepgb.so`` (the C ABI declared in ``include/meepgb.h``).

The structures below mirror the header field for field. Loading fails loudly: there
is no CPU stepping path behind this package, so a missing or stale library is an
error, never a fallback.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Optional

PACKAGE = Path(__file__).resolve().parent

MGB_ABI_VERSION = 4
MGB_MAX_POLES = 8
MGB_MAX_MONITORS = 16
MGB_MAX_MONITOR_COMPONENTS = 6
MGB_DFT_DEPTH = 32
MGB_DFT_MAX_FREQ = 512

MGB_OK = 0
ERROR_NAMES = {-1: "MGB_ERR_ARGUMENT", -2: "MGB_ERR_CUDA", -3: "MGB_ERR_UNSUPPORTED",
               -4: "MGB_ERR_RANGE"}

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class MgbAux(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("axis", ctypes.c_int32),
                ("a0", ctypes.c_int32), ("a1", ctypes.c_int32),
                ("b0", ctypes.c_int32), ("b1", ctypes.c_int32)]


class MgbPole(ctypes.Structure):
    _fields_ = [("two_minus_od", ctypes.c_float), ("gamma1", ctypes.c_float),
                ("omega0dtsqr", ctypes.c_float), ("gamma1inv", ctypes.c_float),
                ("sigma", ctypes.c_void_p * 3),
                ("p", (ctypes.c_void_p * 2) * 3)]


class MgbMonitor(ctypes.Structure):
    _fields_ = [("region", ctypes.c_int32 * 6), ("ncomp", ctypes.c_int32),
                ("comp", ctypes.c_int32 * MGB_MAX_MONITOR_COMPONENTS),
                ("nfreq", ctypes.c_int32), ("decimation", ctypes.c_int32),
                ("scale", ctypes.c_double), ("dt", ctypes.c_double),
                ("omega", ctypes.c_void_p), ("acc", ctypes.c_void_p)]


class MgbConductivity(ctypes.Structure):
    _fields_ = [
        ("condfac", (ctypes.c_void_p * 3) * 2),
        ("condinv", (ctypes.c_void_p * 3) * 2),
        ("fcond", (ctypes.c_void_p * 3) * 2),
        ("chunk_of", (ctypes.c_void_p * 3) * 2),
        ("keeps", (ctypes.c_uint32 * 3) * 2),
    ]


MGB_FOLD_WORDS = 2 + MGB_MAX_POLES


class MgbFold(ctypes.Structure):
    """``mgb_fold``: the B (0) and D (1) ghost lists of mirror-folded axes."""
    _fields_ = [
        ("count", ctypes.c_int32 * 2),
        ("ghost", ctypes.c_void_p * 2),
        ("image", ctypes.c_void_p * 2),
        ("code", ctypes.c_void_p * 2),
        ("saved", ctypes.c_void_p * 2),
    ]


class MgbSimDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("metallic", ctypes.c_int32 * 3),
        ("dtdx", ctypes.c_float),
        ("pml_active", ctypes.c_int32),
        ("kms", (ctypes.c_void_p * 3) * 2),
        ("sinv", (ctypes.c_void_p * 3) * 2),
        ("kps", (ctypes.c_void_p * 3) * 2),
        ("E", ctypes.c_void_p * 3),
        ("D", ctypes.c_void_p * 3),
        ("H", ctypes.c_void_p * 3),
        ("inv_eps", ctypes.c_void_p * 3),
        ("B", MgbAux * 3),
        ("fwH", MgbAux * 3),
        ("fwE", MgbAux * 3),
        ("fuB", MgbAux * 3),
        ("fuD", MgbAux * 3),
        ("npoles", ctypes.c_int32),
        ("pbox", ctypes.c_int32 * 6),
        ("poles", MgbPole * MGB_MAX_POLES),
        ("nsrc", ctypes.c_int32),
        ("src_cell", ctypes.c_void_p),
        ("src_comp", ctypes.c_void_p),
        ("src_box", ctypes.c_int32 * 6),
        ("nmonitors", ctypes.c_int32),
        ("monitors", MgbMonitor * MGB_MAX_MONITORS),
        ("status", ctypes.c_void_p),
        ("conductivity", ctypes.POINTER(MgbConductivity)),
        ("nsrc_magnetic", ctypes.c_int32),
        ("src_box_magnetic", ctypes.c_int32 * 6),
        ("bloch_axes", ctypes.c_int32),
        ("part", ctypes.c_int32),
        ("bloch_phase", (ctypes.c_double * 2) * 3),
        ("partner_E", ctypes.c_void_p * 3),
        ("partner_H", ctypes.c_void_p * 3),
        ("mirror", ctypes.c_int32 * 3),
        ("full", ctypes.c_int32 * 3),
        ("fold", MgbFold),
        ("invariant", ctypes.c_int32),
    ]


class MgbAdjoint(ctypes.Structure):
    _fields_ = [("mu_b", ctypes.c_void_p * 3), ("mu_d", ctypes.c_void_p * 3),
                ("box", ctypes.c_int32 * 6), ("d_after", ctypes.c_void_p),
                ("grad_inv", ctypes.c_void_p)]


# Every symbol include/meepgb.h declares, with its ctypes signature.
SIGNATURES = {
    "mgb_abi_version": (ctypes.c_int, []),
    "mgb_create": (ctypes.c_int, [ctypes.POINTER(MgbSimDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "mgb_set_launch_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "mgb_set_source_words": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_int64]),
    "mgb_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "mgb_step_pair": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                     ctypes.c_void_p]),
    "mgb_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "mgb_flux_spectrum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "mgb_field_energy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mgb_uses_tiles": (ctypes.c_int, [ctypes.c_void_p]),
    "mgb_select_kernels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_select_half": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_int32]),
    "mgb_set_split": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_wave_bytes": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "mgb_set_wave": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_size_t, ctypes.c_void_p]),
    "mgb_destroy": (None, [ctypes.c_void_p]),
    "mgb_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "mgb_dft_scratch_bytes": (ctypes.c_size_t, [ctypes.c_int32]),
    "mgb_set_dft_buffer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_size_t]),
    "mgb_dft_flush": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mgb_read_accumulator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_void_p, ctypes.c_void_p]),
    "mgb_dft_pending": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_dft_contract": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_double, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "mgb_dft_contract_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                                ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                                ctypes.c_int32, ctypes.c_double, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "mgb_dft_contract_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "mgb_set_test_wait_limit": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64]),
    "mgb_adjoint_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(MgbAdjoint), ctypes.c_int64,
                                        ctypes.c_void_p]),
    "mgb_adjoint_inject": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p]),
    "mgb_adjoint_segment": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(MgbAdjoint),
                                           ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "mgb_copy_box": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    "mgb_batch_bytes": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "mgb_batch_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "mgb_batch_set_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32]),
    "mgb_batch_set_family": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_batch_set_slot": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_int64, ctypes.c_void_p]),
    "mgb_batch_clear_slot": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_batch_commit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mgb_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_void_p]),
    "mgb_batch_steps": (ctypes.c_int, [ctypes.c_void_p, c_int64_p]),
    "mgb_batch_items": (ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int32]),
    "mgb_batch_destroy": (None, [ctypes.c_void_p]),
}

_LIB: Optional[ctypes.CDLL] = None


class MeepGBError(RuntimeError):
    """A failure reported by libmeepgb (negative return code) with its message."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


def library_path() -> Path:
    override = os.environ.get("MEEPGB_LIBRARY")
    return Path(override) if override else PACKAGE / "libmeepgb.so"


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library; raise if it cannot be had."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build_if_missing and "MEEPGB_LIBRARY" not in os.environ:
        from . import build as _build
        try:
            _build.build()
        except Exception as exc:  # noqa: BLE001 - re-raised with the reason
            if not path.exists():
                raise RuntimeError(f"libmeepgb.so is not built and building it failed: {exc}") from exc
    if not path.exists():
        raise RuntimeError(f"libmeepgb.so not found at {path}; run meep_gpu_gb300.build.build()")
    lib = ctypes.CDLL(str(path))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    version = lib.mgb_abi_version()
    if version != MGB_ABI_VERSION:
        raise RuntimeError(f"libmeepgb.so ABI {version} does not match the binding's {MGB_ABI_VERSION}")
    _LIB = lib
    return lib


def last_error(lib: ctypes.CDLL) -> str:
    buf = ctypes.create_string_buffer(1024)
    lib.mgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(lib: ctypes.CDLL, code: int) -> None:
    if code != MGB_OK:
        raise MeepGBError(code, last_error(lib))
