"""Helpers to read the committed golden fixtures."""

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def fields(case: str):
    return np.load(GOLDEN / f"fields_{case}.npz")


def digest():
    return json.loads((GOLDEN / "digest_sphere80.json").read_text())


def tables():
    return np.load(GOLDEN / "tables.npz"), json.loads((GOLDEN / "tables.json").read_text())


def meep_identity():
    """MEEP's stored digests of the 2-D identity cases and how to build each run
    (``tests/golden/make_meep_identity.py``)."""
    return json.loads((GOLDEN / "meep_identity.json").read_text()), np.load(GOLDEN / "meep_identity.npz")


def _identity_value(node, arrays):
    if isinstance(node, dict):
        if set(node) == {"uniform"}:
            return float(node["uniform"])
        if set(node) == {"array"}:
            return arrays[node["array"]]
        if set(node) == {"complex"}:
            return complex(*node["complex"])
        if set(node) == {"mirror"}:
            from meep_gpu_gb300 import Mirror
            return Mirror(node["mirror"][0], node["mirror"][1])
        if set(node) == {"absorber"}:
            from meep_gpu_gb300.conductivity import AbsorberLayer
            return AbsorberLayer(**node["absorber"])
        return {k: _identity_value(v, arrays) for k, v in node.items()}
    if isinstance(node, list):
        return [_identity_value(v, arrays) for v in node]
    return node


def identity_masks(case: str):
    """Per component the stored cells an identity case compares (None: every cell)."""
    record, arrays = meep_identity()
    masks = record["cases"][case].get("masks", {})
    return {c: (arrays[masks[c]] if c in masks else None) for c in record["components"]}


def build_identity(case: str, driver_cls, susceptibility_cls, **driver_kwargs):
    """One identity case built on ``driver_cls`` by its recorded construction calls."""
    record, arrays = meep_identity()
    entry = record["cases"][case]
    constructor = {k: _identity_value(v, arrays) for k, v in entry["constructor"].items()}
    constructor["boundaries"] = constructor["boundaries"] or None
    constructor.update(driver_kwargs)
    driver = driver_cls(**constructor)
    for name, kwargs in entry["calls"]:
        kwargs = _identity_value(kwargs, arrays)
        if name == "add_susceptibility":
            kwargs["susceptibility"] = susceptibility_cls(**kwargs["susceptibility"]["susceptibility"])
        getattr(driver, name)(**kwargs)
    return driver, entry


def word_digest(array) -> str:
    """SHA-256 of an array's float32 words in C order, little-endian (how the identity
    records digest MEEP's stored words)."""
    import hashlib
    words = np.ascontiguousarray(array, dtype=np.float32).view("<u4")
    return hashlib.sha256(np.ascontiguousarray(words).tobytes()).hexdigest()


def compared_digest(array, mask) -> str:
    """``word_digest`` of the cells ``mask`` selects (all of them when None), C order."""
    values = np.ascontiguousarray(array, dtype=np.float32)
    return word_digest(values if mask is None else values[mask])
