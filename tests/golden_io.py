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
