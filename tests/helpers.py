"""Shared helpers of the test suite."""
from __future__ import annotations

from functools import lru_cache
from pathlib import Path

import numpy as np

from rayfactorcl_gb300.scene import Scene, read_scene

GOLDEN = Path(__file__).resolve().parent / "golden"
SCENES = GOLDEN / "scenes"
SAMPLE_NAMES = ["input-C109", "input-C122", "input-C14-BV", "input-C14", "input-C47", "input-C52-BV",
                "input-C52", "input-C77", "input-W100", "input-furnace", "input-uni"]
GEN_NAMES = ["gen_enclosure3", "gen_mixed64", "gen_furnace", "gen_precision_stress", "gen_sweep0",
             "gen_sweep1", "gen_sweep2"]


@lru_cache(maxsize=None)
def golden_scene(name: str) -> Scene:
    """Tables written by the reference's own Scene loader."""
    return Scene.from_bytes((SCENES / f"{name}.bin").read_bytes())


@lru_cache(maxsize=None)
def gen_scene(name: str) -> Scene:
    """Our loader on a committed generated scene XML."""
    return read_scene(SCENES / f"{name}.xml")


def binom_sigma(F: np.ndarray, n) -> np.ndarray:
    n = np.maximum(np.asarray(n, np.float64), 1.0)
    return np.sqrt(np.clip(F * (1 - F), 1e-300, None) / n)
