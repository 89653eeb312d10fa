"""Shared test set-up: markers, paths, scene helpers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "test-_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"
for p in (str(PKG), str(Path(__file__).resolve().parent)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product's kernels")


def scene_arrays_from_ctx(ctx):
    import oracle_bind as ob

    s = ctx.get_scene()
    return ob.SceneArrays(s["geom_modes"], s["geom_offsets"], s["geom"], s["field_modes"], s["field_offsets"],
                          s["field"], s["corners"])


@pytest.fixture(scope="session")
def oracle():
    import oracle_bind as ob

    ob.build_oracle()
    return ob


def classify(gpu_hits, ref_hits):
    """Per-ray agreement of two hit arrays: ids (kind, elem, face) and t."""
    g_face = gpu_hits["face"].astype(np.int32)
    same = (gpu_hits["kind"] == ref_hits["kind"]) & (gpu_hits["elem"] == ref_hits["elem"]) & (
        g_face == ref_hits["face"])
    return same
