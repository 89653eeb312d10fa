"""The command-line renderer on the GPU: its image equals the library's own
path trace of the same scene, camera, samples, depth and seed, byte for
byte; the second view and the PNG copies are written too."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

import horender as hr
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "test-_gb300" / "horender_cli"
SCENE = GOLDEN / "nektar" / "nek_faces.xml"


def read_ppm(path: Path, w: int, h: int) -> np.ndarray:
    data = path.read_bytes()
    head = f"P6\n{w} {h}\n255\n".encode()
    assert data.startswith(head)
    return np.frombuffer(data[len(head):], np.uint8).reshape(h, w, 3)


def test_cli_image_equals_library_path_trace(tmp_path):
    if not CLI.exists():
        pytest.fail("horender_cli not built")
    W, H, spp, depth, seed = 48, 32, 2, 3, 5
    out = tmp_path / "o"
    r = subprocess.run([str(CLI), str(SCENE), "--width", str(W), "--height", str(H), "--spp", str(spp), "--depth",
                        str(depth), "--seed", str(seed), "--out", str(out), "--png"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    cam_line = [l for l in r.stdout.splitlines() if l.startswith("Camera:")][0].split()
    lookfrom = tuple(float(x) for x in cam_line[2:5])
    lookat = tuple(float(x) for x in cam_line[6:9])
    img = read_ppm(Path(f"{out}.ppm"), W, H)
    back = read_ppm(Path(f"{out}_back.ppm"), W, H)
    assert Path(f"{out}.png").exists() and Path(f"{out}_back.png").exists()

    ctx = hr.Context(0)
    ctx.load_xml_fld(str(SCENE), str(SCENE.with_suffix(".fld")))
    ctx.build_bvh()
    cam = hr.Camera(lookfrom, lookat, vfov_deg=20.0)
    want, _ = ctx.path_trace(cam, [0.0], W, H, spp=spp, max_depth=depth, seed=seed, iso_zero_disables=True)
    assert np.array_equal(img, want[0])
    # the scene is in view, and the view from the other side is another image
    assert (img != img[0, 0]).any()
    assert not np.array_equal(img, back)
