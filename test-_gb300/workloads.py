"""Named synthetic workloads (pure Python: no library is loaded).

A workload is a seeded scene (ho_generate_synthetic's parameters), a pinhole
camera, an image size and isovalues. The benchmark's CPU arm builds the same
scene with the oracle's generator, so it reads these definitions without
loading libhorender.so; horender.py re-exports them.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Camera:
    """Pinhole camera (FEM-AABB/raytracer.h:31-48 with aperture 0)."""
    lookfrom: tuple
    lookat: tuple
    vup: tuple = (0.0, 1.0, 0.0)
    vfov_deg: float = 60.0
    focus_dist: float = 0.0


@dataclass
class Workload:
    """A named synthetic workload: scene + view + isovalues."""
    name: str
    nx: int
    order_min: int
    order_max: int
    curve_amp: float
    n_gauss: int
    seed: int
    width: int
    height: int
    isovalues: list = field(default_factory=list)
    camera: Camera = field(default_factory=lambda: Camera((2.5, 2.0, 1.8), (0.5, 0.5, 0.5), (0, 1, 0), 60.0))

    def synth(self) -> dict:
        return dict(nx=self.nx, ny=self.nx, nz=self.nx, order_min=self.order_min, order_max=self.order_max,
                    curve_amp=self.curve_amp, n_gauss=self.n_gauss, seed=self.seed)


# Benchmark workloads (seeded synthetic stand-ins for the reference's meshes).
WORKLOADS = {
    "hex4_p4": Workload("hex4_p4", 4, 4, 4, 0.05, 8, 1, 256, 256, [0.2]),
    "hex32_p6": Workload("hex32_p6", 32, 6, 6, 0.08, 64, 2, 1920, 1080, [-0.3, 0.0, 0.3]),
    "hex48_mixed": Workload("hex48_mixed", 48, 2, 8, 0.1, 64, 3, 1024, 1024, [-0.2, 0.1, 0.3]),
    "hex64_p5": Workload("hex64_p5", 64, 5, 5, 0.12, 64, 4, 3840, 2160, [0.1]),
    "hex96_mixed": Workload("hex96_mixed", 96, 3, 8, 0.1, 256, 5, 2048, 2048, [-0.4, 0.1, 0.6]),
}


RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
ISO_POOL = [-0.3, -0.2, -0.1, 0.0, 0.1, 0.2, 0.3]


def sphere_views(n_views: int = 64, radius: float = 2.5, centre=(0.5, 0.5, 0.5), seed: int = 7,
                 shrink: int = 1) -> tuple[list, list, list, list]:
    """n seeded camera views on a Fibonacci sphere around the cube centre, each
    with a resolution drawn from RESOLUTIONS (divided by `shrink`) and 1-4
    distinct isovalues drawn from ISO_POOL. Returns cameras, widths, heights,
    isovalue lists (the uneven multi-view workload)."""
    rng = np.random.default_rng(seed)
    golden = np.pi * (3.0 - np.sqrt(5.0))
    cams, ws, hs, isos = [], [], [], []
    for i in range(n_views):
        y = 1.0 - 2.0 * (i + 0.5) / n_views
        r = np.sqrt(max(0.0, 1.0 - y * y))
        phi = golden * i
        pos = tuple(float(c + radius * v) for c, v in zip(centre, (r * np.cos(phi), y, r * np.sin(phi))))
        vup = (0.0, 0.0, 1.0) if abs(y) > 0.99 else (0.0, 1.0, 0.0)
        cams.append(Camera(pos, tuple(centre), vup, 60.0))
        wdt, hgt = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
        ws.append(max(1, wdt // shrink))
        hs.append(max(1, hgt // shrink))
        k = int(rng.integers(1, 5))
        isos.append(sorted(float(v) for v in rng.choice(ISO_POOL, size=k, replace=False)))
    return cams, ws, hs, isos


# multi-view workloads: scene workload + views
MULTIVIEW = {"views64": ("hex48_mixed", dict(n_views=64, seed=7))}
# Path-tracing workloads: scene, and the per-step sample pass (ho_path_trace).
PATHS = {"path96": ("hex96_mixed", dict(spp=1, max_depth=4, seed=1))}
