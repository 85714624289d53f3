"""Seeded synthetic workloads for the batching and serving configurations.

* batch_jobs: many independent optimisation jobs of uneven size -- displaced
  spheres with a log-uniform triangle count, resolution, sample count and
  number of views drawn per job, point-light Lambert shading with vertex
  albedo.
* serving_trace: a Poisson arrival process of such jobs, each with its own
  step count, shading model and resolution.

The triangle counts are met with a closed UV sphere of 2*lon*(lat-1)
triangles (lon = 2*lat), the nearest such count to the draw; icosphere
subdivision only offers 20*4^s triangles.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

from .scene import CamInfo, displace_radially, make_uv_sphere, perturb_vertices, ring_cameras


@dataclass
class JobSpec:
    true_mesh: object
    init_mesh: object
    cams: List[CamInfo]
    mode: int
    spp: int
    steps: int = 1
    arrival: float = 0.0
    triangles: int = 0


def sphere_with_triangles(n_tris: int, seed: int):
    """Displaced UV sphere whose triangle count is close to n_tris."""
    lat = max(3, int(round(math.sqrt(n_tris / 4.0))))
    m = make_uv_sphere(lat, 2 * lat, seed=seed)
    return displace_radially(m, seed=seed + 1000, n_waves=8, amplitude=0.05)


def batch_jobs(n: int = 64, seed: int = 0, tri_range=(500, 50_000), resolutions=(128, 256, 512),
               spps=(4, 8, 16, 32), views=(1, 4), mode: int = 16) -> List[JobSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n):
        t = int(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1]))))
        res = int(rng.choice(resolutions))
        spp = int(rng.choice(spps))
        nv = int(rng.integers(views[0], views[1] + 1))
        true = sphere_with_triangles(t, seed=seed * 1000 + j)
        init = perturb_vertices(true, 0.02, seed=seed * 1000 + j + 500, radial=True)
        cams = ring_cameras(nv, 3.0, res, res)
        out.append(JobSpec(true, init, cams, mode, spp, triangles=true.face_count))
    return out


def serving_trace(n_jobs: int, seed: int = 0, rate: float = 20.0, tri_range=(1_000, 100_000),
                  res_range=(256, 1024), views=(1, 8), steps=(50, 500), modes=(16, 2), spp: int = 4) -> List[JobSpec]:
    """Poisson arrivals (rate jobs/s); resolution drawn from multiples of 64
    in res_range; model drawn from `modes` (point-light Lambert or vertex
    colour)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for j in range(n_jobs):
        t += float(rng.exponential(1.0 / rate))
        tri = int(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1]))))
        res = int(rng.integers(res_range[0] // 64, res_range[1] // 64 + 1)) * 64
        nv = int(rng.integers(views[0], views[1] + 1))
        st = int(rng.integers(steps[0], steps[1] + 1))
        mode = int(rng.choice(modes))
        true = sphere_with_triangles(tri, seed=seed * 100000 + j)
        init = perturb_vertices(true, 0.02, seed=seed * 100000 + j + 50000, radial=True)
        if mode == 2:
            init.colors = np.clip(true.colors + rng.normal(0, 0.1, true.colors.shape), 0, 1).astype(np.float32)
        out.append(JobSpec(true, init, ring_cameras(nv, 3.0, res, res), mode, spp, steps=st, arrival=t,
                           triangles=true.face_count))
    return out
