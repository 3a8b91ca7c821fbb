"""The parity cases at the benchmark configurations' own sizes, shared by
tests/golden/gen_configs.py (the reference's digests) and the tests.

Each render case names a scene, its parameters, a seed and a window of the
film; the window's pixels are keyed as in the full render, so a window of a
large film gives exactly the full render's samples there.
"""
from __future__ import annotations

import hashlib

import numpy as np

from ajisai_render_gb300 import scenes as S


def digest(*arrays) -> str:
    """sha256 over the raw bytes of the arrays, in order."""
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def f32_bits(a) -> list:
    """float32 values as their 32-bit patterns (exact in JSON)."""
    return [int(x) for x in np.asarray(a, np.float32).view(np.uint32)]


def from_f32_bits(bits) -> np.ndarray:
    return np.asarray(bits, np.uint32).view(np.float32)


def case_scene(name, digests=None):
    """(flat scene, case) of a render case; with the digest record, the
    camera record is the reference's own."""
    case = RENDER_CASES[name]
    flat = S.flatten(case["scene"]())
    if digests is not None:
        flat.camera = from_f32_bits(digests[name]["camera_f32_bits"])
    return flat, case


def _c3(seed_index):
    """Job `seed_index` of the batched workload's 48-job list (seed 1)."""
    j = S.batch_workload(48, seed=1)[seed_index]
    return j, S.mixed_scene(j["scene_seed"], j["tris"], j["res"], j["res"])


def c3_smallest_clutter():
    """The batched list's smallest clutter scene: job 34, 1,611 target
    triangles (134 boxes), 1024x1024, 25 spp."""
    return _c3(34)


def c3_largest_icosphere():
    """The batched list's largest icosphere: job 43, 1,942,191 target
    triangles (the generator's subdivision-8 cap: 1,310,720), 512x512,
    31 spp."""
    return _c3(43)


RENDER_CASES = {
    # the Cornell-style box at its full size: 256x256, 64 spp, depth 8,
    # Russian roulette after bounce 3
    "c1_cornell_full": dict(
        scene=lambda: S.cornell_box(256, 256), radius=14, seed=1,
        params=dict(spp=64, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=1),
        window=(0, 0, 256, 256)),
    # a 64x64 crop of the single-job workload (1,310,722 triangles, 1024x1024,
    # depth 16) at 16 spp, over the full-size tree
    "c2_icosphere_crop": dict(
        scene=lambda: S.icosphere_scene(subdiv=8, seed=0, width=1024, height=1024),
        radius=16, seed=1,
        params=dict(spp=16, min_bounces=5, max_bounces=16, cont_prob=0.9, use_mis=1),
        window=(480, 480, 64, 64)),
    # two jobs of the batched workload (depth 12) at their own spp
    "c3_clutter_crop": dict(
        scene=lambda: c3_smallest_clutter()[1], radius=16, seed=7,
        params=dict(spp=25, min_bounces=5, max_bounces=12, cont_prob=0.9, use_mis=1),
        window=(448, 448, 128, 128)),
    "c3_icosphere_crop": dict(
        scene=lambda: c3_largest_icosphere()[1], radius=16, seed=7,
        params=dict(spp=31, min_bounces=5, max_bounces=12, cont_prob=0.9, use_mis=1),
        window=(224, 224, 64, 64)),
}


def full_size_geometry():
    """The single-job workload's geometry (1,310,722 triangles)."""
    return S.flatten(S.icosphere_scene(subdiv=8, seed=0, width=8, height=8))


def full_size_rays(n=200_000, seed=5):
    """Seeded rays around the single-job workload's sphere: origins in
    [-2, 2]^3 aimed at [-1, 1]^3, 30% with a finite t_max."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-2, 2, (n, 3))
    d = rng.uniform(-1, 1, (n, 3)) - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = np.where(rng.uniform(size=n) < 0.3, rng.uniform(0.2, 3, n), np.inf)
    return np.concatenate([o, d, np.full((n, 1), 1e-4), tmax[:, None]],
                          1).astype(np.float32)
