"""Digests of what the reference computes at the benchmark configurations'
own sizes, for pinning the oracle there.

Run in the development container, where the reference is present:

    python tests/golden/gen_configs.py

The cases are too large to commit as arrays (the Cornell box at full size
is 4.2 M samples), so configs.json keeps sha256 digests of the reference's
outputs: the per-sample radiance of each render case's window
(tests/config_cases.py), the reference's own PLOC tree over the single-job
workload's 1,310,722 triangles (its Morton sort, ploc_aggregate.cpp:97-130,
as built), and the closest and any hits of 200,000 seeded rays against that
tree.  tests/test_oracle_configs.py recomputes each with the oracle and
compares the digests.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import config_cases as CC  # noqa: E402
from ajisai_render_gb300 import scenes as S  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "configs.json"


def main():
    if O.ref() is None:
        sys.exit("the reference sources are not available here")
    out = {}
    for name, case in CC.RENDER_CASES.items():
        t = time.time()
        rs = O.RefScene(case["scene"](), search_radius=case["radius"])
        x0, y0, w, h = case["window"]
        li = rs.render_window(case["params"], case["seed"], x0, y0, w, h)
        out[name] = {"li_sha256": CC.digest(li), "shape": list(li.shape),
                     "camera_f32_bits": CC.f32_bits(rs.dump().camera)}
        rs.close()
        print(name, li.shape, "%.1f s" % (time.time() - t))
    t = time.time()
    # the workload's triangles as one harness mesh, so that every hit (the
    # ground's too) names its triangle
    P = CC.full_size_geometry().tris.reshape(-1, 3)
    I = np.arange(P.shape[0], dtype=np.int32).reshape(-1, 3)
    spec = S.Scene([S.Mesh(P, I, None, 0)], [S.Diffuse((0.5, 0.5, 0.5))], [], None)
    rs = O.RefScene(spec, search_radius=16)
    nb, ncf, perm = rs.ploc()
    rays = CC.full_size_rays()
    tt, p, u, v = rs.trace(rays)
    _, occ, _, _ = rs.trace(rays, any_hit=True)
    out["c2_reference_tree"] = {"perm_sha256": CC.digest(perm),
                                "node_count_first_sha256": CC.digest(ncf),
                                "node_bounds_sha256": CC.digest(nb),
                                "triangles": int(rs.n),
                                "distinct_leaves": int(len(set(perm.tolist())))}
    out["c2_reference_rays"] = {"closest_sha256": CC.digest(tt, p, u, v),
                                "any_sha256": CC.digest(occ), "rays": int(len(rays)),
                                "hits": int((p >= 0).sum()), "occluded": int((occ == 1).sum())}
    print("tree + rays %.1f s" % (time.time() - t))
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
