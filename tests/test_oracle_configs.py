"""The oracle against the reference at the benchmark configurations' own
sizes (CPU): the per-sample radiance of every render case's window, the
reference's own PLOC tree over the single-job workload's 1,310,722
triangles, and the hits of 200,000 rays against it, each equal bit for bit
to the digest of what the reference computed (tests/golden/configs.json,
written by tests/golden/gen_configs.py), with the camera record as the
reference computes it.  The reference renders over its own tree (its Morton
sort drops and repeats leaves) and traverses it depth first, a strictly
closer hit replacing the best, so the oracle runs here over the same tree
(radix_compat) in the same order (ORC_TEST_REF_ORDER): camera rays through a
shared edge hit two triangles at one t, and the reference keeps the first it
visits where the product's rule keeps the lower index.  How often that rule
changes a sample at these sizes is counted too."""
REF_ORDER = 2
import json

import numpy as np
import pytest

import config_cases as CC
from oracle import pyoracle as O


@pytest.fixture(scope="module")
def digests():
    from conftest import GOLDEN
    return json.loads((GOLDEN / "configs.json").read_text())


@pytest.mark.parametrize("name", list(CC.RENDER_CASES))
def test_oracle_window_matches_reference(digests, name):
    flat, case = CC.case_scene(name, digests)
    sc = O.OracleScene(flat, case["radius"], radix_compat=True, tri_test=REF_ORDER)
    x0, y0, w, h = case["window"]
    li = sc.render_window(flat.camera, case["params"], case["seed"], x0, y0, w, h)
    sc.close()
    assert list(li.shape) == digests[name]["shape"]
    assert CC.digest(li) == digests[name]["li_sha256"]
    # the lowest-index tie rule on the same tree: the same samples but for
    # the few whose path crosses a tie
    lo = O.OracleScene(flat, case["radius"], radix_compat=True)
    li_lo = lo.render_window(flat.camera, case["params"], case["seed"], x0, y0, w, h)
    lo.close()
    moved = (li.view(np.uint32) != li_lo.view(np.uint32)).any(-1).mean()
    assert moved < 1e-4, moved


def test_oracle_full_size_reference_tree_and_hits(digests):
    fl = CC.full_size_geometry()
    nb, ncf, perm = O.ploc_build(fl.tris, fl.world, 16, radix_compat=True)
    d = digests["c2_reference_tree"]
    assert fl.n_tris == d["triangles"] == 1310722
    assert len(np.unique(perm)) == d["distinct_leaves"] < fl.n_tris   # Q14
    assert CC.digest(perm) == d["perm_sha256"]
    assert CC.digest(ncf) == d["node_count_first_sha256"]
    assert CC.digest(nb) == d["node_bounds_sha256"]
    rays = CC.full_size_rays()
    t, p, u, v = O.trace(fl.tris, rays, bvh=(nb, ncf, perm), tri_test=REF_ORDER)
    _, occ, _, _ = O.trace(fl.tris, rays, any_hit=True, bvh=(nb, ncf, perm),
                           tri_test=REF_ORDER)
    r = digests["c2_reference_rays"]
    assert int((p >= 0).sum()) == r["hits"] and int((occ == 1).sum()) == r["occluded"]
    assert CC.digest(t, p, u, v) == r["closest_sha256"]
    assert CC.digest(occ) == r["any_sha256"]
