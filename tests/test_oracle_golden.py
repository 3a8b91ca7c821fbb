"""Pin the oracle against the golden vectors the reference's own sources
produced (tests/golden/gen_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import pyoracle as O

PLOC_CASES = ["ploc_cornell.npz", "ploc_ico4.npz", "ploc_soup.npz", "ploc_flat.npz"]


@pytest.mark.parametrize("case", PLOC_CASES)
def test_ploc_tree_matches_reference(golden, case):
    g = golden(case)
    nb, ncf, perm = O.ploc_build(g["tris"], g["world"], int(g["radius"]),
                                 radix_compat=True)
    assert np.array_equal(perm, g["perm"])
    assert np.array_equal(ncf, g["node_count_first"])
    assert np.array_equal(nb.view(np.uint32), g["node_bounds"].view(np.uint32))


@pytest.mark.parametrize("case", PLOC_CASES)
def test_ploc_correct_sort_is_a_permutation(golden, case):
    """With the stable sort the build covers every triangle once; the
    reference's sort drops and duplicates some on the larger inputs."""
    g = golden(case)
    n = g["tris"].shape[0]
    nb, ncf, perm = O.ploc_build(g["tris"], g["world"], int(g["radius"]))
    assert np.array_equal(np.sort(perm), np.arange(n))
    leaves = ncf[ncf[:, 0] == 1, 1]
    assert np.array_equal(np.sort(leaves), np.arange(n))
    # interior nodes have two children and bound them
    inner = np.where(ncf[:, 0] == 0)[0]
    assert inner.size == n - 1
    c0 = ncf[inner, 1]
    for c in (c0, c0 + 1):
        # a point box is absorbed by Join (math/bounds.h:108-113), so only
        # non-point children are guaranteed to lie inside their parent
        solid = ~np.all(nb[c, :3] == nb[c, 3:], axis=1)
        assert np.all(nb[inner[solid], :3] <= nb[c[solid], :3])
        assert np.all(nb[inner[solid], 3:] >= nb[c[solid], 3:])
    if case == "ploc_ico4.npz":
        assert len(np.unique(g["perm"])) < n  # the reference lost triangles


@pytest.mark.parametrize("case", ["trace_ico4.npz", "trace_soup.npz"])
def test_closest_hit_matches_reference(golden, case):
    g = golden(case)
    bvh = O.ploc_build(g["tris"], g["world"], int(g["radius"]), radix_compat=True)
    t, p, u, v = O.trace(g["tris"], g["rays"], bvh=bvh, tri_test=0)
    hit = g["prim"] >= 0
    assert np.array_equal(p, g["prim"])
    assert np.array_equal(t[hit].view(np.uint32), g["t"][hit].view(np.uint32))
    assert np.array_equal(u[hit].view(np.uint32), g["u"][hit].view(np.uint32))
    assert np.array_equal(v[hit].view(np.uint32), g["v"][hit].view(np.uint32))


@pytest.mark.parametrize("case", ["trace_ico4.npz", "trace_soup.npz"])
def test_any_hit_matches_reference(golden, case):
    g = golden(case)
    bvh = O.ploc_build(g["tris"], g["world"], int(g["radius"]), radix_compat=True)
    _, occ, _, _ = O.trace(g["tris"], g["rays"], any_hit=True, bvh=bvh)
    assert np.array_equal(occ, g["occluded"])


def test_brute_force_agrees_where_reference_tree_is_complete(golden):
    """Brute force over all triangles equals the reference except on rays
    whose closest triangle the reference's tree dropped."""
    g = golden("trace_ico4.npz")
    t, p, u, v = O.trace(g["tris"], g["rays"], bvh=None)
    kept = np.zeros(g["tris"].shape[0], bool)
    kept[np.unique(golden("ploc_ico4.npz")["perm"])] = True
    differ = p != g["prim"]
    assert differ.sum() < 0.01 * len(p)
    assert np.all(~kept[p[differ & (p >= 0)]])


@pytest.mark.parametrize("case", ["bsdf.npz", "bsdf_more.npz"])
def test_bsdf_matches_reference(golden, case):
    """Lambertian and Disney (bsdf.npz); mirror, glass, metal, plastic and
    null (bsdf_more.npz; the sample's flag is valid + 2 * delta)."""
    g = golden(case)
    n = g["op"].shape[0]
    out = np.stack([O.bsdf(g["material"][i], g["ng"][i], g["ns"][i], g["wo"][i],
                           g["wi"][i], g["sam"][i], g["op"][i]) for i in range(n)])
    ref = g["out"]
    # the stated bar: f and pdf within 1e-5 relative; the restatement is in
    # fact bit-exact against the reference build
    np.testing.assert_allclose(out[:, :4], ref[:, :4], rtol=1e-5, atol=1e-30)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def same_bits_or_nan(a, b):
    """Bitwise equality, with any NaN equal to any NaN (the payload and sign
    of a NaN depend on the machine that made it)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(
        np.where(na, 0, a).view(np.uint32), np.where(nb, 0, b).view(np.uint32))


@pytest.mark.parametrize("case", ["render_cornell.npz", "render_ico.npz",
                                  "render_cornell_nomis.npz", "render_area.npz",
                                  "render_area_nomis.npz", "render_materials.npz",
                                  "render_materials_nomis.npz"])
def test_render_matches_reference_per_sample(golden, case):
    from ajisai_render_gb300.scenes import FlatScene
    g = golden(case)
    fl = FlatScene(g["tris"], g["corner_n"], g["tri_mat"], g["tri_flags"],
                   g["world"], g["materials"], g["lights"], g["camera"],
                   g["emit_rad"], g["emit_info"])
    p = g["params"]
    params = dict(spp=int(p[0]), min_bounces=int(p[1]), max_bounces=int(p[2]),
                  cont_prob=float(p[3]), use_mis=int(p[4]), radix_compat=1)
    li, film = O.render(fl, params, seed=int(g["seed"]))
    H, W = g["film"].shape[:2]
    assert same_bits_or_nan(li.reshape(H * W, -1, 3), g["li"])
    # the reference sums in float32 over one tile; the oracle in float64
    np.testing.assert_allclose(film[..., :3], g["film"][..., :3], rtol=2e-5,
                               atol=1e-5)
    assert np.array_equal(film[..., 3], g["film"][..., 3])


def test_camera_rays_match_reference(golden):
    g = golden("camera.npz")
    for tag in ("pinhole", "lens"):
        rays = O.camera_rays(g[tag + "_camera"], g[tag + "_raster"])
        assert np.array_equal(rays.view(np.uint32), g[tag + "_rays"].view(np.uint32))


def test_counter_rng_known_answers():
    """Known answers of the counter sampler keys (SplitMix64 finaliser),
    shared by the oracle, the harness and the GPU library."""
    vals = [O.rng(0, 0, 0, 0), O.rng(7, 123, 4, 9), O.rng(2**40 + 3, 2**20, 1023, 77)]
    assert all(0.0 <= v < 1.0 for v in vals)
    # pure-Python restatement of the three functions
    M = (1 << 64) - 1

    def mix(z):
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    def ref(seed, px, s, d):
        key = mix((seed * 0x9E3779B97F4A7C15 + ((px << 32) | s)) & M)
        u = mix((key + (d + 1) * 0x9E3779B97F4A7C15) & M) >> 32
        b = (u >> 9) | 0x3F800000
        return float(np.array([b], np.uint32).view(np.float32)[0]) - 1.0

    for (a, b, c, d), v in zip([(0, 0, 0, 0), (7, 123, 4, 9), (2**40 + 3, 2**20, 1023, 77)], vals):
        assert np.float32(ref(a, b, c, d)) == np.float32(v)


@pytest.mark.parametrize("case", ["sppm_cornell.npz", "sppm_area.npz",
                                  "sppm_materials.npz"])
def test_sppm_matches_reference(golden, case):
    """SPPM (camera pass, visible-point grid, photon tracing from every light
    kind, radius updates) bit for bit against the reference's own SPPM
    functions."""
    from ajisai_render_gb300.scenes import FlatScene
    g = golden(case)
    fl = FlatScene(g["tris"], g["corner_n"], g["tri_mat"], g["tri_flags"],
                   g["world"], g["materials"], g["lights"], g["camera"],
                   g["emit_rad"], g["emit_info"])
    p = g["params"]
    params = dict(iterations=int(p[0]), photons_per_iteration=int(p[1]),
                  forward_max_depth=int(p[2]), photon_min_depth=int(p[3]),
                  photon_max_depth=int(p[4]), photon_cont_prob=float(p[5]),
                  init_radius=float(p[6]), update_alpha=float(p[7]))
    sc = O.OracleScene(fl, search_radius=14, radix_compat=True)
    rad, film = sc.sppm(fl.camera, params, seed=int(g["seed"]))
    assert same_bits_or_nan(rad, g["rad"])
    np.testing.assert_allclose(film[..., :3], g["film"][..., :3], rtol=2e-5, atol=1e-5)
    assert np.array_equal(film[..., 3], g["film"][..., 3])
