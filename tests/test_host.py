"""Host-side scene description: the flat layout matches what the
reference's aggregate gathers, and the camera matrices match ThinLensCamera.
CPU only."""
import numpy as np

from ajisai_render_gb300 import scenes as S


def test_cornell_flatten_matches_reference_gather(golden):
    g = golden("render_cornell.npz")
    fl = S.flatten(S.cornell_box(32, 32))
    assert np.array_equal(fl.tris, g["tris"])
    assert np.array_equal(fl.tri_flags, g["tri_flags"])
    assert np.array_equal(fl.tri_mat, g["tri_mat"])
    assert np.array_equal(fl.world, g["world"])


def test_icosphere_flatten_matches_reference_gather(golden):
    g = golden("render_ico.npz")
    fl = S.flatten(S.icosphere_scene(subdiv=3, seed=5, width=24, height=24))
    assert np.array_equal(fl.tris, g["tris"])
    assert np.array_equal(fl.corner_n, g["corner_n"])
    assert np.array_equal(fl.tri_flags, g["tri_flags"])


def test_camera_matrices_close_to_reference(golden):
    g = golden("render_cornell.npz")
    mine = S.cornell_box(32, 32).camera.pack()
    np.testing.assert_allclose(mine, g["camera"], rtol=1e-6, atol=1e-9)
    g2 = golden("camera.npz")
    cam = S.Camera((1.0, 0.5, 3.0), (0, 0.1, 0), (0, 1, 0), 50.0, 40, 30,
                   lens_radius=0.08, focal_distance=3.1)
    np.testing.assert_allclose(cam.pack(), g2["lens_camera"], rtol=2e-6, atol=1e-8)


def test_icosphere_sizes():
    v, f = S.icosphere(3)
    assert f.shape == (20 * 4 ** 3, 3)
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
    # closed manifold: every edge shared by two faces
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)


def test_light_and_material_records():
    d = S.DirectionalLight((0.3, 1.0, 0.2), 3.0).pack()
    assert d[0] == S.LIGHT_DIRECTIONAL and d[7] == 1.0 and list(d[1:4]) == [3, 3, 3]
    e = S.EnvLight(0.2).pack()
    assert e[0] == S.LIGHT_ENV and e[8] == 1.0
    m = S.Disney((0.1, 0.2, 0.3), roughness=0.4, clearcoat=0.5).pack()
    assert m[0] == S.MAT_DISNEY and m[8] == np.float32(0.4) and m[12] == 0.5
