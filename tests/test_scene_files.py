"""The host side of the drop-in: Ajisai YAML scene files (the reference's
factory keys) and OBJ meshes read into the flat scene the C ABI takes, and
the film written as PFM / PNG.  CPU only (no CUDA in the host library),
except the last test, which runs the command line on the GPU."""
import struct
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

from ajisai_render_gb300 import api
from ajisai_render_gb300 import scenes as S

GOLDEN = Path(__file__).resolve().parent / "golden" / "scenes"


@pytest.fixture(scope="module", autouse=True)
def host_lib():
    from ajisai_render_gb300 import build
    build.build_host()


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", ["cornell_box.yaml", "cornell_box_flow.yaml"])
def test_cornell_scene_file_matches_the_python_scene(name):
    """Block and flow style read to the same flat scene as
    scenes.cornell_box -- triangles, flags, materials, lights, bounds and the
    camera matrices bit for bit."""
    f = api.load_scene_file(GOLDEN / name)
    ref = S.flatten(S.cornell_box(256, 256))
    assert same_bits(f.flat.tris, ref.tris)
    assert np.array_equal(f.flat.tri_flags, ref.tri_flags)
    assert same_bits(f.flat.world, ref.world)
    # one material per primitive in the file: compare through the triangles
    assert same_bits(f.flat.materials[f.flat.tri_mat], ref.materials[ref.tri_mat])
    assert same_bits(f.flat.lights, ref.lights)
    assert same_bits(f.camera, ref.camera)
    assert (f.args.spp, f.args.min_bounces, f.args.max_bounces) == (64, 3, 8)
    assert f.args.use_mis and f.args.cont_prob == np.float32(0.9)
    assert f.aggregate.search_radius == 14
    assert f.outputs == ["cornell.png.png"]  # filename + "." + ext


def test_area_scene_file_reads_its_emitters():
    """`emission` on quad, two-sided quad, mesh and cube primitives: the same
    triangles, emitters (first triangle, count, geometry, sidedness,
    radiance) and lights as scenes.cornell_area; the OBJ mesh carries the
    normals the reference's loader computes."""
    f = api.load_scene_file(GOLDEN / "cornell_area.yaml")
    ref = S.flatten(S.cornell_area(256, 256))
    assert same_bits(f.flat.tris, ref.tris)
    first, count = ref.emit_info[2, 0], ref.emit_info[2, 1]
    flags = f.flat.tri_flags.copy()
    assert np.all(flags[first:first + count] & S.TRI_HAS_NORMALS)
    flags[first:first + count] &= ~S.TRI_HAS_NORMALS
    assert np.array_equal(flags, ref.tri_flags)
    assert np.array_equal(f.flat.emit_info, ref.emit_info)
    assert same_bits(f.flat.emit_rad, ref.emit_rad)
    assert same_bits(f.flat.lights, ref.lights)
    assert same_bits(f.flat.materials[f.flat.tri_mat], ref.materials[ref.tri_mat])
    assert same_bits(f.camera, ref.camera)


def test_material_scene_file_reads_every_material():
    """mirror, glass, metal and plastic nodes and a primitive without a
    material (the null material) read to scenes.material_box's records; the
    glass ball's OBJ carries its normals."""
    f = api.load_scene_file(GOLDEN / "material_box.yaml")
    ref = S.flatten(S.material_box(256, 256))
    assert same_bits(f.flat.tris, ref.tris)
    assert np.array_equal(f.flat.tri_flags, ref.tri_flags)
    # the loader normalises the file's normals (the Python mesh keeps them)
    m = ref.tri_flags & S.TRI_HAS_NORMALS > 0
    np.testing.assert_allclose(f.flat.corner_n[m], ref.corner_n[m], rtol=0, atol=3e-7)
    assert same_bits(f.flat.materials[f.flat.tri_mat], ref.materials[ref.tri_mat])
    assert np.array_equal(f.flat.emit_info, ref.emit_info)
    assert same_bits(f.flat.emit_rad, ref.emit_rad)
    assert same_bits(f.flat.lights, ref.lights)


def write_obj(path, pos, idx, nrm=None, quads=False):
    with open(path, "w") as fh:
        fh.write("# test mesh\no mesh\n")
        for p in pos:
            fh.write("v %r %r %r\n" % tuple(float(x) for x in p))
        if nrm is not None:
            for n in nrm:
                fh.write("vn %r %r %r\n" % tuple(float(x) for x in n))
        for t in idx:
            if nrm is not None:
                fh.write("f " + " ".join(f"{i + 1}//{i + 1}" for i in t) + "\n")
            else:
                fh.write("f " + " ".join(str(i + 1) for i in t) + "\n")


def mesh_yaml(obj, transform=None, material="diffuse"):
    xf = ""
    if transform is not None:
        xf = ", transform: {type: matrix, matrix: [%s]}" % ", ".join(
            np.format_float_positional(np.float32(v), unique=True, trim="-")
            for v in transform)
    mat = ("{type: diffuse, albedo: {type: constant, texel: 0.5}}" if material == "diffuse"
           else "{type: disney, base_color: {type: constant, texel: [0.8, 0.3, 0.2]}, "
                "subsurface: {type: constant, texel: 0}, metallic: {type: constant, texel: 0.4},"
                " specular: {type: constant, texel: 0.5}, specular_tint: {type: constant,"
                " texel: 0}, roughness: {type: constant, texel: [0.35, 0.9, 0.9]},"
                " anisotropic: {type: constant, texel: 0}, sheen: {type: constant, texel: 0},"
                " sheen_tint: {type: constant, texel: 0}, clearcoat: {type: constant,"
                " texel: 0.2}, clearcoat_gloss: {type: constant, texel: 0.7}}")
    return f"""scene:
  primitives:
    - type: geometry
      geometry: {{type: mesh, filename: {obj}{xf}}}
      material: {mat}
  lights:
    - {{type: envmap, texture: {{type: constant, texel: [0.5, 0.5, 0.5]}}, scaler: 2, rot: 30}}
camera: {{type: thin_lens, resolution: [32, 24], position: [0, 0, 4], look_at: [0, 0, 0],
         up: [0, 1, 0], fov: 45, lens_radius: 0.05, focal_distance: 4}}
renderer: {{type: pt_gpu, spp: 8}}
"""


def test_mesh_with_normals_and_transform(tmp_path):
    pos, nrm, idx = S.displaced_icosphere(2, 1)
    write_obj(tmp_path / "m.obj", pos, idx, nrm)
    xf = [2, 0, 0, 0.5, 0, 2, 0, -1, 0, 0, 2, 0.25, 0, 0, 0, 1]
    (tmp_path / "s.yaml").write_text(mesh_yaml("m.obj", xf, "disney"))
    f = api.load_scene_file(tmp_path / "s.yaml")
    m = S.yaml_matrix(xf)
    tpos = S.transform_point(m, pos)
    # Matrix4::transformVector then normalized, in float32
    tn = np.zeros_like(nrm)
    for row in range(3):
        acc = np.zeros(len(nrm), np.float32)
        for col in range(3):
            acc = acc + m[col][row] * nrm[:, col]
        tn[:, row] = acc
    ln = np.sqrt(np.float32(0) + tn[:, 0] * tn[:, 0] + tn[:, 1] * tn[:, 1] + tn[:, 2] * tn[:, 2])
    tn = tn * (np.float32(1) / ln)[:, None]
    assert same_bits(f.flat.tris, tpos[idx].reshape(-1, 9))
    assert same_bits(f.flat.corner_n, tn[idx].reshape(-1, 9))
    assert np.all(f.flat.tri_flags == S.TRI_HAS_NORMALS)
    mat = f.flat.materials[0]
    assert mat[0] == 1 and np.allclose(mat[1:4], [0.8, 0.3, 0.2])
    assert mat[5] == np.float32(0.4) and mat[8] == np.float32(0.35)  # SampleReal: texel[0]
    assert same_bits(f.flat.world, np.concatenate([tpos.min(0), tpos.max(0)]))
    env = f.flat.lights[0]
    assert env[0] == 1 and env[8] == 2 and env[9] == 30
    cam = S.Camera((0, 0, 4), (0, 0, 0), (0, 1, 0), 45, 32, 24, 0.05, 4)
    assert same_bits(f.camera, cam.pack())


def test_mesh_without_normals_takes_the_first_face_normal(tmp_path):
    """A vertex shared by several faces gets the normal of the first face
    that uses it (the reference's loader computes it once per new vertex)."""
    pos, _, idx = S.displaced_icosphere(1, 2)
    write_obj(tmp_path / "m.obj", pos, idx)
    (tmp_path / "s.yaml").write_text(mesh_yaml(str(tmp_path / "m.obj")))
    f = api.load_scene_file(tmp_path / "s.yaml")
    first = {}
    for t in idx:
        a, b, c = pos[t[0]], pos[t[1]], pos[t[2]]
        e0, e1 = b - a, c - a
        n = np.array([e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2],
                      e0[0] * e1[1] - e0[1] * e1[0]], np.float32)
        n = n * (np.float32(1) / np.sqrt(np.float32(0) + n[0] * n[0] + n[1] * n[1] + n[2] * n[2]))
        for v in t:
            first.setdefault(int(v), n)
    expect = np.stack([np.concatenate([first[int(v)] for v in t]) for t in idx])
    np.testing.assert_allclose(f.flat.corner_n, expect, rtol=2e-6, atol=2e-7)


def test_polygons_are_split_into_fans(tmp_path):
    (tmp_path / "q.obj").write_text(
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0.5 1.5 0\nf 1 2 3 5 4\nf -3 -2 -1\n")
    (tmp_path / "s.yaml").write_text(mesh_yaml(str(tmp_path / "q.obj")))
    f = api.load_scene_file(tmp_path / "s.yaml")
    assert f.flat.n_tris == 4
    t = f.flat.tris.reshape(-1, 3, 3)
    assert np.array_equal(t[0], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    assert np.array_equal(t[2], [[0, 0, 0], [0.5, 1.5, 0], [0, 1, 0]])
    assert np.array_equal(t[3], [[1, 1, 0], [0, 1, 0], [0.5, 1.5, 0]])


@pytest.mark.parametrize("snippet,message", [
    ("{type: geometry, geometry: {type: sphere, radius: 1, center: [0, 0, 0]},"
     " material: {type: diffuse, albedo: {type: constant, texel: 0.5}}}", "sphere"),
    ("{type: geometry, geometry: {type: quad}, material: {type: velvet}}", "velvet"),
    ("{type: geometry, geometry: {type: quad},"
     " material: {type: diffuse, albedo: {type: image, filename: a.png}}}", "constant"),
    ("{type: geometry, geometry: {type: quad}, material: {type: diffuse},"
     " med_in: {type: homogeneous}}", "media"),
])
def test_unsupported_nodes_are_refused_with_the_reason(tmp_path, snippet, message):
    (tmp_path / "s.yaml").write_text(f"""scene:
  primitives:
    - {snippet}
camera: {{type: thin_lens, resolution: [8, 8], position: [0, 0, 3], look_at: [0, 0, 0],
         up: [0, 1, 0], fov: 40}}
renderer: {{type: pt, spp: 1}}
""")
    with pytest.raises(ValueError) as e:
        api.load_scene_file(tmp_path / "s.yaml")
    assert message in str(e.value) and "s.yaml" in str(e.value)


def test_yaml_syntax_errors_name_the_line(tmp_path):
    (tmp_path / "s.yaml").write_text("scene:\n  primitives: [a, b\ncamera: 1\n")
    with pytest.raises(ValueError) as e:
        api.load_scene_file(tmp_path / "s.yaml")
    assert "YAML line" in str(e.value)


def read_png(path):
    data = Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xffffffff
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def test_png_and_pfm_output(tmp_path):
    rng = np.random.default_rng(3)
    h, w = 13, 17
    rgbw = np.zeros((h, w, 4), np.float32)
    rgbw[..., :3] = rng.uniform(0, 3, (h, w, 3))
    rgbw[..., 3] = rng.integers(0, 4, (h, w))
    api.write_image(tmp_path / "a.png", rgbw)
    api.write_image(tmp_path / "a.pfm", rgbw)
    wgt = rgbw[..., 3:4]
    img = np.where(wgt != 0, rgbw[..., :3] / np.where(wgt != 0, wgt, 1), 0).astype(np.float32)
    a = np.float32(0.055)
    srgb = np.where(img > np.float32(0.0031308),
                    (np.float32(1) + a) * np.power(img, np.float32(1) / np.float32(2.4)) - a,
                    img * np.float32(12.92)).astype(np.float32)
    expect = np.clip(np.round(np.clip(srgb, 0, 1).astype(np.float64) * 255.5), 0, 255)
    got = read_png(tmp_path / "a.png")
    # rows flipped on write; powf may differ from numpy's in the last ulp
    assert np.abs(got.astype(int) - expect[::-1].astype(int)).max() <= 1
    assert (got == expect[::-1]).mean() > 0.99
    pfm = (tmp_path / "a.pfm").read_bytes()
    head = b"PF\n%d %d\n-1.0\n" % (w, h)
    assert pfm.startswith(head)
    body = np.frombuffer(pfm[len(head):], "<f4").reshape(h, w, 3)
    assert same_bits(body, img[::-1])


def test_film_pfm_writers_agree(tmp_path):
    rgbw = np.random.default_rng(1).uniform(0, 2, (6, 9, 4)).astype(np.float32)
    film = api.Film(9, 6)
    film.rgbw[...] = rgbw
    film.write_pfm(tmp_path / "py.pfm")
    api.write_image(tmp_path / "c.pfm", rgbw)
    assert (tmp_path / "py.pfm").read_bytes() == (tmp_path / "c.pfm").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell_box.yaml", "cornell_area.yaml",
                                  "material_box.yaml"])
def test_command_line_renders_the_scene_file(tmp_path, name):
    """ajisai_gpu -s scene.yaml: the film equals the Python API's render of
    the same file (with and without emitters)."""
    from ajisai_render_gb300 import build
    build.build()
    build.build_host()
    src = (GOLDEN / name).read_text().replace("spp: 64", "spp: 8") \
        .replace("resolution: [256, 256]", "resolution: [64, 48]")
    for obj in ("ball.obj", "glass_ball.obj"):
        (tmp_path / obj).write_text((GOLDEN / obj).read_text())
    (tmp_path / "c.yaml").write_text(src.replace("filename: cornell.png",
                                                 f"filename: {tmp_path / 'out.png'}"))
    r = subprocess.run([str(build.CLI), "-s", str(tmp_path / "c.yaml"), "--out",
                        str(tmp_path / "c.pfm"), "--seed", "5"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    if name == "cornell_box.yaml":
        assert (tmp_path / "out.png.png").exists()
    f = api.load_scene_file(tmp_path / "c.yaml")
    ctx = api.Context(0)
    try:
        sc = api.GpuScene(ctx, f.flat, f.aggregate)
        film = api.PTRenderer(f.args, seed=5).Render(sc, f.camera)
        film.write_pfm(tmp_path / "py.pfm")
    finally:
        ctx.close()
    assert (tmp_path / "c.pfm").read_bytes() == (tmp_path / "py.pfm").read_bytes()


def test_sppm_renderer_node(tmp_path):
    """renderer: {type: sppm, ...} reads SPPMCreatorImpl's keys and defaults."""
    src = (GOLDEN / "cornell_box.yaml").read_text()
    i = src.index("renderer:")
    j = src.index("post_processors:")
    (tmp_path / "s.yaml").write_text(
        src[:i] + "renderer: {type: sppm, iteration_count: 12, init_radius: 0.02,"
        " photon_max_depth: 7}\n" + src[j:])
    f = api.load_scene_file(tmp_path / "s.yaml")
    assert isinstance(f.args, api.SPPMRendererArgs)
    assert (f.args.iteration_count, f.args.photon_max_depth) == (12, 7)
    assert f.args.init_radius == np.float32(0.02)
    assert (f.args.forward_max_depth, f.args.photons_per_iteration,
            f.args.photon_min_depth) == (8, 100000, 5)
    assert f.args.update_alpha == np.float32(2.0 / 3)


@pytest.mark.gpu
def test_command_line_renders_sppm(tmp_path):
    """ajisai_gpu with an sppm renderer node: the image agrees with the
    Python API's SPPM render of the same file (deposits are summed
    atomically, so to float tolerance)."""
    from ajisai_render_gb300 import build
    build.build()
    build.build_host()
    src = (GOLDEN / "cornell_box.yaml").read_text() \
        .replace("resolution: [256, 256]", "resolution: [64, 64]")
    i, j = src.index("renderer:"), src.index("post_processors:")
    src = (src[:i] + "renderer: {type: sppm, iteration_count: 3,"
           " photons_per_iteration: 20000, init_radius: 0.03, forward_max_depth: 6}\n"
           + src[j:])
    (tmp_path / "c.yaml").write_text(src.replace("filename: cornell.png",
                                                 f"filename: {tmp_path / 'out.png'}"))
    r = subprocess.run([str(build.CLI), "-s", str(tmp_path / "c.yaml"), "--out",
                        str(tmp_path / "c.pfm"), "--seed", "4"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Mphotons/s" in r.stdout
    f = api.load_scene_file(tmp_path / "c.yaml")
    ctx = api.Context(0)
    try:
        sc = api.GpuScene(ctx, f.flat, f.aggregate)
        film = api.SPPMRenderer(f.args, seed=4).Render(sc, f.camera)
    finally:
        ctx.close()
    data = (tmp_path / "c.pfm").read_bytes()
    cli = np.frombuffer(data[data.index(b"-1.0\n") + 5:], "<f4").reshape(64, 64, 3)[::-1]
    np.testing.assert_allclose(cli, film.image(), rtol=1e-3, atol=1e-5)
