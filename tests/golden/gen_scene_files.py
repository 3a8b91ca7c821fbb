"""Writes the scene-file fixtures in the reference's YAML format
(factory/creator/*.cpp keys): the Cornell-style box of
ajisai_render_gb300.scenes.cornell_box, block style, and the same scene in
flow style; scenes.cornell_area with its emitters (and ball.obj, its
emissive mesh).  The cube matrices and mesh vertices are the float32 values
scenes.py uses, printed so that they read back bit for bit.

    python tests/golden/gen_scene_files.py
"""
from pathlib import Path

import numpy as np

import sys
ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from ajisai_render_gb300 import scenes as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "scenes"


def f32(v) -> str:
    """Shortest decimal that reads back (decimal -> float) as the float32."""
    x = np.float32(v)
    return str(int(x)) if float(x).is_integer() else np.format_float_positional(
        x, unique=True, trim="-")


def vec(v) -> str:
    return "[" + ", ".join(f32(x) for x in v) + "]"


def cornell_yaml(flow: bool) -> str:
    sc = S.cornell_box(256, 256)
    mats = {0: (0.73, 0.73, 0.73), 1: (0.65, 0.05, 0.05), 2: (0.12, 0.45, 0.15)}
    lines = ["# Cornell-style box: 5 walls (open front), two rotated boxes,",
             "# a directional light and a constant environment.",
             "scene:", "  type: default", "  primitives:"]
    for p in sc.primitives:
        if isinstance(p, S.Quad):
            geo = (f"{{type: twosided, internal: {{type: quad, a: {vec(p.a)}, "
                   f"b: {vec(p.b)}, c: {vec(p.c)}, d: {vec(p.d)}}}}}")
        else:
            geo = (f"{{type: cube, transform: {{type: matrix, matrix: "
                   f"{vec(p.transform)}}}}}")
        mat = f"{{type: diffuse, albedo: {{type: constant, texel: {vec(mats[p.material])}}}}}"
        if flow:
            lines.append(f"    - {{type: geometry, geometry: {geo}, material: {mat}}}")
        else:
            lines += ["    - type: geometry", f"      geometry: {geo}",
                      "      material:", "        type: diffuse",
                      f"        albedo: {{type: constant, texel: {vec(mats[p.material])}}}"]
    lines += ["  lights:",
              "    - type: directional",
              "      direction: [0.3, 1.0, 0.2]   # toward the light",
              "      emission: [3, 3, 3]",
              "    - type: envmap",
              "      texture:",
              "        type: constant",
              "        texel: 0.2",
              "  aggregate: {type: ploc, search_radius: 14}",
              "camera:",
              "  type: thin_lens",
              "  resolution: [256, 256]",
              "  position: [0, 0, 1.9]",
              "  look_at: [0, 0, 0]",
              "  up: [0, 1, 0]",
              "  fov: 40",
              "renderer:",
              "  type: pt",
              "  spp: 64",
              "  min_bounces: 3",
              "  max_bounces: 8",
              "post_processors:",
              "  - type: save_to_img",
              "    filename: cornell.png"]
    return "\n".join(lines) + "\n"


def _texel(v) -> str:
    return "{type: constant, texel: %s}" % (vec(v) if np.ndim(v) else f32(v))


def _material_yaml(m) -> str:
    if m.type == S.MAT_DIFFUSE:
        return "{type: diffuse, albedo: %s}" % _texel(m.base_color)
    p = list(m.params) if m.params is not None else []
    if m.type == S.MAT_MIRROR:
        return "{type: mirror, kr: %s}" % _texel(m.base_color)
    if m.type == S.MAT_GLASS:
        return ("{type: glass, color_reflection: %s, color_refraction: %s, ior: %s}"
                % (_texel(m.base_color), _texel(p[0:3]), _texel(p[3])))
    if m.type == S.MAT_METAL:
        return ("{type: metal, color: %s, k: %s, eta: %s, uroughness: %s, vroughness: %s}"
                % (_texel(m.base_color), _texel(p[0:3]), _texel(p[3:6]), f32(p[6]),
                   f32(p[7])))
    if m.type == S.MAT_PLASTIC:
        return ("{type: plastic, albedo: %s, ior: %s, thickness: %s, sigma_a: %s}"
                % (_texel(m.base_color), f32(p[0]), f32(p[1]), f32(p[2])))
    keys = ("subsurface", "metallic", "specular", "specular_tint", "roughness",
            "anisotropic", "sheen", "sheen_tint", "clearcoat", "clearcoat_gloss")
    return "{type: disney, base_color: %s, %s}" % (
        _texel(m.base_color),
        ", ".join(f"{k}: {_texel(getattr(m, k))}" for k in keys))


def scene_files(sc, header, obj_name, lights, env) -> tuple[str, str]:
    """A scene of quads, cubes and one mesh (written to `obj_name`, with its
    normals when it has them) as a scene file."""
    obj = ["# " + header[0]]
    lines = ["# " + h for h in header] + ["scene:", "  type: default", "  primitives:"]
    for p in sc.primitives:
        if isinstance(p, S.Quad):
            geo = (f"{{type: quad, a: {vec(p.a)}, b: {vec(p.b)}, c: {vec(p.c)}, "
                   f"d: {vec(p.d)}}}")
        elif isinstance(p, S.Cube):
            geo = (f"{{type: cube, transform: {{type: matrix, matrix: "
                   f"{vec(p.transform)}}}}}")
        else:
            for v in p.positions:
                obj.append("v " + " ".join(f32(x) for x in v))
            if p.normals is not None:
                for v in p.normals:
                    obj.append("vn " + " ".join(f32(x) for x in v))
                for t in p.indices:
                    obj.append("f " + " ".join(f"{int(i) + 1}//{int(i) + 1}" for i in t))
            else:
                for t in p.indices:
                    obj.append("f " + " ".join(str(int(i) + 1) for i in t))
            geo = f"{{type: mesh, filename: {obj_name}}}"
        if p.two_sided:
            geo = f"{{type: twosided, internal: {geo}}}"
        lines += ["    - type: geometry", f"      geometry: {geo}"]
        mat = sc.materials[p.material]
        if mat.type != S.MAT_NULL:  # the null material is the absent node
            lines.append(f"      material: {_material_yaml(mat)}")
        if p.emission is not None:
            lines.append(f"      emission: {vec(p.emission)}")
    lines += ["  lights:",
              f"    - {{type: directional, direction: [0.3, 1.0, 0.2], emission: {lights}}}",
              f"    - {{type: envmap, texture: {{type: constant, texel: {env}}}}}",
              "  aggregate: {type: ploc, search_radius: 14}",
              "camera: {type: thin_lens, resolution: [256, 256], position: [0, 0, 1.9],",
              "         look_at: [0, 0, 0], up: [0, 1, 0], fov: 40}",
              "renderer: {type: pt, spp: 64, min_bounces: 3, max_bounces: 8}"]
    return "\n".join(lines) + "\n", "\n".join(obj) + "\n"


if __name__ == "__main__":
    OUT.mkdir(exist_ok=True)
    (OUT / "cornell_box.yaml").write_text(cornell_yaml(False))
    (OUT / "cornell_box_flow.yaml").write_text(cornell_yaml(True))
    yml, obj = scene_files(S.cornell_area(256, 256),
                           ["scenes.cornell_area: the box lit by a one-sided ceiling quad, a",
                            "two-sided quad, an emissive icosphere mesh and an emissive cube."],
                           "ball.obj", "[1, 1, 1]", "0.05")
    (OUT / "cornell_area.yaml").write_text(yml)
    (OUT / "ball.obj").write_text(obj)
    yml, obj = scene_files(S.material_box(256, 256),
                           ["scenes.material_box: plastic, mirror, metal, glass and a",
                            "null-material emitter."],
                           "glass_ball.obj", "[1, 1, 1]", "0.1")
    (OUT / "material_box.yaml").write_text(yml)
    (OUT / "glass_ball.obj").write_text(obj)
    print("wrote", OUT)
