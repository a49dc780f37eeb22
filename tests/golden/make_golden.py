#!/usr/bin/env python3
"""Regenerates the golden fixtures in tests/golden/ (run where the reference sources exist).

texture_kats.json
    The known-answer assertions of the reference's own texture test
    (Source/test/tests/TextureTest.cpp), read from that file as text: pyramid fields,
    texel offsets, pixel reads after writes, nearest sampling and the 8-bit linear mix.
occlusion_sessions.json
    The renderer session of tests/occlusion_script.py (occlusion grid: box occluders, existing
    triangles, top rows, box tests, two frames) played by the reference: its answers and the
    sha256 of its images, for seeded scenes whose inputs are identified by their own digest.
texture_resize.json
    texture_create_RgbaU8 of seeded images whose sizes are not powers of two (filter_resize to
    the next powers of two, then the pyramid), by the reference: fields and pyramid digests.
render_*.npz
    Small seeded scenes (inputs stored in the file) rendered by the reference itself, built
    from its sources as the exact (scalar, no-FMA) variant by oracle/Makefile.ref, through
    model_render / renderer_* / model_renderDepth.

Usage: python tests/golden/make_golden.py [reference root, default $DFPSR_REFERENCE or a
`reference` checkout beside the repository]
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def f32_expr(text):
    """Evaluates a C float expression of literals, +, -, *, / and parentheses in binary32."""
    tokens = re.findall(r"\d+\.\d*f?|\d+f|\d+u?|[-+*/()]", text.replace(" ", ""))

    def literal(tok):
        return np.float32(float(tok.rstrip("fu")))

    pos = 0

    def expr():
        nonlocal pos
        value = term()
        while pos < len(tokens) and tokens[pos] in "+-":
            op = tokens[pos]; pos += 1
            rhs = term()
            value = np.float32(value + rhs) if op == "+" else np.float32(value - rhs)
        return value

    def term():
        nonlocal pos
        value = factor()
        while pos < len(tokens) and tokens[pos] in "*/":
            op = tokens[pos]; pos += 1
            rhs = factor()
            value = np.float32(value * rhs) if op == "*" else np.float32(value / rhs)
        return value

    def factor():
        nonlocal pos
        tok = tokens[pos]
        if tok == "-":
            pos += 1
            return np.float32(-factor())
        if tok == "(":
            pos += 1
            v = expr()
            pos += 1
            return v
        pos += 1
        return literal(tok)

    return float(expr())


def split_args(text):
    depth, cur, out = 0, "", []
    for ch in text:
        if ch == "," and depth == 0:
            out.append(cur.strip()); cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def int_literal(tok):
    tok = tok.strip().rstrip("u")
    return int(tok, 2) if tok.startswith("0b") else int(tok)


def lanes(tok):
    m = re.match(r"U32x(\d+)\((.*)\)$", tok.strip())
    vals = [int_literal(v) for v in split_args(m.group(2))]
    n = int(m.group(1))
    return vals * n if len(vals) == 1 else vals


def texture_kats(reference_root):
    path = os.path.join(reference_root, "Source", "test", "tests", "TextureTest.cpp")
    blocks, current, mix = [], None, []
    for raw in open(path, encoding="utf-8-sig"):
        line = raw.strip()
        m = re.match(r"TextureRgbaU8 texture = TextureRgbaU8\((.*)\);", line)
        if m:
            args = [int(a) for a in split_args(m.group(1))]
            current = {"log2w": args[0], "log2h": args[1], "maxMip": args[2] if len(args) > 2 else 15,
                       "fields": {}, "layer": [], "offset": [], "writes": [], "read": [], "nearest": []}
            blocks.append(current)
            continue
        if line.startswith("U32x4 mixedColor = texture_interpolate_color_linear"):
            mix.append(line)
            continue
        if mix and len(mix) < 8 and not line.startswith("ASSERT_EQUAL_SIMD(mixedColor"):
            mix.append(line)
            continue
        if current is None:
            continue
        m = re.match(r"ASSERT_EQUAL\(texture\.impl_(\w+)\s*,\s*(\w+)\);", line)
        if m:
            current["fields"][m.group(1)] = int_literal(m.group(2)); continue
        m = re.match(r"ASSERT_EQUAL\(texture_get(MaxWidth|MaxHeight|SmallestMipLevel)\(texture\),\s*(\d+)\);", line)
        if m:
            current["fields"][m.group(1)] = int(m.group(2)); continue
        m = re.match(r"ASSERT\((!?)texture_hasPyramid\(texture\)\);", line)
        if m:
            current["fields"]["hasPyramid"] = 0 if m.group(1) else 1; continue
        m = re.match(r"ASSERT_EQUAL\(texture_getPixelOffsetToLayer\(texture,\s*(\w+)\),\s*(\w+)\);", line)
        if m:
            current["layer"].append([int_literal(m.group(1)), int_literal(m.group(2))]); continue
        m = re.match(r"ASSERT_EQUAL\(texture_getPixelOffset\(texture,(.*)\),\s*(\w+)\);", line)
        if m:
            a = [int_literal(v) for v in split_args(m.group(1))]
            current["offset"].append(a + [int_literal(m.group(2))]); continue
        m = re.match(r"ASSERT_EQUAL_SIMD\(texture_getPixelOffset\(texture, (.*)\), (U32x\d+\(.*\))\);", line)
        if m:
            xs, ys, ms = [lanes(v) for v in split_args(m.group(1))]
            expected = lanes(m.group(2))
            for x, y, mm, e in zip(xs, ys, ms, expected):
                current["offset"].append([x, y, mm, e])
            continue
        m = re.match(r"texture_writePixel\(texture,(.*)\);", line)
        if m:
            current["writes"].append([int_literal(v) for v in split_args(m.group(1))]); continue
        m = re.match(r"ASSERT_EQUAL\(texture_readPixel\(texture,(.*)\),\s*(\w+)\);", line)
        if m:
            current["read"].append([int_literal(v) for v in split_args(m.group(1))] + [int_literal(m.group(2))]); continue
        m = re.match(r"ASSERT_EQUAL\(texture_sample_nearest\(texture,(.*)\),\s*(\w+)\);", line)
        if m:
            a = split_args(m.group(1))
            current["nearest"].append([f32_expr(a[0]), f32_expr(a[1]), int_literal(a[2]), int_literal(m.group(2))]); continue
    # the 8-bit linear mix: four packed lanes of colour A, colour B, weight and the expected result
    text = " ".join(mix)
    packs = re.findall(r"packOrder_packBytes\((U32x4\([^)]*\)), (U32x4\([^)]*\)), (U32x4\([^)]*\)), (U32x4\([^)]*\))\)", text)
    weight = lanes(re.search(r"\),\s*(U32x4\([^)]*\))\s*\);", text).group(1))
    expect_text = open(path, encoding="utf-8-sig").read()
    em = re.search(r"U32x4 expectedColor = packOrder_packBytes\((U32x4\([^)]*\)), (U32x4\([^)]*\)), (U32x4\([^)]*\)), (U32x4\([^)]*\))\);", expect_text)

    def pack(groups):
        ch = [lanes(g) for g in groups]
        return [ch[0][i] | (ch[1][i] << 8) | (ch[2][i] << 16) | (ch[3][i] << 24) for i in range(4)]

    linear = {"a": pack(packs[0]), "b": pack(packs[1]), "weight": weight, "expected": pack(em.groups())}
    return {"source": "Source/test/tests/TextureTest.cpp", "textures": blocks, "linear_mix": linear}


def render_cases():
    from dfpsr_gb300 import scenes
    cases = {}
    cases["random_small"] = scenes.random_triangles(seed=101, triangles=260, width=128, height=96, texture_size=64)
    cases["terrain_small"] = scenes.terrain(seed=102, grid=48, width=160, height=96, texture_size=64, camera_height=40.0)
    clip = scenes.random_triangles(seed=103, triangles=400, width=128, height=96, texture_size=32)
    clip.camera_location = scenes.camera_location((0.1, 0.2, -0.3), (0.0, 0.0, 1.0))
    cases["near_clipping"] = clip
    base = scenes.random_triangles(seed=104, triangles=200, width=96, height=72, texture_size=32)
    cases["variant_untextured"] = scenes.with_variant(base, texture=False)
    cases["variant_colorless"] = scenes.with_variant(base, colors="white")
    cases["variant_lightmap"] = scenes.with_variant(base, light=True)
    ortho = scenes.random_triangles(seed=105, triangles=240, width=96, height=80, texture_size=32)
    ortho.perspective = False
    ortho.slope = 1.3
    cases["orthogonal"] = ortho
    return cases


def save_case(name, scene, variant="exact"):
    from oracle import ref
    model = ref.RefModel(scene, variant)
    color, depth = model.render()
    threaded_color, threaded_depth = model.render(threaded=True)
    assert np.array_equal(color, threaded_color) and np.array_equal(depth.view(np.uint32), threaded_depth.view(np.uint32))
    bgra, _ = model.render(pack_order=1)
    depth_only = model.render_depth()
    payload = dict(width=scene.width, height=scene.height, positions=scene.positions, poly_indices=scene.poly_indices,
                   tex_coords=scene.tex_coords, colors=scene.colors, filter=scene.filter,
                   camera_location=scene.camera_location, perspective=int(scene.perspective), slope=scene.slope,
                   near_clip=scene.near_clip, far_clip=scene.far_clip, model_to_world=scene.model_to_world,
                   diffuse_levels=scene.diffuse_levels, light_levels=scene.light_levels,
                   color=color, depth=depth, color_bgra=bgra, depth_only=depth_only)
    if scene.diffuse is not None:
        payload["diffuse"] = scene.diffuse
    if scene.light is not None:
        payload["light"] = scene.light
    np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), **payload)


OCCLUSION_CASES = {"perspective": dict(seed=77, width=160, height=120, props=16, field_triangles=600, perspective=True),
                   "orthogonal": dict(seed=78, width=160, height=120, props=16, field_triangles=600, perspective=False)}


def scene_digest(sc):
    """sha256 of a session's inputs, so that a change of the seeded generator is caught."""
    import hashlib
    h = hashlib.sha256()
    for s in [sc.camera, sc.wall, sc.panel, sc.field] + list(sc.props):
        for a in (s.positions, s.poly_indices, s.tex_coords, s.colors, s.camera_location, s.model_to_world):
            h.update(np.ascontiguousarray(a).tobytes())
        if s.diffuse is not None:
            h.update(np.ascontiguousarray(s.diffuse).tobytes())
    h.update(sc.depth.tobytes())
    h.update(sc.color.tobytes())
    return h.hexdigest()


def image_digest(a):
    import hashlib
    return None if a is None else hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def occlusion_sessions():
    """The occlusion-grid session of tests/occlusion_script.py played by the reference itself:
    box-test answers, hasOccluders and digests of every frame's images."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import occlusion_script
    from dfpsr_gb300 import scenes
    out = {}
    for name, params in OCCLUSION_CASES.items():
        sc = scenes.occlusion_scene(**params)
        for use_color, use_depth, debug in ((True, True, False), (True, False, False), (False, True, False), (True, True, True)):
            r = occlusion_script.play(occlusion_script.RefEngine(), sc, use_color=use_color, use_depth=use_depth, debug=debug)
            out[f"{name}_c{int(use_color)}d{int(use_depth)}{'_debug' if debug else ''}"] = dict(
                params=params, use_color=use_color, use_depth=use_depth, debug=debug, inputs=scene_digest(sc),
                visible=r["visible"], has_occluders=r["has_occluders"],
                frames=[[image_digest(f[0]), image_digest(f[1])] for f in r["frames"]])
    return out


TEXTURE_RESIZE_CASES = [(1, 1, 16), (3, 5, 16), (20, 12, 16), (12, 20, 3), (100, 60, 16), (60, 100, 2), (64, 48, 16),
                        (48, 64, 16), (129, 31, 5), (255, 257, 16), (33, 2, 16), (300, 256, 16), (256, 300, 16)]


def texture_resize_image(w, h):
    rng = np.random.default_rng(1000 * w + h)
    return rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)


def texture_resizes():
    """texture_create_RgbaU8 of images that are not powers of two (filter_resize, then the
    pyramid) by the reference itself: fields and the sha256 of the pyramid buffer."""
    import hashlib
    from oracle import ref
    lib = ref._load("exact")
    out = []
    for w, h, levels in TEXTURE_RESIZE_CASES:
        fields, pixels = ref.RefTexture(lib, texture_resize_image(w, h), levels).info()
        out.append(dict(width=w, height=h, resolutions=levels, fields=[int(v) for v in fields],
                        pyramid=hashlib.sha256(pixels.tobytes()).hexdigest()))
    return out


DENSE_CASES = [  # (seed, view index, prefilled, high quality)
    (60, 0, False, False), (61, 2, True, True), (62, 5, False, True), (63, 7, True, False),
]


def dense_renders():
    """renderDenseModel of the reference itself on seeded dense scenes: the sha256 of the height,
    diffuse and normal images it leaves."""
    from dfpsr_gb300 import scenes
    from oracle import ref
    out = []
    for seed, view_index, prefilled, high_quality in DENSE_CASES:
        sc = scenes.dense_scene(seed=seed, view_index=view_index, prefilled=prefilled)
        h, d, n = ref.dense_render(sc.positions, sc.polygons, sc.colors, sc.camera_tilt, sc.pixels_per_tile, sc.view_index,
                                   sc.height, sc.diffuse, sc.normal, sc.origin, sc.model_to_world, high_quality)
        out.append(dict(seed=seed, view_index=view_index, prefilled=prefilled, high_quality=high_quality,
                        inputs=image_digest(np.concatenate([sc.positions.reshape(-1), sc.colors.reshape(-1), sc.model_to_world,
                                                            sc.height.reshape(-1)]).view(np.uint32)),
                        height=image_digest(h.view(np.uint32)), diffuse=image_digest(d), normal=image_digest(n)))
    return out


def main():
    reference_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(
        "DFPSR_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "..", "reference"))
    from oracle import ref
    os.environ["DFPSR_REFERENCE"] = reference_root
    if not ref.build():
        raise SystemExit("the reference could not be built from " + reference_root)
    with open(os.path.join(HERE, "texture_kats.json"), "w") as f:
        json.dump(texture_kats(reference_root), f, indent=0)
    for name, scene in render_cases().items():
        save_case(name, scene)
        print("wrote", name)
    with open(os.path.join(HERE, "occlusion_sessions.json"), "w") as f:
        json.dump(occlusion_sessions(), f, indent=1)
    print("wrote occlusion_sessions")
    with open(os.path.join(HERE, "texture_resize.json"), "w") as f:
        json.dump(texture_resizes(), f, indent=1)
    print("wrote texture_resize")
    with open(os.path.join(HERE, "dense_render.json"), "w") as f:
        json.dump(dense_renders(), f, indent=1)
    print("wrote dense_render")


if __name__ == "__main__":
    main()
