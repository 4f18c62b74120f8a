"""Regenerates the golden fixtures in this folder (run here, where the reference checkout is).

    python tests/golden/make_golden.py

kat.json       known-answer values written in the reference's own unit tests, with the file and
               line each comes from (painty/core/test/src/*.cxx, painty/image/test/src/MatTest.cxx).
stamps_ref.npz canvas and pickup-map planes after imprint sequences run by painty's own
               FootprintBrush / Canvas / Renderer headers, compiled unmodified against the
               repository's Eigen/OpenCV stand-ins (oracle/_ref). The GPU tests compare the
               library's F64 mode against these bit for bit; the GPU machine has no reference
               checkout, so the fixtures travel with the tests.
texture_ref.npz canvas planes after texture-brush stroke sessions (TextureBrush + Smudge) run
               by painty's own TextureBrush.hxx through the same harness.
render_ref.npz  Renderer::render (the lit canvas) of random canvases and of a painted one, by
               painty's own Renderer.hxx through the same harness.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.oracle import REFERENCE_ROOT, Reference  # noqa: E402
from painty_gb300 import workloads  # noqa: E402


def _num(s: str) -> float:
    return float(s)


def kat() -> dict:
    core = REFERENCE_ROOT / "painty/core/test/src"
    km = (core / "KubelkaMunkTest.cxx").read_text()
    math = (core / "MathTest.cxx").read_text()
    spl = (core / "SplineTest.cxx").read_text()
    mat = (REFERENCE_ROOT / "painty/image/test/src/MatTest.cxx").read_text()
    vec = lambda name, text: [float(x) for x in re.search(
        name + r"\s*=\s*\{([^}]*)\}", text).group(1).split(",")]
    near = re.findall(r"EXPECT_NEAR\(r1\[(\d)\],\s*([0-9.eE+-]+)", km)
    out = {
        "reflectance": {
            "source": "painty/core/test/src/KubelkaMunkTest.cxx:14-31",
            "d": 0.5, "K": vec(r"k", km), "S": vec(r"s", km), "R0": vec(r"r0", km),
            "expected": [float(v) for _, v in sorted(near)],
            "tolerance": 1e-5,
            "s_zero_channel0": float(re.search(r"s2, r0, d\)\[0\],\s*([0-9.]+)", km).group(1)),
        },
        "coth": {
            "source": "painty/core/test/src/MathTest.cxx:83-91",
            "cases": [[float(a), float(b)] for a, b in
                      re.findall(r"EXPECT_NEAR\(painty::coth\(([0-9.]+)\),\s*([0-9.]+)", math)],
            "tolerance": 1e-5,
        },
        "catmull_rom": {
            "source": "painty/core/test/src/SplineTest.cxx:26",
            "args": [float(x) for x in re.search(
                r"EXPECT_NEAR\(([0-9.]+), painty::CatmullRom\(([^)]*)\)", spl).group(2).split(",")],
            "expected": float(re.search(r"EXPECT_NEAR\(([0-9.]+), painty::CatmullRom\(", spl).group(1)),
            "tolerance": 1e-7,
        },
        "spline_eval": {
            "source": "painty/core/test/src/SplineTest.cxx:36-41",
            "points": [[float(a), float(b)] for a, b in re.findall(r"\{([0-9.]+), ([0-9.]+)\}",
                                                                  spl.split("points =")[1])],
            "u": 0.2,
            "expected": [float(x) for x in re.findall(
                r"EXPECT_NEAR\(([0-9.]+), spline\.catmullRom", spl)],
            "tolerance": 1e-7,
        },
        "bilinear": {
            "source": "painty/image/test/src/MatTest.cxx:42-55",
            "image_channel0": [[1.5, 1.5], [2.5, 2.5]],
            "position": [0.5, 0.5],
            "expected": 2.0,
            "tolerance": 1e-7,
        },
    }
    assert len(out["reflectance"]["expected"]) == 3
    assert len(out["coth"]["cases"]) == 4
    assert len(out["spline_eval"]["expected"]) == 2
    return out


def stamps_fixture() -> dict:
    ref = Reference()
    fp = workloads.footprint_image(seed=7)
    rng = np.random.default_rng(2024)
    arrays = {"footprint_full": fp}
    cases = [
        # name, rows, cols, snapshot, pickup rate, deposit rate, strokes
        ("snap_small", 37, 53, True, 0.05, 0.1, 5),
        ("nosnap_small", 29, 41, False, 0.9, 0.05, 4),
        ("snap_default_rates", 48, 48, True, 0.9, 0.05, 4),
    ]
    for name, rows, cols, snap, pr, dr, nstrokes in cases:
        c = ref.canvas(rows, cols)
        r0 = rng.uniform(0.8, 0.95, (rows, cols, 3))
        c.set("R0", r0)
        b = ref.brush(3.0, fp)
        b.set_rates(pr, dr)
        b.set_snapshot(snap)
        script = []
        for s in range(nstrokes):
            rad = float(rng.uniform(1.0, 9.0))
            K = rng.uniform(0.01, 5, 3)
            S = rng.uniform(0.05, 3, 3)
            b.set_radius(rad)
            b.dip(K, S)
            n = int(rng.integers(3, 12))
            st = np.stack([rng.uniform(-6, cols + 6, n), rng.uniform(-6, rows + 6, n),
                           rng.uniform(-np.pi, np.pi, n)], axis=1)
            st[0, :2] = [0.5, 0.25]  # an edge stamp: duplicated canvas column and row
            b.stamps(c, st)
            script.append((rad, K, S, st))
        arrays[f"{name}/r0"] = r0
        arrays[f"{name}/meta"] = np.array([rows, cols, int(snap), pr, dr], dtype=np.float64)
        for i, (rad, K, S, st) in enumerate(script):
            arrays[f"{name}/stroke{i}/radius"] = np.array([rad])
            arrays[f"{name}/stroke{i}/paint"] = np.stack([K, S])
            arrays[f"{name}/stroke{i}/stamps"] = st
        for p in ("K", "S", "V"):
            arrays[f"{name}/out_{p}"] = c.get(p)
        arrays[f"{name}/out_compose"] = c.compose()
        for p in ("K", "S", "V"):
            arrays[f"{name}/pickup_{p}"] = b.pickup(p)
        c.dry()
        arrays[f"{name}/dry_R0"] = c.get("R0")
        arrays[f"{name}/dry_h"] = c.get("h")
    # a spline stroke with the reference's 1-pixel chord stepping
    c = ref.canvas(40, 60)
    c.set("R0", np.full((40, 60, 3), 0.9))
    b = ref.brush(4.0, fp)
    b.set_rates(0.05, 0.1)
    b.dip(np.array([0.3, 1.2, 2.0]), np.array([0.5, 0.4, 0.9]))
    path = np.array([[5.0, 5.0], [30.0, 12.5], [52.0, 30.0], [20.0, 33.0]])
    n = b.paint_stroke(c, path)
    arrays["stroke/path"] = path
    arrays["stroke/count"] = np.array([n])
    for p in ("K", "S", "V"):
        arrays[f"stroke/out_{p}"] = c.get(p)
    return arrays


def texture_session(rng, rows, cols, n, rmin=4.0, rmax=18.0):
    """n random strokes (2-5 control points, partly off the canvas) with radius and paint."""
    out = []
    for _ in range(n):
        k = int(rng.integers(2, 6))
        path = np.stack([rng.uniform(-10, cols + 10, k), rng.uniform(-10, rows + 10, k)], axis=1)
        out.append((path, float(rng.uniform(rmin, rmax)), rng.uniform(0.01, 5, 3),
                    rng.uniform(0.05, 3, 3)))
    return out


def texture_fixture() -> dict:
    ref = Reference()
    arrays = {}
    cases = [
        # name, rows, cols, smudge, thickness scale, texture seed, strokes
        ("smudge", 48, 64, True, 1.0, 13, 5),
        ("nosmudge", 40, 56, False, 1.5, 5, 4),
    ]
    rng = np.random.default_rng(77)
    for name, rows, cols, smudge, scale, tseed, nstrokes in cases:
        tex = workloads.stroke_texture(seed=tseed)
        sess = texture_session(rng, rows, cols, nstrokes)
        r0 = rng.uniform(0.8, 0.95, (rows, cols, 3))
        c = ref.canvas(rows, cols)
        c.set("R0", r0)
        b = ref.texture_brush(tex)
        b.enable_smudge(smudge)
        b.set_thickness_scale(scale)
        for i, (path, rad, K, S) in enumerate(sess):
            b.set_radius(rad)
            b.dip(K, S)
            b.paint_stroke(c, path)
            arrays[f"{name}/stroke{i}/path"] = path
            arrays[f"{name}/stroke{i}/radius"] = np.array([rad])
            arrays[f"{name}/stroke{i}/paint"] = np.stack([K, S])
        arrays[f"{name}/meta"] = np.array([rows, cols, int(smudge), scale, tseed], dtype=np.float64)
        arrays[f"{name}/r0"] = r0
        for p in ("K", "S", "V"):
            arrays[f"{name}/out_{p}"] = c.get(p)
    return arrays


def render_fixture() -> dict:
    ref = Reference()
    rng = np.random.default_rng(404)
    arrays = {}
    for name, (rows, cols) in (("random_a", (24, 40)), ("random_b", (37, 29))):
        c = ref.canvas(rows, cols)
        planes = {"R0": rng.uniform(0.8, 0.95, (rows, cols, 3)),
                  "K": rng.uniform(0.01, 5, (rows, cols, 3)),
                  "S": rng.uniform(0.05, 3, (rows, cols, 3)),
                  "V": rng.uniform(0, 1, (rows, cols)) * (rng.random((rows, cols)) < 0.6)}
        for p, a in planes.items():
            c.set(p, a)
            arrays[f"{name}/{p}"] = a
        arrays[f"{name}/out"] = c.render()
    # a canvas painted by the imprint brush (smooth volume: the normals see brush ridges)
    c = ref.canvas(40, 60)
    c.set("R0", np.full((40, 60, 3), 0.9))
    b = ref.brush(6.0, workloads.footprint_image(seed=7))
    b.set_rates(0.05, 0.1)
    b.dip(np.array([0.3, 1.2, 2.0]), np.array([0.5, 0.4, 0.9]))
    b.paint_stroke(c, np.array([[5.0, 5.0], [30.0, 12.5], [52.0, 30.0], [20.0, 33.0]]))
    for p in ("R0", "K", "S", "V"):
        arrays[f"painted/{p}"] = c.get(p)
    arrays["painted/out"] = c.render()
    return arrays


def main() -> None:
    if not Reference.available():
        raise SystemExit("reference checkout / oracle/_ref build not available")
    (HERE / "kat.json").write_text(json.dumps(kat(), indent=1) + "\n")
    np.savez_compressed(HERE / "stamps_ref.npz", **stamps_fixture())
    np.savez_compressed(HERE / "texture_ref.npz", **texture_fixture())
    np.savez_compressed(HERE / "render_ref.npz", **render_fixture())
    print("wrote kat.json, stamps_ref.npz, texture_ref.npz, render_ref.npz")


if __name__ == "__main__":
    main()
