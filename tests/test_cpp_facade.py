"""The C++ facade (include/painty_gb300.hpp): compiles against the C ABI, translates statuses
into painty's exception types, and paints the same result as the Python binding."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from painty_gb300 import workloads

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "painty_gb300" / "_lib"


def _cuda_lib():
    for c in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if Path(c, "libcudart.so").exists():
            return c
    return "/usr/local/cuda/lib64"


@pytest.fixture(scope="module")
def demo(tmp_path_factory, pg):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("cpp") / "facade_demo"
    cmd = ["g++", "-std=c++17", "-O1", "-pthread", "-Wall", "-Werror", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "facade_demo.cpp"), "-o", str(exe), f"-L{LIB}",
           "-lpainty_gb300", f"-Wl,-rpath,{LIB}", f"-Wl,-rpath,{_cuda_lib()}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_facade_translates_argument_errors(demo):
    r = subprocess.run([str(demo), "errors"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "errors ok" in r.stdout


def test_facade_palette_round_trip(demo, tmp_path):
    """LoadPalette / SavePalette in C++ read painty's palette format and write what the Python
    side writes (nlohmann's compact form)."""
    from painty_gb300 import palette as P
    rng = np.random.default_rng(3)
    pal = [(rng.uniform(0, 5, 3), rng.uniform(0, 3, 3)) for _ in range(6)]
    pal.append((np.array([0.0, 0.5, 1.0]), np.array([1e-05, 0.003, 123.25])))
    src = tmp_path / "in.json"
    # painty's files are indented; the reader must not care
    import json
    src.write_text(json.dumps([{"K": list(K), "S": list(S)} for K, S in pal], indent=2))
    dst = tmp_path / "out.json"
    r = subprocess.run([str(demo), "palette", str(src), str(dst)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert dst.read_text() == P.dumps_palette(pal)
    back = P.load_palette(dst)
    for (K, S), (K2, S2) in zip(pal, back):
        assert np.array_equal(K, K2) and np.array_equal(S, S2)


@pytest.mark.gpu
def test_facade_sbr_render_thread(demo):
    """SbrRenderThread's futures, on its worker thread, paint what direct calls paint."""
    r = subprocess.run([str(demo), "sbr"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "sbr ok" in r.stdout


@pytest.mark.gpu
def test_facade_paints_like_python_binding(demo, pg, tmp_path):
    rows, cols = 70, 90
    fp = workloads.footprint_image(seed=7)
    s = workloads.strokes(cols, rows, 1, seed=29, rmin=5, rmax=12)[0]
    r0 = workloads.substrate(rows, cols, seed=5)
    buf = np.concatenate([[rows, cols, fp.shape[0], fp.shape[1]], fp.ravel(), [len(s.path)],
                          s.path.ravel(), [s.radius, s.spacing, 0.05, 0.1], s.K, s.S, r0.ravel()])
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    buf.astype(np.float64).tofile(inp)
    r = subprocess.run([str(demo), "paint", str(inp), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out, dtype=np.float64)
    c = pg.Canvas(rows, cols, "f64")
    c.setBackground(r0)
    b = pg.FootprintBrush(s.radius, fp)
    b.setPickupRate(0.05)
    b.setDepositionRate(0.1)
    b.dip((s.K, s.S))
    n = b.paintStroke(s.path, c, spacing=s.spacing)
    want = [np.array([n], dtype=np.float64), c.download("K").ravel(), c.download("S").ravel(),
            c.download("V").ravel(), pg.Renderer().compose(c).download().ravel()]
    assert np.array_equal(got, np.concatenate(want))


@pytest.mark.gpu
def test_facade_texture_brush_and_render(demo, pg, tmp_path):
    """TextureBrush and Renderer::render through the C++ facade equal the Python binding."""
    rows, cols = 60, 80
    tex = workloads.stroke_texture(seed=13)
    path = np.array([[5.0, 10.0], [40.0, 30.0], [75.0, 22.0]])
    K, S = np.array([0.4, 1.1, 2.2]), np.array([0.6, 0.3, 0.2])
    buf = np.concatenate([[rows, cols, tex.shape[0], tex.shape[1]], tex.ravel(), [len(path)],
                          path.ravel(), [9.0], K, S])
    inp, out = tmp_path / "tin.bin", tmp_path / "tout.bin"
    buf.astype(np.float64).tofile(inp)
    r = subprocess.run([str(demo), "texture", str(inp), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out, dtype=np.float64)
    c = pg.Canvas(rows, cols, "f64")
    c.setBackground(np.full((rows, cols, 3), 0.9))
    b = pg.TextureBrush(tex)
    b.setRadius(9.0)
    b.dip((K, S))
    n = b.paintStroke(path, c)
    npx = rows * cols
    assert got[0] == n and n > 0
    o = 1
    for p, nch in (("K", 3), ("S", 3), ("V", 1)):
        want = c.download(p).ravel()
        assert np.array_equal(got[o:o + npx * nch], want), p
        o += npx * nch
    assert np.array_equal(got[o:o + npx * 3], pg.Renderer().render(c).download().ravel())


def test_facade_reads_painty_palettes_as_painty_does(demo, tmp_path):
    """The facade's LoadPalette on painty's own palette files gives painty's own LoadPalette's
    values (Serialization.cxx:38-44 compiled in the oracle's reference build), bit for bit."""
    from oracle.oracle import Reference
    from painty_gb300 import palette as P
    root = Path(os.environ.get("PAINTY_REFERENCE_ROOT", "/root/reference")) / "data" / "paint_palettes"
    if not root.is_dir() or not Reference.available():
        pytest.skip("reference checkout not present")
    ref = Reference()
    for src in sorted(root.glob("*.json")):
        dst = tmp_path / src.name
        r = subprocess.run([str(demo), "palette", str(src), str(dst)], capture_output=True,
                           text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        ours, theirs = P.load_palette(dst), ref.load_palette(src.read_text())
        assert len(ours) == len(theirs) > 0
        for (K, S), (K2, S2) in zip(ours, theirs):
            assert np.array_equal(K, K2) and np.array_equal(S, S2), src.name
