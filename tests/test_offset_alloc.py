"""The server heap's bookkeeping on the CPU: tests/cpp/offset_alloc_test.cpp drives
painty_gb300/csrc/offset_alloc.h (the layout of the server's device reservation) through
200,000 random allocations and releases against a byte map: no overlaps, best fits, merged
free ranges, one free range of the full size at the end."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_offset_allocator_against_a_byte_map(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "offset_alloc_test"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
           f"-I{ROOT / 'painty_gb300' / 'csrc'}", str(ROOT / "tests" / "cpp" / "offset_alloc_test.cpp"),
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
