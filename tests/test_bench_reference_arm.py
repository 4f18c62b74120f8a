"""bench.py's reference arm runs the oracle's CPU restatement only: it never imports the
painty_gb300 package or maps its CUDA library, and it reports the headline line's config."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

PROBE = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"]
sys.path.insert(0, ROOT)
import bench
bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"package": "painty_gb300" in sys.modules,
                  "library": "libpainty_gb300" in maps,
                  "config": bench._headline_config(1)}))
"""


def test_reference_arm_does_not_load_the_library():
    r = subprocess.run([sys.executable, "-c", f"ROOT = {str(ROOT)!r}\n" + PROBE],
                       capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    ref, probe = lines[0], lines[-1]
    assert ref["impl"] == "reference"
    assert not probe["package"] and not probe["library"]
    assert ref["config"] == probe["config"]
    assert ref["e2e"]["h2d_bytes_per_step"] == 0 and ref["value"] > 0
