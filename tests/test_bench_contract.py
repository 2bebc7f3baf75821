"""CPU: the bench's reference arm prints one JSON line with the contract's keys
(it times the FP64 CPU path, so it runs without a GPU), and the launch-shape
option parses as documented."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "asm",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    o = json.loads(lines[0])
    assert o["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "config", "cpu_baseline",
              "e2e"):
        assert k in o, k
    assert o["value"] > 0 and o["unit"] == o["e2e"]["unit"] == o["cpu_baseline"]["unit"]
    assert o["e2e"]["h2d_bytes_per_step"] == 0 and o["e2e"]["d2h_bytes_per_step"] == 0
    assert o["cpu_baseline"]["kind"] in ("port", "reference") and o["cpu_baseline"]["cores"] >= 1


class _FakeOg:
    def __init__(self):
        self.calls = []

    def set_variant(self, kind, n, idx):
        self.calls.append((kind, n, idx))


def test_pinned_variants_parser():
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.pop(0)
    og = _FakeOg()
    tuned = bench.pinned_variants(og, {(0, 2048): 4}, "0:2048=1,1:2048=11,2:2048=3")
    assert og.calls == [(0, 2048, 1), (1, 2048, 11), (2, 2048, 3)]
    assert tuned == {(0, 2048): 1, (1, 2048): 11, (2, 2048): 3}
    assert bench.pinned_variants(og, {(1, 4096): 2}, "") == {(1, 4096): 2}
    with pytest.raises(ValueError):
        bench.pinned_variants(og, {}, "0:2048")
