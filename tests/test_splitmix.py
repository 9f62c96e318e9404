"""The counter-based draws (csrc/splitmix.h, its Python restatement in
connectivity.py, and the oracle's copy) on the CPU: the SplitMix64 finaliser
of Steele, Lea & Flood (2014) against its published first output for seed 0,
and the C++ header against the Python restatement bit for bit."""
import os
import shutil
import subprocess

import pytest

import connectivity as CN

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300", "csrc", "splitmix.h")
CASES = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (12345, 678, 9), ((1 << 64) - 1, 2 ** 40 + 3, 77),
         (2147483647, 1599, 123456), (42, 780403, 8000)]


def test_published_first_output():
    # SplitMix64 seeded with 0 gives 0xE220A8397B1DCDAF first; the draw is its top 53 bits, + 1, / 2^53
    assert CN.splitmix_uniform(0, 0, 0) == float((0xE220A8397B1DCDAF >> 11) + 1) * 2.0 ** -53


def test_draws_lie_in_unit_interval():
    for s, i, c in CASES:
        u = CN.splitmix_uniform(s, i, c)
        assert 0.0 < u <= 1.0


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_header_matches_python(tmp_path):
    src = tmp_path / "sm.cpp"
    calls = "\n".join(f'  std::printf("%a\\n", gbrkc::splitmix_uniform({s}ull, {i}ll, {c}ll));' for s, i, c in CASES)
    src.write_text(f'#include <cstdio>\n#include "{HDR}"\nint main() {{\n{calls}\n  return 0;\n}}\n')
    exe = tmp_path / "sm"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert [float.fromhex(x) for x in out] == [CN.splitmix_uniform(s, i, c) for s, i, c in CASES]
