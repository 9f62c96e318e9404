"""The C-ABI library loads and exports every function include/*.h declares
(no device calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
LIB = os.path.join(PKG, "libgbrkc.so")

DECL = re.compile(r"^(?:__global__\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"__attribute__\(\(\w+(?:\(\"\w+\"\))?\)\)\s*", "", text)
    names = set()
    for m in DECL.finditer(text):
        line = text[m.start():text.find("\n", m.start())]
        if line.lstrip().startswith(("#", "typedef", "return", "static")):
            continue
        names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import build as B
        B.build()
    return ctypes.CDLL(LIB)


@pytest.mark.parametrize("header", ["gbrkc.h", "gbrkc_compat.h"])
def test_every_declared_symbol_is_exported(lib, header):
    names = declared(header)
    assert len(names) > 10, names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, f"{header}: not exported: {missing}"


def header_kernels(header):
    """Kernels the header defines itself (compiled into each caller's module)."""
    return set(re.findall(r"^static __global__ void (\w+)\(", open(os.path.join(INCLUDE, header)).read(), re.M))


def test_reference_entry_points_present():
    names = declared("gbrkc_compat.h") | header_kernels("gbrkc_compat.h")
    for t in ("gr", "go", "pkj", "io"):
        for f in ("initialize", "solve_initialize", "solve_update_v", "set_current", "output_file", "finalize",
                  "solve_finalize"):
            assert f"{t}_{f}" in names


@pytest.mark.parametrize("header", ["gbrkc.h", "gbrkc_compat.h"])
@pytest.mark.parametrize("lang", [("gcc", "c", "-std=c99"), ("g++", "c++", "-std=c++17")])
def test_header_compiles_alone(tmp_path, header, lang):
    """Each public header is self-contained C99 and C++17 (a caller may be either)."""
    import shutil
    import subprocess
    cc, x, std = lang
    if shutil.which(cc) is None:
        pytest.skip(f"no {cc}")
    src = tmp_path / "h.c"
    src.write_text(f'#include "{header}"\n')
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", x, f"-I{INCLUDE}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
