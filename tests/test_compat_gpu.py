"""The reference-named drop-in path (include/gbrkc_compat.h) end to end,
through the gbrkc_main CLI: model files in the reference formats, the
reference's stimulus kernels, rand() jitter seeded as main.cu:38, and the
reference's CSV outputs."""
import os
import subprocess

import numpy as np
import pytest

import morph as M
from test_oracle_golden import load_gold

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300", "gbrkc_main")


def run_cli(tmp_path, dims, ts, files):
    for name, text in files.items():
        (tmp_path / name).write_text(text)
    args = [CLI]
    for nx, ny in dims:
        args += ["RKC", str(nx), str(ny)]
    args.append(str(ts))
    env = dict(os.environ, GBRKC_MODEL_DIR=str(tmp_path))
    r = subprocess.run(args, cwd=tmp_path, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def read_v(path):
    rows = []
    for line in open(path):
        vals = [float(x) for x in line.strip().rstrip(",").split(",") if x != ""]
        rows.append(vals)
    return np.array(rows)


def test_io_raster_matches_reference_golden(tmp_path):
    """io_raster_by_RKC.csv of the reference (8x8 IO, default stimulus)."""
    run_cli(tmp_path, [(0, 0), (0, 0), (0, 0), (8, 8)], 809.0, {"IO.txt": M.write_rows(M.io_rows(), M.IO)})
    mine = []
    for line in open(tmp_path / "io_raster_by_RKC.csv"):
        t, c = line.strip().split(",")
        mine.append((float(t), int(c)))
    gold = {c: t for t, c in load_gold()}
    assert sorted(c for _, c in mine) == list(range(64)), "every cell spikes exactly once"
    times = {c: t for t, c in mine}
    assert all(abs(times[c] - gold[c]) <= 0.125 for c in range(64))
    exact = sum(times[c] == gold[c] for c in range(64))
    assert exact >= 62, f"only {exact}/64 spike times identical"
    v = read_v(tmp_path / "io_v_by_RKC.csv")
    assert v.shape == (int(809.0 / 0.125), 1 + 3 * 64)
    assert (tmp_path / "comptime.csv").exists()


def test_go_pkj_blocks_match_oracle(tmp_path, oracle):
    """GoC 2x2 and PC 2x1 blocks (synthetic trees in the reference formats)
    against the oracle in canonical mode: every written soma voltage equal
    to the printed precision (%lf, 1e-6 mV)."""
    go_rows, pkj_rows = M.go_synthetic(3), M.pkj_synthetic(4)
    gj = "\n".join(f"{a},{b}" for a, b in M.PKJ_GJ_PAIRS) + "\n"
    ts = 3.0
    run_cli(tmp_path, [(0, 0), (2, 2), (2, 1), (0, 0)], ts,
            {"Go_131.txt": M.write_rows(go_rows, M.GO), "Pkj.txt": M.write_rows(pkj_rows, M.PKJ), "Pkj_GJ.csv": gj})
    O = oracle
    O.libc_srand(0)
    jit_go = O.draw_jitter(O.GO, 4)
    jit_pkj = O.draw_jitter(O.PKJ, 2)
    cases = [("go", O.System(O.GO, 2, 2, go_rows, jit_go, go_gj=True, canon=True), 30, 131),
             ("pkj", O.System(O.PKJ, 2, 1, pkj_rows, jit_pkj, gj_pairs=M.PKJ_GJ_PAIRS, pkj_gj=True, canon=True),
              1599, 1600)]
    for name, s, soma, ncomp in cases:
        assert s.init() == 0
        v = read_v(tmp_path / f"{name}_v_by_RKC.csv")
        t = 0.0
        for k in range(int(ts / 0.125)):
            assert s.advance(t) == 0
            t += 0.125
            ref = s.vnew()[soma::ncomp]
            assert v[k, 0] == pytest.approx(t, abs=1e-9)
            np.testing.assert_allclose(v[k, 1:], ref, atol=1.5e-6, rtol=0, err_msg=f"{name} interval {k}")


def test_reference_script_solver_names(tmp_path):
    """The reference's run scripts name CN or BE for the types they leave
    empty (`./main CN 0 0 RKC 1 1 CN 0 0 CN 0 0`): accepted, their files are
    opened under those names and stay empty, and the RKC block writes the
    same bytes as with RKC everywhere."""
    files = {"Go_131.txt": M.write_rows(M.go_synthetic(3), M.GO)}
    out = {}
    for tag, names in (("mixed", ("CN", "RKC", "CN", "BE")), ("rkc", ("RKC",) * 4)):
        d = tmp_path / tag
        d.mkdir()
        for name, text in files.items():
            (d / name).write_text(text)
        args = [CLI]
        for s, (nx, ny) in zip(names, [(0, 0), (1, 1), (0, 0), (0, 0)]):
            args += [s, str(nx), str(ny)]
        args.append("2.0")
        r = subprocess.run(args, cwd=d, env=dict(os.environ, GBRKC_MODEL_DIR=str(d)), capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[tag] = (d / "go_v_by_RKC.csv").read_bytes()
        if tag == "mixed":
            for f in ("gr_v_by_CN.csv", "pkj_raster_by_CN.csv", "io_v_by_BE.csv"):
                assert (d / f).exists() and (d / f).stat().st_size == 0, f
    assert out["mixed"] == out["rkc"] and out["rkc"].count(b"\n") == 16


def test_batched_cli_writes_identical_files(tmp_path):
    """gbrkc_main with batch > 1 (several intervals per launch, voltage
    record and raster on the device, CSV from a writer thread) writes the
    same bytes as the per-interval path, for every type."""
    files = {"Gr.txt": M.write_rows(M.gr_synthetic(11), M.GR), "Go_131.txt": M.write_rows(M.go_synthetic(3), M.GO),
             "Pkj.txt": M.write_rows(M.pkj_synthetic(4), M.PKJ),
             "Pkj_GJ.csv": "\n".join(f"{a},{b}" for a, b in M.PKJ_GJ_PAIRS) + "\n",
             "IO.txt": M.write_rows(M.io_rows(), M.IO)}
    dims = [(2, 1), (1, 1), (1, 1), (4, 4)]
    out = {}
    for batch in (1, 70):
        d = tmp_path / f"b{batch}"
        d.mkdir()
        for name, text in files.items():
            (d / name).write_text(text)
        args = [CLI]
        for nx, ny in dims:
            args += ["RKC", str(nx), str(ny)]
        args += ["60", str(batch)]
        r = subprocess.run(args, cwd=d, env=dict(os.environ, GBRKC_MODEL_DIR=str(d)), capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[batch] = {f: (d / f).read_bytes() for f in sorted(os.listdir(d)) if f.endswith("_by_RKC.csv")}
    assert sorted(out[1]) == sorted(out[70]) and len(out[1]) == 8
    for f in out[1]:
        assert out[1][f] == out[70][f], f
    assert out[1]["gr_v_by_RKC.csv"].count(b"\n") == 480


def test_network_mode_dropin_matches_native(tmp_path, oracle):
    """gbrkc_main with main.cu's network branch (coupling objects, synapse
    updates after every interval) against the native ABI wired by the same
    rules (connectivity.py, SplitMix target draws, rand() seeds in the
    constructors' order): every written soma voltage identical."""
    import ctypes
    import connectivity as CN
    import gbrkc as G
    O = oracle
    gr, go, pk = M.gr_synthetic(11), M.go_synthetic(3), M.pkj_synthetic(4)
    px = np.random.default_rng(8).uniform(-150, 150, 1600)
    loc = "".join(f"{i},{x:.6f},0.0,0.0,3\n" for i, x in enumerate(px))
    gj = "\n".join(f"{a},{b}" for a, b in M.PKJ_GJ_PAIRS) + "\n"
    files = {"Gr.txt": M.write_rows(gr, M.GR), "Go_131.txt": M.write_rows(go, M.GO),
             "Pkj.txt": M.write_rows(pk, M.PKJ), "Pkj_GJ.csv": gj, "Pkj_location_info.csv": loc}
    for name, text in files.items():
        (tmp_path / name).write_text(text)
    ts, n_iv = 2.0, 16
    args = [CLI, "RKC", "2", "2", "RKC", "1", "1", "RKC", "1", "1", "RKC", "0", "0", str(ts), "1", "1"]
    r = subprocess.run(args, cwd=tmp_path, env=dict(os.environ, GBRKC_MODEL_DIR=str(tmp_path)), capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    # the constructors open the synapse rasters (syn.cu:76, 726); main.cu writes no rows to them
    assert (tmp_path / "MF_RASTER.csv").read_text() == "" and (tmp_path / "MLI_RASTER.csv").read_text() == ""
    # the same run through the native ABI
    O.libc_srand(0)
    jit = {t: O.draw_jitter(t, n) for t, n in ((M.GR, 4), (M.GO, 1), (M.PKJ, 1))}
    libc = ctypes.CDLL(None)
    seed_mf = libc.rand()        # mfgr_create
    seed_pk = libc.rand()        # grpkj_create
    rows = [gr, go, pk]
    nc = [r_.shape[0] for r_ in rows]
    eng = G.Engine(G.FP64)
    sid = [eng.add_system(M.GR, 2, 2, gr, jit[M.GR]), eng.add_system(M.GO, 1, 1, go, jit[M.GO]),
           eng.add_system(M.PKJ, 1, 1, pk, jit[M.PKJ], gj_pairs=M.PKJ_GJ_PAIRS)]
    g = CN.reference_synapses(2, 2, 1, 1, 1, 1, px, uniform=lambda k: CN.splitmix_uniform(seed_pk, k))
    for kind, seed in ((CN.SYN_MFGR, seed_mf), (CN.SYN_GRGO, 0), (CN.SYN_GOGR, 0), (CN.SYN_GRPKJ, 0)):
        one = {k: (g[k] if k == kind else dict(post_cell=[])) for k in g}
        CN.add_reference_network(eng, one, lambda ty, c: (sid[ty], c * nc[ty]), seed=seed)
    eng.build()
    soma = {M.GR: 16, M.GO: 30, M.PKJ: 1599}
    got = {name: (tmp_path / f"{name}_v_by_RKC.csv").read_text().splitlines() for name in ("gr", "go", "pkj")}
    t = 0.0
    for k in range(n_iv):
        eng.advance(t, 1)
        t += 0.125
        for name, ty, s in (("gr", M.GR, sid[0]), ("go", M.GO, sid[1]), ("pkj", M.PKJ, sid[2])):
            v = eng.vnew(s)
            n = v.size // nc[ty]
            line = "%f," % t + "".join("%f," % v[soma[ty] + j * nc[ty]] for j in range(n))
            assert got[name][k] == line, (name, k)
    syn = eng.read_synapses(G.SYNF_S0, sum(len(g[k]["post_cell"]) for k in g))
    assert syn[:16].max() >= 0.0
    eng.close()
