"""The drop-in's coupling-object constructors and synapse raster writers on
the CPU (they make no device call before network mode starts): the files
syn.cu's constructors open, the rows mf_output_file / mli_output_file write
(all values 0 without network mode), and rand() drawn only by non-empty
random families, as the reference's constructors draw their cuRAND seeds."""
import ctypes as C
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cerebellum-neuron-model-simulation-using-rkc_gb300")
LIB = os.path.join(PKG, "libgbrkc.so")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import build as B
        B.build()
    L = C.CDLL(LIB)
    P = C.c_void_p
    L.mfgr_create.restype = P
    L.mfgr_create.argtypes = [C.c_int]
    L.mlipkj_create.restype = P
    L.mlipkj_create.argtypes = [C.c_int, C.c_int]
    L.grpkj_create.restype = P
    L.grpkj_create.argtypes = [C.c_int] * 4
    for f in ("mfgr_finalize", "mlipkj_finalize", "grpkj_finalize"):
        getattr(L, f).argtypes = [P, C.c_int]
    for f in ("mf_output_file", "mli_output_file"):
        getattr(L, f).argtypes = [P, C.c_double, P]
    return L


def test_raster_files_and_rows(lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    mf = lib.mfgr_create(3)                      # 3 granule cells: 12 fibres
    mli = lib.mlipkj_create(2, 3)                # 2 Purkinje cells: 2 MLI synapses
    assert (tmp_path / "MF_RASTER.csv").exists() and (tmp_path / "MLI_RASTER.csv").exists()
    for t in (0.125, 0.25):
        lib.mf_output_file(mf, t, None)
        lib.mli_output_file(mli, t, None)
    lib.mfgr_finalize(mf, 3)
    lib.mlipkj_finalize(mli, 6)
    mf_rows = (tmp_path / "MF_RASTER.csv").read_text().splitlines()
    assert mf_rows == ["0.125000," + "0.000000," * 12, "0.250000," + "0.000000," * 12]
    mli_rows = (tmp_path / "MLI_RASTER.csv").read_text().splitlines()
    assert mli_rows == ["0.125000," + "0.000000," * 2, "0.250000," + "0.000000," * 2]


def test_empty_families_open_no_file(lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    mf = lib.mfgr_create(0)
    mli = lib.mlipkj_create(4, 0)                # no granule cells: no MLI synapses
    lib.mf_output_file(mf, 0.125, None)          # nothing to write to
    lib.mfgr_finalize(mf, 0)
    lib.mlipkj_finalize(mli, 0)
    assert not (tmp_path / "MF_RASTER.csv").exists() and not (tmp_path / "MLI_RASTER.csv").exists()


def test_rand_drawn_by_non_empty_random_families(lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    libc = C.CDLL(None)
    libc.srand(7)
    seq = [libc.rand() for _ in range(5)]
    libc.srand(7)
    objs = [(lib.mfgr_create(0), lib.mfgr_finalize), (lib.grpkj_create(2, 2, 0, 0), lib.grpkj_finalize),
            (lib.mlipkj_create(0, 4), lib.mlipkj_finalize)]
    assert libc.rand() == seq[0]                 # empty families draw nothing
    objs += [(lib.mfgr_create(2), lib.mfgr_finalize), (lib.grpkj_create(2, 2, 1, 1), lib.grpkj_finalize),
             (lib.mlipkj_create(1, 4), lib.mlipkj_finalize)]
    assert libc.rand() == seq[4]                 # one draw each (syn.cu:82, 623, 755)
    for o, fin in objs:
        fin(o, 0)


def test_raster_plot(lib, tmp_path, monkeypatch, capfd):
    """output.cu's post-run Golgi raster: a row per interval, the index of
    each cell whose voltage crossed 0 mV upward, "," for the others."""
    monkeypatch.chdir(tmp_path)
    rows = [(0.125, -65.0, -60.0, 5.0), (0.25, 12.0, -1.0, 20.0), (0.375, -50.0, 3.0, -70.0),
            (0.5, 8.0, 4.0, 1.0)]
    (tmp_path / "go_v_by_RKC.csv").write_text("".join(",".join("%lf" % x for x in r) + ",\n" for r in rows))
    lib.raster_plot.argtypes = [C.c_int, C.c_char_p]
    lib.raster_plot(3, b"RKC")
    C.CDLL(None).fflush(None)
    assert capfd.readouterr().out == "Debug for output \n2,0,1,0,2,"
    got = (tmp_path / "go_raster_by_RKC.csv").read_text().splitlines()
    # cell 2 crosses in the first row (from -70 mV); 0 in the second; 1 in the third; 0 and 2 in the fourth
    assert got == ["0.125000,,,2,", "0.250000,0,,,", "0.375000,,1,,", "0.500000,0,,2,"]


def test_pkj_poisson_draws_one_rand_per_call(lib):
    """pkj_set_current_Poisson draws one rand() per call, as pkj.cu:364 does
    (no cells: nothing is launched)."""
    lib.pkj_set_current_Poisson.argtypes = [C.c_int, C.c_void_p, C.c_double]
    libc = C.CDLL(None)
    libc.srand(11)
    seq = [libc.rand() for _ in range(4)]
    libc.srand(11)
    for t in (0.0, 400.0, 400.125):
        lib.pkj_set_current_Poisson(0, None, t)
    assert libc.rand() == seq[3]
