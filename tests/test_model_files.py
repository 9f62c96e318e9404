"""Model ingest in the reference's file formats, on the CPU: the writer and
reader round-trip every synthetic generator exactly, and -- where the
reference checkout is mounted (it is read, never copied) -- its own model
files parse to the row layouts the library assumes (gr.cu:31-35,
go.cu:33-38, pkj.cu:35-40, io.cu:28-33), its Pkj_GJ.csv is the pair table
the library carries, and the oracle integrates each of its cells."""
import os

import numpy as np
import pytest

import refsrc

import connectivity as CN
import morph as M

REF = refsrc.reference_dir() or ""
needs_ref = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "Gr.txt")), reason="reference checkout not mounted")
FILES = {"Gr.txt": (M.GR, 578), "Go_131.txt": (M.GO, 131), "Go_5.txt": (M.GO, 5), "Pkj.txt": (M.PKJ, 1600),
         "IO.txt": (M.IO, 3)}


@pytest.mark.parametrize("t, gen", [(M.GR, lambda: M.gr_synthetic(11)), (M.GR, M.gr_reduced4),
                                    (M.GO, lambda: M.go_synthetic(3)), (M.PKJ, lambda: M.pkj_synthetic(4)),
                                    (M.IO, M.io_rows)])
def test_write_parse_round_trip(t, gen):
    rows = gen()
    np.testing.assert_array_equal(M.parse_rows(M.write_rows(rows, t), t), rows)


@needs_ref
@pytest.mark.parametrize("name", sorted(FILES))
def test_reference_model_files(name):
    t, n = FILES[name]
    rows = M.parse_rows(open(os.path.join(REF, name)).read(), t)
    assert rows.shape == (n, M.ROW_FIELDS[t])
    np.testing.assert_array_equal(rows[:, 0], np.arange(n))          # row index = compartment
    parent = rows[:, 1]
    assert np.all((parent >= -1) & (parent < n) & (parent != np.arange(n)))


@needs_ref
def test_reference_gap_and_location_tables():
    gj = np.loadtxt(os.path.join(REF, "Pkj_GJ.csv"), delimiter=",", dtype=np.int32)
    np.testing.assert_array_equal(gj, M.PKJ_GJ_PAIRS)
    x, z, ty = CN.read_pkj_location(os.path.join(REF, "Pkj_location_info.csv"))
    assert x.size == z.size == ty.size == 1600 and np.all(np.isfinite(x))


@needs_ref
@pytest.mark.parametrize("name", ["Gr.txt", "Go_131.txt", "Pkj.txt", "IO.txt"])
def test_oracle_integrates_reference_cells(oracle, name):
    t, n = FILES[name]
    rows = M.parse_rows(open(os.path.join(REF, name)).read(), t)
    O = oracle
    O.libc_srand(0)
    s = O.System(t, 1, 1, rows, O.draw_jitter(t, 1), gj_pairs=M.PKJ_GJ_PAIRS if t == M.PKJ else None)
    assert s.init() == 0
    for k in range(2):
        assert s.advance(k * 0.125) == 0
    assert np.all(np.isfinite(s.vnew())) and s.vnew().size == n
