"""FreeFEM's text forms of a matrix (``f << A`` / ``f >> A``) and of a vector, through the
host-only C ABI entries (no device): files FreeFEM wrote are read back exactly, files written
here are read by FreeFEM itself (when it is installed) into the same matrix."""
import os
import subprocess

import numpy as np
import pytest

import ffgpu
from golden_cases import load

from paths import FF_BIN   # oracle/paths.py


def test_read_freefem_coo_text(tmp_path):
    d, _ = load("io_p1sq_n4")
    p = tmp_path / "A.txt"
    p.write_text(str(d["text_A_coo"]))
    n, m, half, rp, cl, vl = ffgpu.read_matrix_text(p)
    assert (n, m, half) == (25, 25, 0)
    I = np.repeat(np.arange(n), np.diff(rp))
    assert np.array_equal(I, d["I"]) and np.array_equal(cl, d["J"])
    assert np.array_equal(vl, d["C"])   # 20 significant digits: every double round-trips


def test_read_freefem_vector_text(tmp_path):
    d, _ = load("io_p1sq_n4")
    p = tmp_path / "b.txt"
    p.write_text(str(d["text_b"]))
    b = ffgpu.read_vector_text(p)
    assert b.size == 25
    assert np.abs(b - d["b"]).max() <= 1e-9 * np.abs(d["b"]).max()   # FreeFEM prints 10 digits


@pytest.mark.parametrize("fmt", ["coo", "morse"])
def test_matrix_text_round_trip(tmp_path, fmt):
    d, _ = load("io_p1sq_n4")
    rp = np.concatenate([[0], np.cumsum(np.bincount(d["I"], minlength=25))]).astype(np.int32)
    vals = d["C"].copy()
    vals[3] = 1e-310          # below 1e-305: Morse prints 0, as FreeFEM's removeeps
    vals[5] = -0.1 / 3
    p = tmp_path / f"A_{fmt}.txt"
    ffgpu.write_matrix_text(p, rp, d["J"], vals, format=fmt)
    n, m, half, rp2, cl2, vl2 = ffgpu.read_matrix_text(p)
    assert n == 25 and np.array_equal(rp2, rp) and np.array_equal(cl2, d["J"])
    want = vals.copy()
    if fmt == "morse":
        want[3] = 0.0
    assert np.array_equal(vl2, want)
    first = p.read_text().splitlines()[0]
    assert ("(Morse)" if fmt == "morse" else "(COO)") in first


def test_repeated_entries_keep_the_last_value(tmp_path):
    p = tmp_path / "dup.txt"
    p.write_text("#  HashMatrix Matrix (COO) 0\n#    n m nnz half fortran state\n"
                 "2 2 4 0 1 0 0\n 1 1 4.0\n 2 2 5.0\n 1 1 7.0\n 2 1 -1.0\n")
    n, m, half, rp, cl, vl = ffgpu.read_matrix_text(p)
    assert list(rp) == [0, 1, 3] and list(cl) == [0, 0, 1] and list(vl) == [7.0, -1.0, 5.0]


def test_vector_text_round_trip(tmp_path):
    v = np.random.default_rng(1).standard_normal(13)
    p = tmp_path / "v.txt"
    ffgpu.write_vector_text(p, v)
    assert np.array_equal(ffgpu.read_vector_text(p), v)


@pytest.mark.skipif(not os.path.exists(FF_BIN), reason="FreeFEM is not installed here")
@pytest.mark.parametrize("fmt", ["coo", "morse"])
def test_freefem_reads_files_written_here(tmp_path, fmt):
    d, _ = load("io_p1sq_n4")
    rp = np.concatenate([[0], np.cumsum(np.bincount(d["I"], minlength=25))]).astype(np.int32)
    ffgpu.write_matrix_text(tmp_path / "A.txt", rp, d["J"], d["C"], format=fmt)
    (tmp_path / "r.edp").write_text(
        'cout.precision(17);\nmatrix B;\n{ ifstream f("A.txt"); f >> B; }\n'
        '{ int[int] I(1),J(1); real[int] C(1); [I,J,C]=B;\n'
        '  for (int k=0;k<I.n;k++) cout << "A " << I[k] << " " << J[k] << " " << C[k] << endl; }\n')
    r = subprocess.run([FF_BIN, "-nw", "r.edp", "-v", "0"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    rows = [l.split()[1:] for l in r.stdout.splitlines() if l.startswith("A ")]
    I = np.array([int(x[0]) for x in rows]); J = np.array([int(x[1]) for x in rows])
    C = np.array([float(x[2]) for x in rows])
    assert np.array_equal(I, d["I"]) and np.array_equal(J, d["J"]) and np.array_equal(C, d["C"])
