"""Host ingest (no GPU): the Matrix Market reader against the reference's
own read_matrix_market_to_csr output (tests/golden/mtx.npz, made by
tests/golden/make_golden.py from the reference source), the header kinds the
reference ignores (symmetric, skew-symmetric, pattern, integer), error
reporting, and the binary BSR format (round trip, checksum, structure)."""
import os

import numpy as np
import pytest

from conftest import golden
from isai_kernel_gb300 import api, gen
from isai_kernel_gb300._lib import BiluError


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_general_file_matches_reference_reader(tmp_path):
    d = golden("mtx")
    path = _write(tmp_path, "a.mtx", bytes(d["text"]).decode())
    m, n, row, col, val = api.read_matrix_market_to_csr(path)
    assert (m, n) == (int(d["nrows"]), int(d["ncols"]))
    assert np.array_equal(row, d["row"]) and np.array_equal(col, d["col"])
    assert np.array_equal(val, d["val"])


def test_symmetric_skew_pattern_integer(tmp_path):
    body = "3 3 4\n1 1 2.0\n2 1 -1.5\n3 2 0.25\n3 3 4\n"
    sym = _write(tmp_path, "s.mtx", "%%MatrixMarket matrix coordinate real symmetric\n% c\n\n"
                 + body)
    m, n, row, col, val = api.read_matrix_market_to_csr(sym)
    D = np.zeros((3, 3))
    for i in range(3):
        D[i, col[row[i]:row[i + 1]]] = val[row[i]:row[i + 1]]
    ref = np.array([[2.0, -1.5, 0], [-1.5, 0, 0.25], [0, 0.25, 4.0]])
    assert np.array_equal(D, ref) and len(val) == 6
    skew = _write(tmp_path, "k.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric\n"
                  "3 3 2\n2 1 1.5\n3 2 -2\n")
    _, _, row, col, val = api.read_matrix_market_to_csr(skew)
    assert list(col) == [1, 0, 2, 1] and list(val) == [-1.5, 1.5, 2.0, -2.0]
    pat = _write(tmp_path, "p.mtx", "%%MatrixMarket matrix coordinate pattern general\n"
                 "2 3 3\n2 3\n1 1\n2 1\n")
    m, n, row, col, val = api.read_matrix_market_to_csr(pat)
    assert (m, n) == (2, 3) and list(row) == [0, 1, 3] and list(col) == [0, 0, 2]
    assert list(val) == [1.0, 1.0, 1.0]
    it = _write(tmp_path, "i.mtx", "%%MatrixMarket matrix coordinate integer general\n"
                "2 2 2\n2 2 7\n1 2 -3\n")
    _, _, row, col, val = api.read_matrix_market_to_csr(it)
    assert list(col) == [1, 1] and list(val) == [-3.0, 7.0]


def test_duplicates_are_kept_in_file_order(tmp_path):
    p = _write(tmp_path, "d.mtx", "%%MatrixMarket matrix coordinate real general\n"
               "2 2 3\n1 1 1.0\n1 1 2.0\n2 2 3.0\n")
    _, _, row, col, val = api.read_matrix_market_to_csr(p)
    assert list(row) == [0, 2, 3] and list(val) == [1.0, 2.0, 3.0]


@pytest.mark.parametrize("text,status", [
    ("not a banner\n1 1 1\n1 1 1.0\n", -9),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n3 1 1.0\n", -9),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n2 x 1.0\n", -9),
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n", -9),
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", -8),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1.0 0.0\n", -8),
])
def test_bad_files(tmp_path, text, status):
    p = _write(tmp_path, "bad.mtx", text)
    with pytest.raises(BiluError) as e:
        api.read_matrix_market_to_csr(p)
    assert e.value.status == status
    with pytest.raises(BiluError):
        api.read_matrix_market_to_csr(str(tmp_path / "missing.mtx"))


def test_bad_entry_index_is_reported(tmp_path):
    import ctypes

    from isai_kernel_gb300 import _lib

    p = _write(tmp_path, "b.mtx", "%%MatrixMarket matrix coordinate real general\n"
               "3 3 3\n1 1 1.0\n2 2 2.0\n9 1 1.0\n")
    m, n, nnz, bad = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
    st = _lib.lib().bilu_mtx_read(p.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz),
                                  None, None, None, ctypes.byref(bad))
    assert st == -9 and bad.value == 2


def test_binary_bsr_round_trip_and_checks(tmp_path):
    A = gen.powerlaw(300, bs=8, seed=4, kmax=25)
    p = str(tmp_path / "a.bsr")
    api.bsr_save(p, A.nb, A.bs, A.rowptr, A.colind, A.val)
    nb, bs, row, col, val = api.bsr_load(p)
    assert (nb, bs) == (A.nb, A.bs)
    assert np.array_equal(row, A.rowptr) and np.array_equal(col, A.colind)
    assert np.array_equal(val, A.val)
    # one flipped value bit: checksum mismatch
    raw = bytearray(open(p, "rb").read())
    raw[-5] ^= 0x10
    q = str(tmp_path / "c.bsr")
    open(q, "wb").write(bytes(raw))
    with pytest.raises(BiluError) as e:
        api.bsr_load(q)
    assert e.value.status == -9
    # truncated file
    open(q, "wb").write(bytes(raw[: len(raw) // 2]))
    with pytest.raises(BiluError):
        api.bsr_load(q)
    # a generated system written as .mtx reads back to the same matrix
    m = str(tmp_path / "l.mtx")
    B = gen.laplace2d(6, bs=4, seed=2)
    gen.write_mtx(m, B)
    nr, nc, r, c, v = api.read_matrix_market_to_csr(m)
    D = np.zeros((nr, nc))
    for i in range(nr):
        D[i, c[r[i]:r[i + 1]]] = v[r[i]:r[i + 1]]
    assert np.array_equal(D, B.to_dense())
    assert os.path.getsize(p) == 40 + 4 * (A.nb + 1) + 4 * A.nnzb + 8 * A.val.size
