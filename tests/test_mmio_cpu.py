"""Matrix Market exchange files (rsg_mm_*): the reading rules of
CompRowMatrix(MatrixVectorReader) (mtj/.../sparse/CompRowMatrix.java:68-146)
and DenseVector(MatrixVectorReader) (mtj/.../DenseVector.java:52-96), and
the lines MatrixVectorWriter prints (mtj/.../io/MatrixVectorWriter.java).
Host code: no GPU needed."""
import numpy as np
import pytest

from ressim_gb300 import abi, api


def _random_csr(n, m, density, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    rp, col, val = [0], [], []
    for i in range(n):
        cs = np.flatnonzero(g.random(m) < density)
        col.extend(cs.tolist())
        val.extend((g.standard_normal(len(cs)) * 10.0 ** g.integers(-20, 20, len(cs))).tolist())
        rp.append(len(col))
    return np.array(rp, np.int32), np.array(col, np.int32), np.array(val)


def test_write_read_round_trip(tmp_path):
    """Written entries come back as the 13 significant digits printed, with
    the same pattern; the lines have MatrixVectorWriter's widths."""
    rp, col, val = _random_csr(40, 35, 0.2, 1)
    f = tmp_path / "a.mtx"
    api.write_matrix_market(f, 40, 35, rp, col, val)
    lines = f.read_text().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate real general"
    assert lines[1] == "%10d %10d %19d" % (40, 35, len(col))
    rows = np.repeat(np.arange(40), np.diff(rp))
    for k in (0, len(col) // 2, len(col) - 1):
        assert lines[2 + k] == "%10d %10d % .12e" % (rows[k] + 1, col[k] + 1, val[k])
    n, m, rp2, col2, val2 = api.read_matrix_market(f)
    assert (n, m) == (40, 35)
    assert np.array_equal(rp2, rp) and np.array_equal(col2, col)
    assert np.array_equal(val2, np.array([float("%.12e" % v) for v in val]))


def test_reader_semantics(tmp_path):
    """No header means coordinate real general; comments may appear between
    entries; rows come out sorted; a repeated entry keeps its last value."""
    f = tmp_path / "b.mtx"
    f.write_text("% a comment before the size line\n3 4 5\n3 1 2.5\n1 4 -1e-3\n% inside\n1 2 7\n1 4 4.0\n"
                 "2\t2\t1.0E+02\n")
    n, m, rp, col, val = api.read_matrix_market(f)
    assert (n, m) == (3, 4)
    assert rp.tolist() == [0, 2, 3, 4]
    assert col.tolist() == [1, 3, 1, 0]
    assert val.tolist() == [7.0, 4.0, 100.0, 2.5]


def test_symmetric_and_skew_symmetric(tmp_path):
    """Off-diagonal entries are mirrored (negated for skew-symmetric), after
    all the stored entries."""
    body = "3 3 4\n1 1 2.0\n2 1 -1.0\n3 2 -0.5\n3 1 0.25\n"
    f = tmp_path / "s.mtx"
    f.write_text("%%MatrixMarket matrix coordinate real symmetric\n" + body)
    n, m, rp, col, val = api.read_matrix_market(f)
    A = np.zeros((3, 3))
    for i in range(3):
        A[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    assert np.array_equal(A, A.T) and A[1, 0] == -1.0 and A[0, 2] == 0.25
    f.write_text("%%MatrixMarket matrix coordinate real skew-symmetric\n" + body.replace("1 1 2.0", "1 1 0.0"))
    n, m, rp, col, val = api.read_matrix_market(f)
    A = np.zeros((3, 3))
    for i in range(3):
        A[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    assert np.array_equal(A, -A.T) and A[2, 1] == -0.5 and A[1, 2] == 0.5


@pytest.mark.parametrize("header,status", [
    ("%%MatrixMarket matrix coordinate pattern general", abi.UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate complex general", abi.UNSUPPORTED),
    ("%%MatrixMarket matrix array real general", abi.UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate real", abi.BAD_ARG),
    ("%%MatrixMarket vector coordinate real general", abi.BAD_ARG),
])
def test_rejected_headers(tmp_path, header, status):
    f = tmp_path / "r.mtx"
    f.write_text(header + "\n2 2 1\n1 1 1\n")
    with pytest.raises(api.RSGError) as e:
        api.read_matrix_market(f)
    assert e.value.status == status


def test_bad_entries(tmp_path):
    f = tmp_path / "e.mtx"
    for body in ("2 2 1\n3 1 1.0\n", "2 2 2\n1 1 1.0\n", "2 2 1\n1 x 1.0\n", "2 2 1\n1 1 1.0q\n"):
        f.write_text(body)
        with pytest.raises(api.RSGError) as e:
            api.read_matrix_market(f)
        assert e.value.status == abi.BAD_ARG
    with pytest.raises(api.RSGError):
        api.read_matrix_market(tmp_path / "missing.mtx")


def test_vectors(tmp_path):
    x = np.array([1.0, -2.5e-300, 3.0e300, 0.0, 1.0 / 3.0])
    f = tmp_path / "x.mtx"
    api.write_matrix_market_vector(f, x)
    lines = f.read_text().splitlines()
    assert lines[0] == "%%MatrixMarket vector array real" and lines[1] == "%10d" % 5
    assert lines[2:] == ["% .12e" % v for v in x]
    assert np.array_equal(api.read_matrix_market_vector(f), np.array([float("%.12e" % v) for v in x]))
    f.write_text("%%MatrixMarket vector coordinate real\n4 2\n3 1.5\n1 -2\n")
    assert api.read_matrix_market_vector(f).tolist() == [-2.0, 0.0, 1.5, 0.0]
    f.write_text("3 1\n2 7\n")  # no header: a coordinate vector
    assert api.read_matrix_market_vector(f).tolist() == [0.0, 7.0, 0.0]
