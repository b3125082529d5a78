"""io::read_matrix_market_file / write_matrix_market_file through the C ABI:
the reference reader's result on each file of tests/golden/mm (its return
value, the matrix, and the files it rejects), a large file parsed by all host
threads against the Python restatement, and writer round trips."""
import os

import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import GOLDEN, rel_err

pytestmark = pytest.mark.gpu

CASES = [("general", 1), ("general_case", 1), ("symmetric", 1), ("pattern", 1), ("complex", 1),
         ("zero_based", 0), ("extra_lines", 1), ("bad_word", 1), ("bad_field", 1),
         ("bad_symmetry", 1), ("array", 1), ("out_of_range", 1), ("too_few", 1),
         ("missing_value", 1)]


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _csr(V, A):
    import torch
    inf = A.info()
    rp = A.export(0, inf.rows + 1, torch.int32).cpu().numpy().view(np.uint32)
    ci = A.export(1, inf.nnz, torch.int32).cpu().numpy().view(np.uint32)
    v = A.export(2, inf.nnz, torch.float64).cpu().numpy()
    return inf, rp, ci, v


@pytest.mark.parametrize("name,base", CASES)
def test_reader_matches_the_reference(V, golden, name, base):
    d = golden("matrix_market.npz")
    path = os.path.join(GOLDEN, "mm", name + ".mtx")
    ret = int(d[name + "__ret"][0])
    if ret == 0:  # the reference prints an error and returns 0
        with pytest.raises(V.VclgbError) as e:
            V.read_matrix_market_file(path, base)
        assert e.value.status == V.INVALID_ARGUMENT
        return
    A, lines = V.read_matrix_market_file(path, base)
    inf, rp, ci, v = _csr(V, A)
    assert lines == ret and inf.rows == int(d[name + "__ret"][1])
    assert np.array_equal(rp, d[name + "__rp"]) and np.array_equal(ci, d[name + "__ci"])
    assert np.array_equal(v, d[name + "__v"])


def test_missing_file(V):
    with pytest.raises(V.VclgbError) as e:
        V.read_matrix_market_file("/nonexistent/matrix.mtx")
    assert e.value.status == V.INVALID_ARGUMENT


def test_large_file_parsed_in_parallel(V, tmp_path):
    # ~12 MB: split over the host threads; duplicates and symmetric mirroring
    # across chunk boundaries resolved in file order
    rng = np.random.default_rng(7)
    n, k = 20000, 400000
    r = rng.integers(1, n + 1, k)
    c = rng.integers(1, n + 1, k)
    r[1000:2000] = r[:1000]          # repeated positions far apart in the file
    c[1000:2000] = c[:1000]
    val = rng.normal(size=k)
    path = str(tmp_path / "big.mtx")
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n% a comment\n")
        f.write("%d %d %d\n" % (n, n, k))
        f.writelines("%d %d %r\n" % (a, b, float(x)) for a, b, x in zip(r, c, val))
    A, lines = V.read_matrix_market_file(path)
    inf, rp, ci, v = _csr(V, A)
    ref = oracle.read_matrix_market(path)
    assert lines == ref[0] and inf.rows == ref[1]
    assert np.array_equal(rp, ref[3]) and np.array_equal(ci, ref[4]) and np.array_equal(v, ref[5])


def test_writer_round_trip(V, tmp_path):
    rp, ci, v = gen.lognormal_random(3000, mu=1.5, sigma=0.7, hi=50, seed=3)
    A = V.compressed_matrix(rp, ci, v)
    exact = str(tmp_path / "exact.mtx")
    V.write_matrix_market_file(A, exact, digits=17)
    B, _ = V.read_matrix_market_file(exact)
    _, rp2, ci2, v2 = _csr(V, B)
    assert np.array_equal(rp2, rp) and np.array_equal(ci2, ci) and np.array_equal(v2, v)
    # the reference's default: 6 significant digits, as its stream writes them
    short = str(tmp_path / "short.mtx")
    V.write_matrix_market_file(A, short)
    lines = open(short).read().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate real general"
    assert lines[1] == "%d %d %d" % (3000, 3000, int(rp[-1]))
    rows = np.repeat(np.arange(3000), np.diff(rp.astype(np.int64)))
    for k in (0, 17, int(rp[-1]) - 1):
        assert lines[2 + k] == "%d %d %s" % (rows[k] + 1, ci[k] + 1, "%.6g" % v[k])
    C, _ = V.read_matrix_market_file(short)
    x = np.random.default_rng(1).uniform(-1, 1, 3000)
    assert rel_err(V.prod(C, x).cpu().numpy(), oracle.spmv(rp, ci, v, x)) < 1e-5


def test_empty_matrix_file(V, tmp_path):
    # "rows cols 0": an empty matrix (the reference reports a failure here,
    # from its parse of the line after the size line)
    path = str(tmp_path / "empty.mtx")
    open(path, "w").write("%%MatrixMarket matrix coordinate real general\n% nothing\n7 5 0\n")
    A, lines = V.read_matrix_market_file(path)
    inf = A.info()
    assert (inf.rows, inf.cols, inf.nnz, lines) == (7, 5, 0, 3)
