"""Result files on the device: DataSet.dump (full matrix text),
from_lower_triangular[_large] and from_csv against the reference's own
outputs (tests/golden), including the exceptions it raises on malformed
input, and round trips at sizes that take several streamed chunks."""
import numpy as np
import pytest

from goldens import golden_arrays, golden_meta
from oracle import hd_formats as f
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu
EXC = {"ValueError": ValueError, "IndexError": IndexError}


@pytest.fixture(scope="module")
def hd():
    import hammingdist_gb300

    return hammingdist_gb300


def _bytes(a):
    return bytes(np.asarray(a, dtype=np.uint8))


def _dump(ds, tmp_path):
    p = tmp_path / "dump.txt"
    ds.dump(str(p))
    return p.read_bytes()


@pytest.mark.parametrize("case", golden_meta()["formats"]["lt"], ids=lambda c: c["name"])
def test_from_lower_triangular_golden(hd, tmp_path, case):
    z = golden_arrays()
    path = tmp_path / "in.txt"
    path.write_bytes(_bytes(z[f"fmt/lt/{case['name']}/input"]))
    for large, fn in ((0, hd.from_lower_triangular), (1, hd.from_lower_triangular_large)):
        if f"error{large}" in case:
            etype, msg = case[f"error{large}"]
            with pytest.raises(EXC[etype], match=msg):
                fn(str(path))
            continue
        ds = fn(str(path))
        np.testing.assert_array_equal(np.asarray(ds.lt_array),
                                      z[f"fmt/lt/{case['name']}/lt{large}"])
        assert _dump(ds, tmp_path) == _bytes(z[f"fmt/lt/{case['name']}/dump{large}"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["csv"], ids=lambda c: c["name"])
def test_from_csv_golden(hd, tmp_path, case):
    z = golden_arrays()
    path = tmp_path / "in.csv"
    path.write_bytes(_bytes(z[f"fmt/csv/{case['name']}/input"]))
    if "error" in case:
        etype, msg = case["error"]
        with pytest.raises(EXC[etype], match=msg):
            hd.from_csv(str(path))
        return
    ds = hd.from_csv(str(path))
    np.testing.assert_array_equal(np.asarray(ds.lt_array), z[f"fmt/csv/{case['name']}/lt"])
    assert _dump(ds, tmp_path) == _bytes(z[f"fmt/csv/{case['name']}/dump"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["dump"],
                         ids=lambda c: f"{c['name']}{c['large']}")
def test_dump_golden(hd, tmp_path, case):
    z = golden_arrays()
    fa = tmp_path / "a.fasta"
    fa.write_bytes(_bytes(z[f"aln/{case['name']}/fasta"]))
    ds = (hd.from_fasta_large if case["large"] else hd.from_fasta)(str(fa))
    assert _dump(ds, tmp_path) == _bytes(z[f"fmt/dump/{case['name']}{case['large']}"])


def test_missing_files_give_empty_datasets(hd, tmp_path):
    missing = str(tmp_path / "missing.txt")
    assert np.asarray(hd.from_lower_triangular(missing).lt_array).size == 0
    assert _dump(hd.from_lower_triangular(missing), tmp_path) == b"0\n"
    assert np.asarray(hd.from_csv(missing).lt_array).size == 0
    assert _dump(hd.from_csv(missing), tmp_path) == b""


@pytest.mark.parametrize("dt", [np.uint8, np.uint16])
def test_round_trips_several_chunks(tmp_path, dt):
    # a 9,000-row matrix: its full text (0.4-0.6 GB) takes several 256 MB
    # chunks; lower-triangular text -> from_lower_triangular and dump ->
    # from_csv must give the values back; the first and last rows of the
    # dump are checked against the format oracle
    from hammingdist_gb300 import abi

    n = 9000
    rng = np.random.default_rng(3)
    hi = 300 if dt == np.uint8 else 70000
    lt = np.minimum(rng.integers(0, hi, size=n * (n - 1) // 2), np.iinfo(dt).max).astype(dt)
    ctx = abi.Context(0)
    try:
        ltp = tmp_path / "lt.txt"
        ctx.write_lower_triangular(lt, n, str(ltp))
        back, n_back = ctx.read_lower_triangular(str(ltp), dt)
        assert n_back == n
        np.testing.assert_array_equal(back, lt)
        full = tmp_path / "full.txt"
        ctx.write_full_matrix(lt, n, str(full))
        lines = full.read_bytes().splitlines(keepends=True)
        assert len(lines) == n
        for i in (0, 1, 4500, n - 1):
            want = ", ".join(str(f.entry(lt, i, j)) for j in range(n)).encode() + b"\n"
            assert lines[i] == want, i
        csv_vals, n_csv = ctx.read_csv(str(full))
        assert n_csv == n
        np.testing.assert_array_equal(csv_vals[: lt.size], (lt.astype(np.int64) % 256).astype(np.uint8))
        assert not csv_vals[lt.size:].any()
    finally:
        ctx.close()


def test_parse_error_kinds_through_the_abi(tmp_path):
    from hammingdist_gb300 import abi

    ctx = abi.Context(0)
    try:
        p = tmp_path / "e.txt"
        for text, kind in ((b"1\n2,x\n", 1), (b"1\n99999999999,3\n", 2), (b"1\n2,3,\n", 1)):
            p.write_bytes(text)
            with pytest.raises(abi.HDError) as e:
                ctx.read_lower_triangular(str(p))
            assert e.value.code == -12 and e.value.parse_error == kind
        # a later, different error does not mask the first one in file order
        p.write_bytes(b"1\n" + b"5," * 5000 + b"x\n" + b"9" * 20 + b"\n")
        with pytest.raises(abi.HDError) as e:
            ctx.read_lower_triangular(str(p))
        assert e.value.parse_error == 1
        with pytest.raises(ValueError):
            f.from_lower_triangular(p.read_bytes())
    finally:
        ctx.close()
