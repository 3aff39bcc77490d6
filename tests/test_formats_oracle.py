"""The format oracle (oracle/hd_formats.py) against the reference's own
outputs (tests/golden: dump, from_lower_triangular[_large], from_csv,
including the exceptions it raises on malformed input)."""
import numpy as np
import pytest

from goldens import golden_arrays, golden_meta
from oracle import hd_formats as f


def _bytes(a):
    return bytes(np.asarray(a, dtype=np.uint8))


@pytest.mark.parametrize("case", golden_meta()["formats"]["lt"], ids=lambda c: c["name"])
def test_lt_reader_oracle(case):
    z = golden_arrays()
    data = _bytes(z[f"fmt/lt/{case['name']}/input"])
    for large, dt in ((0, np.uint8), (1, np.uint16)):
        if f"error{large}" in case:
            etype = {"ValueError": ValueError, "IndexError": IndexError}[case[f"error{large}"][0]]
            with pytest.raises(etype, match=case[f"error{large}"][1]):
                f.from_lower_triangular(data, dt)
            continue
        lt, n = f.from_lower_triangular(data, dt)
        np.testing.assert_array_equal(lt, z[f"fmt/lt/{case['name']}/lt{large}"])
        assert f.dump_text(lt, n) == _bytes(z[f"fmt/lt/{case['name']}/dump{large}"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["csv"], ids=lambda c: c["name"])
def test_csv_reader_oracle(case):
    z = golden_arrays()
    data = _bytes(z[f"fmt/csv/{case['name']}/input"])
    if "error" in case:
        etype = {"ValueError": ValueError, "IndexError": IndexError}[case["error"][0]]
        with pytest.raises(etype, match=case["error"][1]):
            f.from_csv(data)
        return
    lt, n = f.from_csv(data)
    np.testing.assert_array_equal(lt, z[f"fmt/csv/{case['name']}/lt"])
    assert f.dump_text(lt, n) == _bytes(z[f"fmt/csv/{case['name']}/dump"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["dump"],
                         ids=lambda c: f"{c['name']}{c['large']}")
def test_dump_oracle(case):
    from oracle import hd_oracle as o

    z = golden_arrays()
    fa = _bytes(z[f"aln/{case['name']}/fasta"])
    dt = np.uint16 if case["large"] else np.uint8
    lt, _ = o.from_fasta_dense(fa, max_distance=np.iinfo(dt).max, dtype=dt)
    n = f.nsamples_of(lt.size) if lt.size else len(o.read_fasta(fa)[0])
    assert f.dump_text(lt, n) == _bytes(z[f"fmt/dump/{case['name']}{case['large']}"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["lt"], ids=lambda c: c["name"])
def test_lt_reader_c_oracle(case, tmp_path):
    from oracle import hd_oracle as o

    z = golden_arrays()
    p = tmp_path / "in.txt"
    p.write_bytes(_bytes(z[f"fmt/lt/{case['name']}/input"]))
    for large, dt in ((0, np.uint8), (1, np.uint16)):
        if f"error{large}" in case:
            etype = {"ValueError": ValueError, "IndexError": IndexError}[case[f"error{large}"][0]]
            with pytest.raises(etype, match="stoi"):
                o.read_lower_triangular(str(p), dt)
            continue
        lt, n = o.read_lower_triangular(str(p), dt)
        np.testing.assert_array_equal(lt, z[f"fmt/lt/{case['name']}/lt{large}"])
        out = tmp_path / "dump.txt"
        o.dump_full(lt, n, str(out))
        assert out.read_bytes() == _bytes(z[f"fmt/lt/{case['name']}/dump{large}"])


@pytest.mark.parametrize("case", golden_meta()["formats"]["csv"], ids=lambda c: c["name"])
def test_csv_reader_c_oracle(case, tmp_path):
    from oracle import hd_oracle as o

    z = golden_arrays()
    p = tmp_path / "in.csv"
    p.write_bytes(_bytes(z[f"fmt/csv/{case['name']}/input"]))
    if "error" in case:
        etype = {"ValueError": ValueError, "IndexError": IndexError}[case["error"][0]]
        with pytest.raises(etype, match="stoi"):
            o.read_csv(str(p))
        return
    lt, n = o.read_csv(str(p))
    np.testing.assert_array_equal(lt, z[f"fmt/csv/{case['name']}/lt"])
    out = tmp_path / "dump.txt"
    o.dump_full(lt, n, str(out))
    assert out.read_bytes() == _bytes(z[f"fmt/csv/{case['name']}/dump"])
