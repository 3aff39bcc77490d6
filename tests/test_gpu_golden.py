"""The GPU path against outputs of the reference itself (tests/golden/).

use_gpu=False must reproduce the reference CPU's values (dense or sparse rule,
as its heuristic picks); use_gpu=True must reproduce the reference GPU's
dense AND rule, which the reference CPU also computes whenever it took the
dense branch."""
import numpy as np
import pytest

from gpu_util import seqidx_of, write

pytestmark = pytest.mark.gpu
hd = pytest.importorskip("hammingdist_gb300")


def _run(fn, path, run, use_gpu, tmp_path):
    kw = dict(remove_duplicates=bool(run["dedup"]), use_gpu=use_gpu)
    if "x" in run:
        kw["include_x"] = bool(run["x"])
    if "md" in run:
        kw["max_distance"] = run["md"]
    if "n" in run:
        kw["n"] = run["n"]
    return fn(path, **kw)


def _check(golden, fa, run, tmp_path):
    path = write(tmp_path, "in.fasta", fa)
    fn = hd.from_fasta_large if run.get("large") else hd.from_fasta
    modes = [False]
    if "error" in run or run.get("path") == "dense":
        modes.append(True)
    for use_gpu in modes:
        if use_gpu and run.get("x"):
            with pytest.raises(RuntimeError, match="use_gpu=True cannot be used if include_x=True"):
                _run(fn, path, run, True, tmp_path)
            continue
        if "error" in run:
            with pytest.raises(RuntimeError) as e:
                _run(fn, path, run, use_gpu, tmp_path)
            assert str(e.value) == run["error"]
            continue
        ds = _run(fn, path, run, use_gpu, tmp_path)
        lt = np.asarray(ds.lt_array)
        want = golden[run["key"] + "/lt"]
        assert lt.dtype == want.dtype
        np.testing.assert_array_equal(lt, want, err_msg=f"{run} use_gpu={use_gpu}")
        np.testing.assert_array_equal(seqidx_of(ds, tmp_path), golden[run["key"] + "/seqidx"])


def test_alignments(golden, tmp_path):
    n = 0
    for name, fa, run in golden.alignment_runs():
        _check(golden, fa, run, tmp_path)
        n += 1
    assert n > 300


def test_fasta_parsing(golden, tmp_path):
    for name, fa, run in golden.parse_runs():
        _check(golden, fa, run, tmp_path)


def test_reference_distances_and_indices(golden, tmp_path):
    for case in golden.meta["cases"]:
        name = case["name"]
        path = write(tmp_path, "in.fasta", golden.bytes(f"aln/{name}/fasta"))
        for k, x in case["refdist"]:
            ref = golden.bytes(f"aln/{name}/refseq{k}").decode()
            got = hd.fasta_reference_distances(ref, path, include_x=bool(x))
            assert got.dtype == np.uint32
            np.testing.assert_array_equal(got, golden[f"aln/{name}/refdist{k}x{x}"])
        for nlim in case["seqidx"]:
            got = hd.fasta_sequence_indices(path, n=nlim)
            np.testing.assert_array_equal(got, golden[f"aln/{name}/seqidx_n{nlim}"])
    for entry in golden.meta["parse"]:
        name = entry["name"]
        path = write(tmp_path, "in.fasta", golden.bytes(f"parse/{name}/fasta"))
        ref = golden.bytes(f"parse/{name}/refseq").decode()
        for x in (0, 1):
            np.testing.assert_array_equal(hd.fasta_reference_distances(ref, path, include_x=bool(x)),
                                          golden[f"parse/{name}/refdist{x}"])
        for nlim in (0, 2):
            np.testing.assert_array_equal(hd.fasta_sequence_indices(path, nlim),
                                          golden[f"parse/{name}/seqidx_n{nlim}"])


def test_writers(golden, tmp_path):
    out = str(tmp_path / "out.txt")
    for case in golden.meta["cases"]:
        name = case["name"]
        path = write(tmp_path, "in.fasta", golden.bytes(f"aln/{name}/fasta"))
        for large in (0, 1):
            key = f"aln/{name}/lttext{large}"
            if key not in golden.npz:
                continue
            fn = hd.from_fasta_large if large else hd.from_fasta
            ds = fn(path)
            ds.dump_lower_triangular(out)
            assert open(out, "rb").read() == golden.bytes(key)
            for thr in (0, 1, 3, 20, 255):
                ds.dump_sparse(out, thr)
                got = b"".join(sorted(open(out, "rb").read().splitlines(keepends=True)))
                assert got == golden.bytes(f"aln/{name}/sparse{large}t{thr}")


def test_truth_tables_kat_and_saturation(golden, tmp_path):
    chars = golden.meta["truth_chars"]
    for x in (0, 1):
        dist = golden[f"truth/distance/x{x}"]
        lt1 = golden[f"truth/stringlist/x{x}"]
        for a, ca in enumerate(chars):
            for b, cb in enumerate(chars):
                assert hd.distance(ca, cb, include_x=bool(x)) == dist[a, b]
                assert hd.from_stringlist([ca, cb], bool(x), False, 255)[0, 1] == lt1[a, b]
    for a, b, d_lt, d_dist in golden.meta["kat2"]:
        for use_gpu in (False, True):
            d = hd.from_stringlist([a, b], False, use_gpu, 255)
            assert d[0, 1] == d[1, 0] == 2 and d[0, 0] == d[1, 1] == 0
        assert hd.distance(a, b) == 2 and hd.distance(a, a) == 0
    for m, md, d8, d16 in golden.meta["saturation"]:
        path = write(tmp_path, "sat.fasta", b">a\n" + b"A" * m + b"\n>t\n" + b"T" * m + b"\n")
        for use_gpu in (False, True):
            assert hd.from_fasta(path, use_gpu=use_gpu, max_distance=md)[0, 1] == d8
            assert hd.from_fasta_large(path, use_gpu=use_gpu, max_distance=md)[1, 0] == d16
