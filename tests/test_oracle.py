"""Pins the C restatement (oracle/hd_oracle.c) against outputs of the reference
itself (tests/golden/, generated by tests/golden/make_golden.py from the
reference compiled from its own sources). CPU only."""
import numpy as np
import pytest

from oracle import hd_oracle as o


def _max_clamp(md, large):
    tmax = 65535 if large else 255
    return tmax if md > tmax else (md & tmax)


def _expect_error(fn, msg):
    with pytest.raises(RuntimeError) as e:
        fn()
    assert str(e.value) == msg


def test_truth_tables(golden):
    chars = golden.meta["truth_chars"]
    for x in (0, 1):
        dist = golden[f"truth/distance/x{x}"]
        lt1 = golden[f"truth/stringlist/x{x}"]
        for a, ca in enumerate(chars):
            for b, cb in enumerate(chars):
                assert o.distance(ca, cb, bool(x)) == dist[a, b], (ca, cb, x)
                lt, _ = o.lt_cpu([ca, cb], include_x=bool(x), max_distance=255)
                assert lt[0] == lt1[a, b], (ca, cb, x)


def test_known_answer_pairs(golden):
    for a, b, d_lt, d_dist in golden.meta["kat2"]:
        assert d_lt == 2 and d_dist == 2
        assert o.lt_cpu([a, b])[0][0] == 2
        assert o.lt_dense([a, b])[0] == 2
        assert o.distance(a, b) == 2
        assert o.distance(a, a) == 0


def test_saturation(golden):
    for m, md, d8, d16 in golden.meta["saturation"]:
        fa = b">a\n" + b"A" * m + b"\n>t\n" + b"T" * m + b"\n"
        assert o.from_fasta_dense(fa, max_distance=md, dtype=np.uint8)[0][0] == d8
        assert o.from_fasta_dense(fa, max_distance=md, dtype=np.uint16)[0][0] == d16


def _check_run(fa, run, large_key="large"):
    large = run.get(large_key, 0)
    dtype = np.uint16 if large else np.uint8
    md = run.get("md", 65535 if large else 255)
    dedup = bool(run["dedup"])
    nlim = run.get("n", 0)
    x = bool(run.get("x", 0))
    seqs, idx = o.read_fasta(fa, dedup, nlim)
    if "error" in run:
        _expect_error(lambda: o.lt_cpu(seqs, include_x=x, max_distance=md, dtype=dtype),
                      run["error"])
        return
    lt_ref = run_lt = None
    lt_ref = run["_lt"]
    lt, used_sparse = o.lt_cpu(seqs, include_x=x, max_distance=md, dtype=dtype)
    assert used_sparse == (run["path"] == "sparse")
    np.testing.assert_array_equal(lt, lt_ref)
    if run["path"] == "dense":
        # the dense branch is the reference GPU's AND rule
        np.testing.assert_array_equal(o.lt_dense(seqs, max_distance=md, dtype=dtype), lt_ref)
        lt2, idx2 = o.from_fasta_dense(fa, dedup, nlim, md, dtype)
        np.testing.assert_array_equal(lt2, lt_ref)
    if dedup:
        np.testing.assert_array_equal(idx, run["_seqidx"])
    else:
        np.testing.assert_array_equal(np.arange(len(seqs)), run["_seqidx"])


def test_alignment_runs(golden):
    n = 0
    for name, fa, run in golden.alignment_runs():
        if "error" not in run:
            run = dict(run, _lt=golden[run["key"] + "/lt"], _seqidx=golden[run["key"] + "/seqidx"])
        _check_run(fa, run)
        n += 1
    assert n > 300


def test_parse_runs(golden):
    for name, fa, run in golden.parse_runs():
        if "error" not in run:
            run = dict(run, _lt=golden[run["key"] + "/lt"], _seqidx=golden[run["key"] + "/seqidx"])
        _check_run(fa, run)


def test_reference_distances_and_indices(golden):
    for case in golden.meta["cases"]:
        name = case["name"]
        fa = golden.bytes(f"aln/{name}/fasta")
        for k, x in case["refdist"]:
            refseq = golden.bytes(f"aln/{name}/refseq{k}")
            np.testing.assert_array_equal(o.reference_distances(refseq, fa, bool(x)),
                                          golden[f"aln/{name}/refdist{k}x{x}"])
        for nlim in case["seqidx"]:
            np.testing.assert_array_equal(o.fasta_sequence_indices(fa, nlim),
                                          golden[f"aln/{name}/seqidx_n{nlim}"])
    for entry in golden.meta["parse"]:
        name = entry["name"]
        fa = golden.bytes(f"parse/{name}/fasta")
        refseq = golden.bytes(f"parse/{name}/refseq")
        for x in (0, 1):
            np.testing.assert_array_equal(o.reference_distances(refseq, fa, bool(x)),
                                          golden[f"parse/{name}/refdist{x}"])
        for nlim in (0, 2):
            np.testing.assert_array_equal(o.fasta_sequence_indices(fa, nlim),
                                          golden[f"parse/{name}/seqidx_n{nlim}"])


def test_writers(golden):
    for case in golden.meta["cases"]:
        name = case["name"]
        fa = golden.bytes(f"aln/{name}/fasta")
        for large in (0, 1):
            key = f"aln/{name}/lttext{large}"
            if key not in golden.npz:
                continue
            run = next(r for r in case["runs"] if r["large"] == large and r["x"] == 0
                       and r["dedup"] == 0 and r["md"] == (65535 if large else 255))
            lt = golden[run["key"] + "/lt"]
            assert o.format_lower_triangular(lt) == golden.bytes(key)
            n = int(run["nsamples"])
            nsamp = int(round((1 + (1 + 8 * n) ** 0.5) / 2))
            for thr in (0, 1, 3, 20, 255):
                got = b"".join(sorted(o.format_sparse(lt, nsamp, thr).splitlines(keepends=True)))
                assert got == golden.bytes(f"aln/{name}/sparse{large}t{thr}")
