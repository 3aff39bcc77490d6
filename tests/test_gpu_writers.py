"""Streamed writers: from_fasta_to_lower_triangular, dump_lower_triangular and
dump_sparse against the oracle's restatement of the reference formatters,
including outputs that span several streamed chunks."""
import os

import numpy as np
import pytest

from gpu_util import write
from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu
hd = pytest.importorskip("hammingdist_gb300")


def test_reference_python_case(tmp_path):
    seqs = [b"ACGTGTCGTGTCGACGTGTCGCAGGTGTCGACGTGTCGCAGGTGTCGACGTGTCGCAG",
            b"CCGTGTCGTGTCGACGTGTCGC-GGTGTCGACGTGTCGCAGGTGTCGACGTGTCGCAG",
            b"CAGTGT-GTGTCGACGTGTCGCAGGTGTCGACGTGTCGCAGGTGTCGACGTG--GCAG"]
    path = write(tmp_path, "f.fasta", b"".join(b">seq%d\n%s\n" % (i, s) for i, s in enumerate(seqs)))
    out = str(tmp_path / "o.txt")
    for md in (0, 1, 2, 3, 89, 497, 9999999):
        hd.from_fasta_to_lower_triangular(path, out, max_distance=md)
        assert open(out, "rb").read() == b"%d\n%d,%d\n" % (min(1, md), min(2, md), min(1, md))


@pytest.mark.parametrize("n,L,md", [(2, 17, 65535), (129, 88, 3), (300, 381, 89), (703, 17, 0)])
def test_lt_file_matches_oracle(tmp_path, n, L, md):
    seqs = synth.random_strings(n, L, b"ACGT-", seed=n + L)
    fa = b"".join(b">s\n" + s + b"\n" for s in seqs)
    path = write(tmp_path, "f.fasta", fa)
    out = str(tmp_path / "o.txt")
    hd.from_fasta_to_lower_triangular(path, out, max_distance=md)
    want = o.format_lower_triangular(o.lt_dense(seqs, max_distance=md, dtype=np.uint16))
    assert open(out, "rb").read() == want
    # the reference's own GPU test reads the file back with from_lower_triangular
    back = hd.from_lower_triangular_large(out)
    ds = hd.from_fasta_large(path, max_distance=md)
    np.testing.assert_array_equal(np.asarray(back.lt_array), np.asarray(ds.lt_array))


def test_single_row_leaves_file_untouched(tmp_path):
    path = write(tmp_path, "f.fasta", b">a\nACGT\n")
    out = tmp_path / "o.txt"
    hd.from_fasta_to_lower_triangular(path, str(out))
    assert not out.exists()
    hd.from_fasta(path).dump_lower_triangular(str(out))
    assert not out.exists()
    hd.from_fasta(path).dump_sparse(str(out), 3)
    assert out.exists() and out.read_bytes() == b""


def test_multi_chunk_streaming(tmp_path):
    """n=12,000 gives ~72M entries: several 256 MB text chunks."""
    n, L = 12000, 60
    seqs = synth.random_strings(n, L, b"ACGT-", seed=77)
    fa = b"".join(b">s\n" + s + b"\n" for s in seqs)
    path = write(tmp_path, "f.fasta", fa)
    out = str(tmp_path / "o.txt")
    hd.from_fasta_to_lower_triangular(path, out, max_distance=65535)
    lt = o.lt_dense(seqs, max_distance=65535, dtype=np.uint16)
    want = o.format_lower_triangular(lt)
    got = open(out, "rb").read()
    assert len(got) == len(want) and got == want
    ds = hd.from_fasta_large(path)
    ds.dump_lower_triangular(out)
    assert open(out, "rb").read() == want
    ds.dump_sparse(out, 20)
    got = sorted(open(out, "rb").read().splitlines())
    assert got == sorted(o.format_sparse(lt, n, 20).splitlines())


@pytest.mark.parametrize("threshold", [-1, 0, 2, 9, 255, 497])
def test_sparse_round_trip(tmp_path, threshold):
    """The reference's dump_sparse test shape: a random lower triangle read
    with from_lower_triangular, dumped sparse, each line checked."""
    rng = np.random.default_rng(threshold + 5)
    samples = 532
    lt_file = str(tmp_path / "lt.txt")
    rows = [rng.integers(0, 256, size=k) for k in range(1, samples)]
    with open(lt_file, "w") as f:
        for r in rows:
            f.write(",".join(str(x) for x in r) + "\n")
    data = hd.from_lower_triangular(lt_file)
    flat = np.concatenate(rows).astype(np.uint8)
    np.testing.assert_array_equal(np.asarray(data.lt_array), flat)
    sp = str(tmp_path / "sp.txt")
    data.dump_sparse(sp, threshold)
    got = sorted(open(sp, "rb").read().splitlines())
    assert got == sorted(o.format_sparse(flat, samples, threshold).splitlines())
    assert len(got) == int(np.sum(flat.astype(np.int64) <= threshold))
