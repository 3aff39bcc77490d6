"""FASTA file entry points: the pipelined read + upload gives the same
alignment as the byte entry points; a second call on the same unchanged file
reuses the device bytes; a changed file, or byte input in between, is read
again."""
import os

import numpy as np
import pytest

from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from hammingdist_gb300 import abi

    c = abi.Context(0)
    yield c
    c.close()


def _fasta(seqs):
    return b"".join(b">s%d\n" % k + s + b"\n" for k, s in enumerate(seqs))


def test_file_equals_bytes_and_oracle(ctx, tmp_path):
    seqs = synth.random_strings(400, 3001, b"ACGT-N", seed=11)
    fa = _fasta(seqs + seqs[:57])  # duplicates at the end
    p = tmp_path / "a.fasta"
    p.write_bytes(fa)
    a = ctx.alignment_from_fasta_file(str(p), remove_duplicates=True)
    b = ctx.alignment_from_fasta(fa, remove_duplicates=True)
    assert a.n_rows == b.n_rows == 400
    np.testing.assert_array_equal(ctx.pairwise_lt(a), ctx.pairwise_lt(b))
    np.testing.assert_array_equal(ctx.pairwise_lt(a), o.lt_dense(seqs))
    np.testing.assert_array_equal(a.sequence_indices(), b.sequence_indices())
    a.free()
    b.free()


def test_large_file_parts(ctx, tmp_path):
    # 60 MB: several 8 MB parts read by different threads
    rows, root, _ = synth.alignment(2000, 29903, p=1e-3, seed=3, dup_frac=0.2)
    fa = synth.to_fasta(rows)
    p = tmp_path / "big.fasta"
    p.write_bytes(fa)
    a = ctx.alignment_from_fasta_file(str(p), remove_duplicates=True)
    b = ctx.alignment_from_fasta(fa, remove_duplicates=True)
    np.testing.assert_array_equal(ctx.pairwise_lt(a), ctx.pairwise_lt(b))
    np.testing.assert_array_equal(ctx.reference_distances_file(root.tobytes(), str(p)),
                                  o.reference_distances(root.tobytes(), fa))
    a.free()
    b.free()


def test_device_cache_and_invalidation(ctx, tmp_path):
    seqs = synth.random_strings(300, 1000, b"ACGT-", seed=12)
    ref = seqs[0]
    p = tmp_path / "c.fasta"
    fa = _fasta(seqs)
    p.write_bytes(fa)
    ctx.trace(True)
    try:
        a = ctx.alignment_from_fasta_file(str(p))
        assert "read + upload" in ctx.trace_last()
        rd = ctx.reference_distances_file(ref, str(p))
        assert "file already on the device" in ctx.trace_last()
        np.testing.assert_array_equal(rd, o.reference_distances(ref, fa))
        np.testing.assert_array_equal(ctx.fasta_sequence_indices_file(str(p)),
                                      np.arange(300, dtype=np.uint64))
        # same size, new contents (and a new mtime/ctime): read again
        seqs2 = synth.random_strings(300, 1000, b"ACGT-", seed=13)
        fa2 = _fasta(seqs2)
        assert len(fa2) == len(fa)
        p.write_bytes(fa2)
        st = os.stat(p)
        os.utime(p, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000))
        rd2 = ctx.reference_distances_file(ref, str(p))
        assert "file already on the device" not in ctx.trace_last()
        np.testing.assert_array_equal(rd2, o.reference_distances(ref, fa2))
        # byte input replaces the device buffer: the file is read again
        ctx.reference_distances(ref, fa)
        rd3 = ctx.reference_distances_file(ref, str(p))
        assert "file already on the device" not in ctx.trace_last()
        np.testing.assert_array_equal(rd3, rd2)
        a.free()
    finally:
        ctx.trace(False)


def test_file_errors(ctx, tmp_path):
    from hammingdist_gb300 import abi

    with pytest.raises(abi.HDError, match="Failed to open file"):
        ctx.alignment_from_fasta_file(str(tmp_path / "missing.fasta"))
    with pytest.raises(abi.HDError, match="Failed to open file"):
        ctx.reference_distances_file(b"ACGT", str(tmp_path))  # a directory
    p = tmp_path / "e.fasta"
    p.write_bytes(b"")
    with pytest.raises(abi.HDError, match="Empty sequence"):
        ctx.alignment_from_fasta_file(str(p))


@pytest.mark.parametrize("mode", ["map", "pread"])
def test_read_modes(tmp_path, monkeypatch, mode):
    # HAMMINGDIST_READ_MODE=pread: pread into pinned staging; else, where the
    # device reads pageable memory through the host's page tables, the file's
    # mapping is copied directly. Both give the bytes' results: a 72 MB file
    # (9 parts, more than one copy), and a small one of odd size.
    from hammingdist_gb300 import abi

    if mode == "pread":
        monkeypatch.setenv("HAMMINGDIST_READ_MODE", "pread")
    else:
        monkeypatch.delenv("HAMMINGDIST_READ_MODE", raising=False)
    c = abi.Context(0)
    try:
        rows, root, _ = synth.alignment(2400, 29903, p=1e-3, seed=5, dup_frac=0.2)
        big = synth.to_fasta(rows)
        small = _fasta(synth.random_strings(37, 1001, b"ACGT-", seed=6))[:-1]  # no final '\n'
        for name, fa in (("big.fasta", big), ("small.fasta", small)):
            p = tmp_path / name
            p.write_bytes(fa)
            a = c.alignment_from_fasta_file(str(p), remove_duplicates=True)
            b = c.alignment_from_fasta(fa, remove_duplicates=True)
            np.testing.assert_array_equal(c.pairwise_lt(a), c.pairwise_lt(b))
            np.testing.assert_array_equal(a.sequence_indices(), b.sequence_indices())
            a.free()
            b.free()
            ref = fa[fa.index(b"\n") + 1:].split(b"\n")[0]
            os.utime(p)  # a new modification time: read again
            np.testing.assert_array_equal(c.reference_distances_file(ref, str(p)),
                                          o.reference_distances(ref, fa))
        # the streamed from_fasta on the big file
        p = tmp_path / "big.fasta"
        st = os.stat(p)
        os.utime(p, ns=(st.st_atime_ns, st.st_mtime_ns + 1000))
        lt, aln = c.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
        b = c.alignment_from_fasta(big, remove_duplicates=True)
        np.testing.assert_array_equal(lt, c.pairwise_lt(b))
        aln.free()
        b.free()
    finally:
        c.close()
