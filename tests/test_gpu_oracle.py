"""The GPU path against the oracle (oracle/hd_oracle.c) on seeded inputs:
tile and word boundaries, long rows, the benchmark generator's shape, every
output dtype, both semantics, through the C ABI and through the module."""
import numpy as np
import pytest

from gpu_util import seqidx_of, write
from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu
hd = pytest.importorskip("hammingdist_gb300")


@pytest.fixture(scope="module")
def ctx():
    from hammingdist_gb300 import abi

    c = abi.Context(0)
    yield c
    c.close()


# n around the 128-row tile, L around the 32-site word and 256-site stage
SIZES = [(2, 1), (3, 31), (5, 32), (7, 33), (127, 255), (128, 256), (129, 257), (130, 1023),
         (255, 1025), (256, 100), (257, 29), (300, 513), (384, 64), (513, 77)]


@pytest.mark.parametrize("n,L", SIZES)
def test_pairwise_sizes_abi(ctx, n, L):
    from hammingdist_gb300 import abi

    seqs = synth.random_strings(n, L, b"ACGT-N*X", seed=n * 1000 + L)
    fa = b"".join(b">s\n" + s + b"\n" for s in seqs)
    aln = ctx.alignment_from_fasta(fa, semantics=abi.SEM_GPU)
    assert (aln.n_rows, aln.length, aln.rule) == (n, L, "and")
    for dtype, md in ((np.uint8, 255), (np.uint8, 3), (np.uint16, 65535), (np.uint16, 40),
                      (np.uint32, 10 ** 9)):
        got = ctx.pairwise_lt(aln, dtype=dtype, max_distance=md)
        want = o.lt_dense(seqs, max_distance=md, dtype=dtype if dtype != np.uint32 else np.uint32)
        np.testing.assert_array_equal(got, want, err_msg=f"n={n} L={L} {dtype} md={md}")


@pytest.mark.parametrize("L", [65537, 262145, 1048577])
def test_long_rows(ctx, L):
    seqs = synth.random_strings(4, L, b"ACGT-", seed=L)
    seqs.append(b"A" * L)
    seqs.append(b"G" * L)
    aln = ctx.alignment_from_sequences(seqs)
    for md in (0, 11, 999, 9876544):
        got = ctx.pairwise_lt(aln, dtype=np.uint32, max_distance=md)
        want = o.lt_dense(seqs, max_distance=md, dtype=np.uint32)
        np.testing.assert_array_equal(got, want)
    # identical rows -> 0; all-A vs all-G -> L
    assert ctx.pairwise_lt(aln, dtype=np.uint32, max_distance=10 ** 9)[-1] == L


def test_benchmark_shape_n1000(tmp_path):
    """The n=1,000, L=29,903 workload: dense uint8 lt_array, parity with the
    oracle's dense path, also with duplicates and both dtypes."""
    rows, root, _ = synth.alignment(1000, 29903, p=1e-3, seed=11, dup_frac=0.3)
    fa = synth.to_fasta(rows)
    path = write(tmp_path, "b.fasta", fa)
    for dedup in (False, True):
        ds = hd.from_fasta(path, remove_duplicates=dedup, use_gpu=True)
        want, idx = o.from_fasta_dense(fa, remove_duplicates=dedup)
        np.testing.assert_array_equal(np.asarray(ds.lt_array), want)
        if dedup:
            np.testing.assert_array_equal(seqidx_of(ds, tmp_path), idx)
        # use_gpu=False: the reference CPU takes its dense branch on this input
        ds2 = hd.from_fasta(path, remove_duplicates=dedup, use_gpu=False)
        np.testing.assert_array_equal(np.asarray(ds2.lt_array), want)
    ds16 = hd.from_fasta_large(path, use_gpu=True, max_distance=70)
    np.testing.assert_array_equal(np.asarray(ds16.lt_array),
                                  o.from_fasta_dense(fa, max_distance=70, dtype=np.uint16)[0])


def test_sparse_rule_semantics(tmp_path):
    """use_gpu=False on low-diversity input and with include_x: the sparse
    rule, against the oracle's literal restatement of the reference's sparse
    algorithm."""
    for k, (n, L, p, dash, nrate) in enumerate([(150, 4000, 1e-4, 10, 0.0),
                                                (200, 3000, 2e-4, 5, 5e-5),
                                                (140, 999, 1e-2, 50, 1e-3)]):
        rows, _, _ = synth.alignment(n, L, p=p, seed=40 + k, dash_max=dash, n_rate=nrate)
        rows[::7, ::13] = ord("X")
        seqs = [r.tobytes() for r in rows]
        path = write(tmp_path, "s.fasta", synth.to_fasta(rows))
        for x in (False, True):
            for large in (False, True):
                fn = hd.from_fasta_large if large else hd.from_fasta
                dt = np.uint16 if large else np.uint8
                for md in (2, 255, 65535):
                    got = np.asarray(fn(path, include_x=x, use_gpu=False, max_distance=md).lt_array)
                    want, used_sparse = o.lt_cpu(seqs, include_x=x, max_distance=md, dtype=dt)
                    np.testing.assert_array_equal(got, want, err_msg=f"case {k} x={x} md={md}")


def test_reference_distances_oracle(tmp_path):
    rows, root, _ = synth.alignment(2000, 29903, p=1e-3, seed=12, dup_frac=0.3)
    rows[5, 100:140] = ord("X")
    fa = synth.to_fasta(rows)
    path = write(tmp_path, "r.fasta", fa)
    for x in (False, True):
        got = hd.fasta_reference_distances(root.tobytes().decode(), path, include_x=x)
        np.testing.assert_array_equal(got, o.reference_distances(root.tobytes(), fa, x))
    np.testing.assert_array_equal(hd.fasta_sequence_indices(path), o.fasta_sequence_indices(fa))
    np.testing.assert_array_equal(hd.fasta_sequence_indices(path, n=777),
                                  o.fasta_sequence_indices(fa, 777))


def test_reference_distances_ragged(tmp_path):
    """Records of lengths 1 to past two 4,096-site segments, starting at every
    byte position within 16-byte blocks of the file, against a longer
    reference: each count runs over the record's own length."""
    rng = np.random.default_rng(21)
    alphabet = np.frombuffer(b"ACGT-NXacgt*-", dtype=np.uint8)
    ref = alphabet[rng.integers(0, 5, 9001)].tobytes()  # A, C, G, T, -
    recs = []
    for k in range(300):
        n = k + 1 if k < 40 else int(rng.integers(1, 9002))
        r = bytearray(ref[:n])
        for f in rng.integers(0, n, size=n // 40 + 1):
            r[f] = alphabet[rng.integers(0, len(alphabet))]
        recs.append(bytes(r))
    # names of varying length move each record's start within 16-byte blocks
    fa = b"".join(b">r%d%s\n" % (i, b"x" * (i % 17)) + r + b"\n" for i, r in enumerate(recs))
    path = write(tmp_path, "ragged.fasta", fa)
    for x in (False, True):
        got = hd.fasta_reference_distances(ref.decode(), path, include_x=x)
        np.testing.assert_array_equal(got, o.reference_distances(ref, fa, x))


def test_resident_alignment_queries(ctx):
    rows, root, _ = synth.alignment(600, 2999, p=1e-3, seed=13, dup_frac=0.3)
    fa = synth.to_fasta(rows)
    aln = ctx.alignment_from_fasta(fa, remove_duplicates=True)
    for q in (root.tobytes(), rows[3].tobytes()):
        np.testing.assert_array_equal(ctx.alignment_reference_distances(aln, q),
                                      o.reference_distances(q, fa))


def test_multiline_and_crlf_records(tmp_path):
    rng = np.random.default_rng(3)
    seqs = synth.random_strings(60, 250, b"ACGT-N", seed=4)
    parts = []
    for i, s in enumerate(seqs):
        parts.append(b">r%d\n" % i)
        cuts = sorted(rng.integers(0, 250, 3).tolist())
        prev = 0
        for c in cuts + [250]:
            parts.append(s[prev:c] + b"\n")
            prev = c
        if i % 5 == 0:
            parts.append(b"\n")
    fa = b"".join(parts)
    path = write(tmp_path, "m.fasta", fa)
    for dedup in (False, True):
        ds = hd.from_fasta(path, remove_duplicates=dedup, use_gpu=True)
        np.testing.assert_array_equal(np.asarray(ds.lt_array),
                                      o.from_fasta_dense(fa, remove_duplicates=dedup)[0])


def test_launches_and_device_output(ctx, monkeypatch):
    import torch

    # 200 rows: the tensor-core engine only when its item threshold is off
    monkeypatch.setenv("HAMMINGDIST_MMA_MIN_ITEMS", "0")
    seqs = synth.random_strings(200, 300, b"ACGT-", seed=9)
    aln = ctx.alignment_from_sequences(seqs)
    n = aln.n_rows
    before = ctx.kernel_launches
    out = torch.empty(n * (n - 1) // 2, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    ctx.pairwise_lt(aln, dtype=np.uint8, max_distance=255, out=out.data_ptr(), out_on_device=True)
    assert ctx.kernel_launches > before
    np.testing.assert_array_equal(out.cpu().numpy(), o.lt_dense(seqs))
    # the tensor-core engine: 128-row x 240-column tiles, a short list split
    # into single row tiles, each with the column tiles its rows reach
    ms, tiles = ctx.last_pairwise_timing()
    nb = -(-n // 128)
    assert ms > 0 and tiles == sum((128 * (i + 1) - 2) // 240 + 1 for i in range(nb))
    # the bit-plane engine: square tiles of the autotuned edge
    import os

    os.environ["HAMMINGDIST_KERNEL"] = "lop3"
    try:
        out.zero_()
        ctx.pairwise_lt(aln, dtype=np.uint8, max_distance=255, out=out.data_ptr(),
                        out_on_device=True)
    finally:
        del os.environ["HAMMINGDIST_KERNEL"]
    np.testing.assert_array_equal(out.cpu().numpy(), o.lt_dense(seqs))
    ms, tiles = ctx.last_pairwise_timing()
    tile, _ = ctx.tune_lookup(n, 300, np.uint8)
    nb = -(-n // tile)
    assert ms > 0 and tiles == nb * (nb + 1) // 2


def test_errors(ctx, tmp_path):
    from hammingdist_gb300 import abi

    with pytest.raises(RuntimeError, match="Failed to open file"):
        hd.from_fasta(str(tmp_path / "missing.fasta"))
    with pytest.raises(RuntimeError, match="Failed to open file"):
        hd.fasta_reference_distances("ACGT", str(tmp_path / "missing.fasta"))
    with pytest.raises(RuntimeError, match="Sequences do not all have the same length"):
        hd.distance("ACGT", "ACG")
    with pytest.raises(abi.HDError) as e:
        ctx.alignment_from_sequences([b"ACGT", b"AC"])
    assert e.value.code == -2
    with pytest.raises(abi.HDError) as e:
        ctx.alignment_from_sequences([b"", b""])
    assert e.value.code == -1
    with pytest.raises(abi.HDError) as e:
        ctx.alignment_from_sequences([b"ACGT", b"ACGA"], include_x=True, semantics=abi.SEM_GPU)
    assert e.value.code == -6
    p = write(tmp_path, "r.fasta", b">a\nACGTACGT\n")
    with pytest.raises(RuntimeError, match="longer than the reference"):
        hd.fasta_reference_distances("ACG", p)
    p = write(tmp_path, "lt.fasta", b">a\nACGT\n>b\nACGA\n")
    with pytest.raises(RuntimeError, match="only available on GPU"):
        hd.from_fasta_to_lower_triangular(p, str(tmp_path / "o.txt"), use_gpu=False)
