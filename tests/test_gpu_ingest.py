"""Device ingest at every record alignment: record starts at all 16 byte
offsets (headers of varying length), lengths at 16/512/1024-byte edges,
duplicates and near-duplicates that differ in the first, a middle or the last
byte only, single- and multi-line records; sequence indices, unique rows and
distances must equal the oracle's read_fasta/dedupe and dense rule."""
import numpy as np
import pytest

from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from hammingdist_gb300 import abi

    c = abi.Context(0)
    yield c
    c.close()


def _records(L, seed, n_base=24):
    rng = np.random.default_rng(seed)
    base = [bytes(rng.choice(list(b"ACGT-N"), size=L).astype(np.uint8)) for _ in range(n_base)]
    recs = []
    for k, s in enumerate(base):
        recs.append(s)
        if k % 3 == 0:
            recs.append(s)  # exact duplicate
        for pos in (0, L // 2, L - 1):
            if k % 4 == (pos % 4):
                t = bytearray(s)
                t[pos] = ord("A") if t[pos] != ord("A") else ord("C")
                recs.append(bytes(t))  # near-duplicate: one byte differs
    rng.shuffle(recs)
    return recs


def _fasta(recs, multiline=False, width=61):
    out = bytearray()
    for k, s in enumerate(recs):
        out += b">" + b"h" * (k % 16) + b"\n"  # header lengths 2..17: every start offset mod 16
        if multiline:
            for i in range(0, len(s), width):
                out += s[i:i + width] + b"\n"
        else:
            out += s + b"\n"
    return bytes(out)


@pytest.mark.parametrize("L", [1, 15, 16, 17, 511, 512, 513, 1023, 1024, 1025, 3001])
@pytest.mark.parametrize("multiline", [False, True])
def test_dedupe_and_pack_all_alignments(ctx, L, multiline):
    recs = _records(L, seed=L * 7 + multiline)
    fa = _fasta(recs, multiline)
    want_lt, want_idx = o.from_fasta_dense(fa, remove_duplicates=True)
    a = ctx.alignment_from_fasta(fa, remove_duplicates=True)
    np.testing.assert_array_equal(a.sequence_indices(), want_idx)
    np.testing.assert_array_equal(ctx.pairwise_lt(a), want_lt)
    np.testing.assert_array_equal(ctx.fasta_sequence_indices(fa), o.fasta_sequence_indices(fa))
    a.free()


def test_unaligned_device_input(ctx):
    # FASTA bytes handed over at an odd device offset are staged; at a
    # 16-byte aligned offset they are read in place, up to their last byte
    torch = pytest.importorskip("torch")
    recs = _records(777, seed=5)
    fa = _fasta(recs)
    want_lt, want_idx = o.from_fasta_dense(fa, remove_duplicates=True)
    buf = torch.zeros(len(fa) + 64, dtype=torch.uint8, device="cuda:0")
    for shift in (0, 3, 16):
        buf[shift:shift + len(fa)] = torch.frombuffer(bytearray(fa), dtype=torch.uint8).cuda()
        torch.cuda.synchronize()
        a = ctx.alignment_from_fasta(buf.data_ptr() + shift, len(fa), on_device=True,
                                     remove_duplicates=True)
        np.testing.assert_array_equal(a.sequence_indices(), want_idx)
        np.testing.assert_array_equal(ctx.pairwise_lt(a), want_lt)
        a.free()
