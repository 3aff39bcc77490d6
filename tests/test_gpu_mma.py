"""The tensor-core engine (hd_mma.cu: block-scaled FP4 tcgen05 MMAs,
matches = <planes> - (P - 1) <dash>)
against the bit-plane engine (HAMMINGDIST_KERNEL=lop3) and the oracle, bit
for bit: lengths at and around the 32/256-site blocks, row counts around the
128 x 240 tiles, every dtype and saturation, '-' against '-', N and other
bytes, the row ranges of the text writer and views."""
import os

import numpy as np
import pytest

from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _every_size(monkeypatch):
    # small matrices too: by default a launch with few items takes the
    # bit-plane engine (HAMMINGDIST_MMA_MIN_ITEMS)
    monkeypatch.setenv("HAMMINGDIST_MMA_MIN_ITEMS", "0")


@pytest.fixture(scope="module")
def ctx():
    from hammingdist_gb300 import abi

    c = abi.Context(0)
    yield c
    c.close()


def _both(ctx, aln, **kw):
    os.environ["HAMMINGDIST_KERNEL"] = "lop3"
    try:
        want = ctx.pairwise_lt(aln, **kw)
    finally:
        del os.environ["HAMMINGDIST_KERNEL"]
    got = ctx.pairwise_lt(aln, **kw)
    return got, want


@pytest.mark.parametrize("n,L", [(2, 1), (3, 33), (5, 127), (17, 128), (129, 129), (255, 257),
                                 (256, 1000), (257, 513), (300, 5000), (130, 29903), (224, 256),
                                 (225, 255), (449, 511), (448, 769), (240, 300), (241, 64),
                                 (481, 1000), (480, 257), (719, 2049)])
def test_mma_equals_lop3_and_oracle(ctx, n, L):
    seqs = synth.random_strings(n, L, b"ACGT-N", seed=n * 7 + L)
    aln = ctx.alignment_from_sequences(seqs)
    got, want = _both(ctx, aln)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, o.lt_dense(seqs))
    aln.free()


@pytest.mark.parametrize("dtype,md", [(np.uint8, 255), (np.uint8, 3), (np.uint16, 65535),
                                      (np.uint16, 200), (np.uint32, 2**32 - 1)])
def test_mma_dtypes_and_saturation(ctx, dtype, md):
    rows, _, _ = synth.alignment(700, 3001, p=5e-2, seed=5, dup_frac=0.0, dash_max=300)
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs)
    got, want = _both(ctx, aln, dtype=dtype, max_distance=md)
    np.testing.assert_array_equal(got, want)
    aln.free()


def test_mma_dashes_and_other_bytes(ctx):
    # '-' against '-' (plane dot 4, minus 3), N, X, lowercase and other
    # bytes (code 0: never match), long dash runs
    rng = np.random.default_rng(9)
    alphabet = np.frombuffer(b"ACGT-NXacgt*?-----", dtype=np.uint8)
    seqs = [alphabet[rng.integers(0, len(alphabet), 2000)].tobytes() for _ in range(300)]
    seqs.append(b"-" * 2000)
    seqs.append(b"N" * 2000)
    aln = ctx.alignment_from_sequences(seqs)
    got, want = _both(ctx, aln)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, o.lt_dense(seqs))
    aln.free()


def test_mma_larger(ctx):
    rows, _, _ = synth.alignment(3000, 29903, p=1e-3, seed=11, dup_frac=0.0)
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs)
    got, want = _both(ctx, aln)
    np.testing.assert_array_equal(got, want)
    pick = np.array([0, 1, 2, 127, 128, 255, 256, 257, 1500, 2998, 2999])
    sub = o.lt_dense([seqs[i] for i in pick])
    g = [got[pick[a] * (pick[a] - 1) // 2 + pick[b]] for a in range(len(pick)) for b in range(a)]
    np.testing.assert_array_equal(np.array(g, dtype=np.uint8), sub)
    aln.free()


@pytest.mark.parametrize("include_x", [False, True])
@pytest.mark.parametrize("n,L", [(3, 100), (129, 1000), (300, 2999), (700, 29903)])
def test_mma_sparse_rules(ctx, include_x, n, L):
    # use_gpu=False semantics on low-diversity rows: the reference CPU takes
    # the sparse rule (5 planes, or 6 with include_x); on the tensor cores
    # match = <planes> - (P - 1) [dash][dash]
    from hammingdist_gb300 import abi

    rows, _, _ = synth.alignment(n, L, p=1e-4, seed=n + L, dash_max=min(10, L // 20),
                                 n_rate=0.0)
    rows[::50, ::101] = ord("X")
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs, include_x=include_x, semantics=abi.SEM_CPU)
    want_lt, used_sparse = o.lt_cpu(seqs, include_x=include_x)
    # the heuristic's choice is the reference's; with include_x it is always sparse
    assert (aln.rule != "and") == used_sparse and (used_sparse or not include_x)
    if used_sparse:
        assert aln.rule == ("sparse_x" if include_x else "sparse")
    for dtype, md in ((np.uint8, 255), (np.uint16, 65535), (np.uint8, 2)):
        got, want = _both(ctx, aln, dtype=dtype, max_distance=md)
        np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(_both(ctx, aln)[0], want_lt)
    aln.free()


@pytest.mark.parametrize("row0,n", [(0, 300), (1, 257), (127, 129), (128, 400), (300, 2)])
def test_mma_views(ctx, row0, n):
    # windows of a resident alignment (serving): the window's rows are
    # expanded into an operand of their own, at any row offset
    from hammingdist_gb300 import abi

    rows, _, _ = synth.alignment(800, 2999, p=1e-3, seed=31, dash_max=60)
    seqs = [r.tobytes() for r in rows]
    base = ctx.alignment_from_sequences(seqs)
    v = base.view(row0, n)
    got, want = _both(ctx, v)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, o.lt_dense(seqs[row0:row0 + n]))
    v.free()
    base.free()
    # a sparse-rule base
    sp = ctx.alignment_from_sequences(seqs, include_x=True, semantics=abi.SEM_CPU)
    v = sp.view(row0, n)
    got, want = _both(ctx, v, dtype=np.uint16, max_distance=65535)
    np.testing.assert_array_equal(got, want)
    v.free()
    sp.free()


def _cap_rows(L, rng, mixed, n=130):
    """n rows of length L whose match counts reach the length: one root with a
    few substitutions and '-' runs at both ends ('-' against '-' carries the
    largest plane products); with `mixed`, long '-' runs, rows all '-', rows
    all 'N' (distance L under the AND rule) and rows over ACGT-N; without, a
    low-diversity set (under 0.5% of sites off the consensus), on which the
    reference CPU takes its sparse rule."""
    acgt = np.frombuffer(b"ACGT", np.uint8)
    root = acgt[rng.integers(0, 4, L)]
    rows = []
    for k in range(n):
        if k < 100 or not mixed:
            r = root.copy()
            pos = rng.integers(0, L, 80)
            r[pos] = acgt[rng.integers(0, 4, pos.size)]
            a, b = rng.integers(0, L // 4 if mixed else L // 1000, 2)
            r[:a] = ord("-")
            r[L - b:] = ord("-")
            if k % 10 == 3:
                r[rng.integers(0, L, 40)] = ord("X")
        elif k < 110:
            r = np.full(L, ord("-"), np.uint8)
        elif k < 115:
            r = np.full(L, ord("N"), np.uint8)
        else:
            r = np.frombuffer(b"ACGT-N", np.uint8)[rng.integers(0, 6, L)]
        rows.append(r.tobytes())
    return rows


@pytest.mark.parametrize("planes,L", [(4, 4_194_303), (5, 3_355_443), (6, 2_796_202)])
def test_mma_exact_at_length_cap(ctx, planes, L):
    # the engine takes alignments with P L < 2^24 (hd_mma.cu mma_eligible):
    # at the largest such L, 130 rows (a full 128-row tile and part of the
    # next), match counts near L and distances up to L in uint32 must equal
    # the bit-plane engine's integer counts and the oracle's
    from hammingdist_gb300 import abi

    assert planes * L < 2**24 and planes * (L + 1) >= 2**24
    seqs = _cap_rows(L, np.random.default_rng(planes), mixed=planes != 5)
    if planes == 4:
        aln = ctx.alignment_from_sequences(seqs)
    else:
        aln = ctx.alignment_from_sequences(seqs, include_x=planes == 6, semantics=abi.SEM_CPU)
    assert aln.rule == {4: "and", 5: "sparse", 6: "sparse_x"}[planes]
    got, want = _both(ctx, aln, dtype=np.uint32, max_distance=2**32 - 1)
    np.testing.assert_array_equal(got, want)
    if planes == 4:
        assert got.max() == L  # an 'N' row against an all-'-' row
    pick = [0, 1, 57, 99, 100, 110, 120, 129] if planes != 5 else [0, 1, 57, 98, 99, 129]
    sub = [seqs[i] for i in pick]
    g = np.array([got[pick[a] * (pick[a] - 1) // 2 + pick[b]]
                  for a in range(len(pick)) for b in range(a)], dtype=np.uint32)
    if planes == 4:
        # the oracle's max_dist is a C int, as in the reference
        np.testing.assert_array_equal(g, o.lt_dense(sub, max_distance=2**31 - 1, dtype=np.uint32))
    else:
        # the reference CPU's DataSet types end at uint16
        ref, sparse = o.lt_cpu(sub, include_x=planes == 6, max_distance=65535, dtype=np.uint16)
        assert sparse
        np.testing.assert_array_equal(np.minimum(g, 65535), ref)
    aln.free()


@pytest.mark.parametrize("schedule", ["static", "queue"])
def test_mma_schedules(ctx, monkeypatch, schedule):
    # both work distributions of the tensor-core engine (round-robin items,
    # or items drawn from the launch's queue), on one matrix and on a batch
    # of matrices of unequal row length, bit for bit against the oracle
    monkeypatch.setenv("HAMMINGDIST_MMA_SCHEDULE", schedule)
    rows, _, _ = synth.alignment(1200, 4001, p=2e-3, seed=77, dash_max=100)
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs)
    np.testing.assert_array_equal(ctx.pairwise_lt(aln), o.lt_dense(seqs))
    inputs = [synth.random_strings(n, L, b"ACGT-N", seed=n + L)
              for n, L in ((300, 5000), (129, 257), (700, 333), (450, 2999), (2, 33))]
    alns = [ctx.alignment_from_sequences(s) for s in inputs]
    b = ctx.batch()
    for a in alns:
        b.add(a, dtype=np.uint16, max_distance=65535)
    for rep in range(2):  # the second run replays the captured graph
        for got, s in zip(b.run(), inputs):
            np.testing.assert_array_equal(got, o.lt_dense(s, max_distance=65535, dtype=np.uint16))
    b.free()
    for a in alns + [aln]:
        a.free()


def test_mma_dash_chunks(ctx):
    # the dash products run only for the 256-site chunks where some row has a
    # '-': a single '-' in one middle chunk of one row, '-' runs that end
    # exactly on chunk boundaries, rows without any '-', and windows of the
    # alignment (a window at row 0 shares the whole alignment's marks; a
    # window elsewhere marks its own rows' chunks)
    from hammingdist_gb300 import abi

    rng = np.random.default_rng(17)
    L = 256 * 9 + 17
    acgt = np.frombuffer(b"ACGT", np.uint8)
    rows = [acgt[rng.integers(0, 4, L)] for _ in range(400)]
    rows[3][256 * 4 + 100] = ord("-")
    rows[250][: 256 * 2] = ord("-")
    rows[251][256 * 7:] = ord("-")
    rows[399][256 * 5 + 255] = ord("-")
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs)
    got, want = _both(ctx, aln, dtype=np.uint16, max_distance=65535)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, o.lt_dense(seqs, max_distance=65535, dtype=np.uint16))
    for row0, n in ((0, 260), (200, 150), (240, 160)):
        v = aln.view(row0, n)
        got, want = _both(ctx, v)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(got, o.lt_dense(seqs[row0:row0 + n]))
        v.free()
    aln.free()
    # the sparse rules (5 and 6 planes) on the same rows
    for include_x in (False, True):
        sp = ctx.alignment_from_sequences(seqs, include_x=include_x, semantics=abi.SEM_CPU)
        got, want = _both(ctx, sp, dtype=np.uint16, max_distance=65535)
        np.testing.assert_array_equal(got, want)
        sp.free()
