"""from_fasta with the distances overlapping the read (hd_pairwise_lt_fasta_file):
for files of 64 MB or more the file is ingested in parts (by default split
after ~35% and ~65% of its bytes; HAMMINGDIST_STREAM_SPLITS sets up to
three),
and each part's complete tile rows run while the rest is read. Every result
must equal the plain order (read, ingest, distances) bit for bit: duplicates
that cross the parts, dtypes, max_distance, no dedupe, every split setting,
multi-line records (everywhere, or one in a later part), errors in a later
part, a file already on the device, and the module's from_fasta."""
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


@pytest.fixture(scope="module")
def big(tmp_path_factory):
    # 3,000 records x 29,903 sites = 90 MB, 30% duplicates of earlier rows
    rows, root, _ = synth.alignment(3000, 29903, p=1e-3, seed=41, dup_frac=0.3)
    fa = synth.to_fasta(rows)
    path = tmp_path_factory.mktemp("stream") / "big.fasta"
    path.write_bytes(fa)
    return str(path), fa, rows


def _plain(ctx, path, dtype, md, dedup):
    a = ctx.alignment_from_fasta(open(path, "rb").read(), remove_duplicates=dedup)
    lt = ctx.pairwise_lt(a, dtype=dtype, max_distance=md)
    idx = a.sequence_indices()
    a.free()
    return lt, idx


def _touch(path):
    import os
    import time

    st = time.time_ns()
    os.utime(path, ns=(st, st))


@pytest.mark.parametrize("dtype,md,dedup", [(np.uint8, 255, True), (np.uint16, 65535, True),
                                            (np.uint8, 7, False), (np.uint16, 300, False)])
def test_streamed_equals_plain(ctx, big, dtype, md, dedup):
    path, fa, rows = big
    _touch(path)  # not on the device: the overlapped order runs
    lt, aln = ctx.pairwise_lt_fasta_file(path, dtype=dtype, max_distance=md, remove_duplicates=dedup)
    want, want_idx = _plain(ctx, path, dtype, md, dedup)
    np.testing.assert_array_equal(lt, want)
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    assert aln.n_input == 3000
    aln.free()


def test_streamed_rows_against_oracle(ctx, big):
    path, fa, rows = big
    _touch(path)
    lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
    uniq = list(dict.fromkeys(r.tobytes() for r in rows))
    assert aln.n_rows == len(uniq)
    pick = np.array([0, 1, 2, len(uniq) // 3, len(uniq) // 2, len(uniq) - 2, len(uniq) - 1])
    want = o.lt_dense([uniq[i] for i in pick])
    got = [lt[pick[a] * (pick[a] - 1) // 2 + pick[b]] for a in range(len(pick)) for b in range(a)]
    np.testing.assert_array_equal(np.array(got, dtype=np.uint8), want)
    aln.free()


def test_already_on_device_and_reference_after(ctx, big):
    path, fa, rows = big
    _touch(path)
    lt1, a1 = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
    lt2, a2 = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)  # same file, on the device
    np.testing.assert_array_equal(lt1, lt2)
    ctx.trace(True)
    try:
        rd = ctx.reference_distances_file(rows[0].tobytes(), path)
        assert "file already on the device" in ctx.trace_last()
        assert "records already parsed" in ctx.trace_last()
    finally:
        ctx.trace(False)
    np.testing.assert_array_equal(rd, o.reference_distances(rows[0].tobytes(), fa))
    a1.free()
    a2.free()


@pytest.mark.parametrize("dedup", [True, False])
def test_reference_after_uses_resident_rows(ctx, big, dedup):
    # after the streamed call, fasta_reference_distances of the same file with
    # a reference of the records' length reads the rows that call packed; a
    # reference with '-', N, X, lowercase and other bytes, include_x, a longer
    # reference and a changed file take the records' bytes; every result
    # equals the oracle's
    path, fa, rows = big
    _touch(path)
    lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=dedup)
    aln.free()
    ref = bytearray(rows[5].tobytes())
    ref[0:40] = b"-" * 40
    ref[100:104] = b"NXac"
    ref[2000:2003] = b"*?-"
    ref = bytes(ref)
    ctx.trace(True)
    try:
        for r, ix, resident in ((ref, False, True), (rows[0].tobytes(), False, True),
                                (ref, True, False), (ref + b"A", False, False)):
            got = ctx.reference_distances_file(r, path, include_x=ix)
            assert ("from the resident rows" in ctx.trace_last()) == resident
            np.testing.assert_array_equal(got, o.reference_distances(r, fa, include_x=ix))
        _touch(path)  # changed: read and parsed again, the rows are gone
        got = ctx.reference_distances_file(ref, path)
        assert "from the resident rows" not in ctx.trace_last()
        np.testing.assert_array_equal(got, o.reference_distances(ref, fa))
    finally:
        ctx.trace(False)


def test_multiline_falls_back(ctx, tmp_path):
    rows, _, _ = synth.alignment(2500, 29903, p=1e-3, seed=42, dup_frac=0.2)
    out = bytearray()
    for k, r in enumerate(rows):
        out += b">s%d\n" % k
        for i in range(0, len(r), 6000):
            out += r[i:i + 6000].tobytes() + b"\n"
    p = tmp_path / "multi.fasta"
    p.write_bytes(bytes(out))
    lt, aln = ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    want, want_idx = _plain(ctx, str(p), np.uint8, 255, True)
    np.testing.assert_array_equal(lt, want)
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    aln.free()


@pytest.mark.parametrize("bad", [b"ACGT", b""])
def test_error_after_the_split(ctx, tmp_path, big, bad):
    from hammingdist_gb300 import abi

    path, fa, rows = big
    p = tmp_path / "bad.fasta"
    p.write_bytes(fa + b">late\n" + bad + b"\n" + fa[: 10 * 29916])
    with pytest.raises(abi.HDError, match="same length"):
        ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    # the context stays usable
    _touch(path)
    lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
    aln.free()


def test_module_from_fasta_uses_it(big):
    import hammingdist_gb300 as hd
    from hammingdist_gb300 import abi

    path, fa, rows = big
    _touch(path)
    ds = hd.from_fasta(path, use_gpu=True, remove_duplicates=True)
    big_ds = hd.from_fasta_large(path, use_gpu=True, remove_duplicates=True, max_distance=1000)
    c = abi.Context(0)
    try:
        want, want_idx = _plain(c, path, np.uint8, 255, True)
        want16, _ = _plain(c, path, np.uint16, 1000, True)
    finally:
        c.close()
    np.testing.assert_array_equal(np.asarray(ds.lt_array), want)
    np.testing.assert_array_equal(np.asarray(big_ds.lt_array), want16)


@pytest.mark.parametrize("where", [0.35, 0.8])
def test_multiline_record_in_a_later_part(ctx, tmp_path, monkeypatch, where):
    # the file is ingested in parts that end after 10%, 30% and 60% of its
    # bytes: one multi-line record in the third or fourth part, found after
    # earlier parts' distances have started, still gives the plain order's
    # results
    monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", "0.1,0.3,0.6")
    rows, _, _ = synth.alignment(2500, 29903, p=1e-3, seed=43, dup_frac=0.2)
    k0 = int(where * len(rows))
    out = bytearray()
    for k, r in enumerate(rows):
        out += b">s%d\n" % k
        if k == k0:
            out += r[:1000].tobytes() + b"\n" + r[1000:].tobytes() + b"\n"
        else:
            out += r.tobytes() + b"\n"
    p = tmp_path / "late_multi.fasta"
    p.write_bytes(bytes(out))
    lt, aln = ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    want, want_idx = _plain(ctx, str(p), np.uint8, 255, True)
    np.testing.assert_array_equal(lt, want)
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    aln.free()


@pytest.mark.parametrize("splits,where", [("0.1,0.3,0.6", 0.35), ("0.1,0.3,0.6", 0.7),
                                          ("", 0.45), ("", 0.7)])
def test_error_in_a_part(ctx, tmp_path, big, monkeypatch, splits, where):
    # a short record in the third or the fourth part (splits at 10%, 30% and
    # 60%), or in the second or the last part (the default splits, 35% and
    # 65%)
    from hammingdist_gb300 import abi

    if splits:
        monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", splits)

    path, fa, rows = big
    cut = fa.index(b"\n>", int(where * len(fa))) + 1  # a record header
    p = tmp_path / "bad2.fasta"
    p.write_bytes(fa[:cut] + b">short\nACGT\n" + fa[cut:])
    with pytest.raises(abi.HDError, match="same length"):
        ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    _touch(path)
    lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
    want, _ = _plain(ctx, path, np.uint8, 255, True)
    np.testing.assert_array_equal(lt, want)
    aln.free()


@pytest.mark.parametrize("n_rec,streamed", [(80_000, True), (5_000_000, False)])
def test_short_records(ctx, tmp_path, monkeypatch, n_rec, streamed):
    # records of 13 bytes (">\n", 10 sites, "\n") drawn from 1,000 distinct
    # rows. Streamed (the threshold lowered to 1 MB), with the parts' ends at
    # the headers of records 16,011 and 48,006: the 15 and 14 bytes before
    # them, which the next part is parsed from, hold a '\n' (and the '>') and
    # then the whole previous record, which must not be counted twice.
    # 5,000,000 records (65 MB): buffers sized for every record to be unique
    # would not fit, so the plain order runs
    rec_bytes = 13
    n = n_rec * rec_bytes
    if streamed:
        monkeypatch.setenv("HAMMINGDIST_STREAM_MIN_BYTES", "1000000")
        ends = [(rec_bytes * k - 5) / n for k in (16_011, 48_006)]
        assert [(rec_bytes * k) % 16 for k in (16_011, 48_006)] == [15, 14]
        monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", ",".join("%.9f" % f for f in ends))
    rng = np.random.default_rng(99)
    acgt = np.frombuffer(b"ACGT-N", np.uint8)
    distinct = acgt[rng.integers(0, 6, (1000, 10))]
    pick = rng.integers(0, 1000, n_rec)
    recs = np.empty((n_rec, rec_bytes), np.uint8)
    recs[:, 0:2] = np.frombuffer(b">\n", np.uint8)
    recs[:, 2:12] = distinct[pick]
    recs[:, 12] = ord("\n")
    p = tmp_path / "short.fasta"
    p.write_bytes(recs.tobytes())
    lt, aln = ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    want, want_idx = _plain(ctx, str(p), np.uint8, 255, True)
    assert aln.n_input == n_rec
    assert aln.n_rows == len({distinct[k].tobytes() for k in np.unique(pick)})
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    np.testing.assert_array_equal(lt, want)
    aln.free()


@pytest.mark.parametrize("splits", ["", "0.5", "0.2,0.5", "0.25,0.5,0.75", "0.9"])
def test_every_split_setting(ctx, big, monkeypatch, splits):
    # no split (one part), one, two and three splits (the default is two:
    # 35%, 65%): the same matrix and sequence indices as the plain order
    path, fa, rows = big
    monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", splits)
    _touch(path)
    lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
    want, want_idx = _plain(ctx, path, np.uint8, 255, True)
    np.testing.assert_array_equal(lt, want)
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    aln.free()


@pytest.mark.parametrize("where", [0.3, 0.6])
def test_multiline_record_with_three_splits(ctx, tmp_path, monkeypatch, where):
    # one multi-line record in the second or third of four parts
    monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", "0.25,0.5,0.75")
    rows, _, _ = synth.alignment(2500, 29903, p=1e-3, seed=44, dup_frac=0.2)
    k0 = int(where * len(rows))
    out = bytearray()
    for k, r in enumerate(rows):
        out += b">s%d\n" % k
        if k == k0:
            out += r[:1000].tobytes() + b"\n" + r[1000:].tobytes() + b"\n"
        else:
            out += r.tobytes() + b"\n"
    p = tmp_path / "late_multi3.fasta"
    p.write_bytes(bytes(out))
    lt, aln = ctx.pairwise_lt_fasta_file(str(p), remove_duplicates=True)
    want, want_idx = _plain(ctx, str(p), np.uint8, 255, True)
    np.testing.assert_array_equal(lt, want)
    np.testing.assert_array_equal(aln.sequence_indices(), want_idx)
    aln.free()


def test_mirror_copy(ctx, big, tmp_path):
    # HD_OUTPUT_MIRROR: a second copy of the result written while the
    # distances run, on the streamed path and on a small file's plain order
    path, fa, rows = big
    _touch(path)
    lt, aln, mirror = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True, mirror=True)
    np.testing.assert_array_equal(mirror, lt)
    assert mirror.ctypes.data != lt.ctypes.data
    aln.free()
    small = tmp_path / "small.fasta"
    small.write_bytes(synth.to_fasta(rows[:300]))
    lt, aln, mirror = ctx.pairwise_lt_fasta_file(str(small), dtype=np.uint16, mirror=True)
    np.testing.assert_array_equal(mirror, lt)
    aln.free()


def test_module_first_lt_array_is_a_fresh_copy(big):
    # the first lt_array access hands out the copy written during the call;
    # every access is still a fresh array that aliases neither the DataSet
    # nor another access
    import hammingdist_gb300 as hd

    path, fa, rows = big
    _touch(path)
    ds = hd.from_fasta(path, use_gpu=True, remove_duplicates=True)
    a = np.asarray(ds.lt_array)
    b = np.asarray(ds.lt_array)
    np.testing.assert_array_equal(a, b)
    a[:] = 7
    c = np.asarray(ds.lt_array)
    np.testing.assert_array_equal(b, c)
    assert ds[1, 0] == int(b[0])


@pytest.mark.parametrize("splits", ["0.2,0.5", "0.25,0.5,0.75"])
def test_incremental_and_full_dedupe_agree(ctx, big, monkeypatch, splits):
    # each part's new records only (the default), and the full dedupe of the
    # prefix that a hash collision falls back to (HAMMINGDIST_STREAM_DEDUPE=full)
    path, fa, rows = big
    monkeypatch.setenv("HAMMINGDIST_STREAM_SPLITS", splits)
    got = {}
    for mode in ("", "full"):
        monkeypatch.setenv("HAMMINGDIST_STREAM_DEDUPE", mode)
        _touch(path)
        lt, aln = ctx.pairwise_lt_fasta_file(path, remove_duplicates=True)
        got[mode] = (lt, aln.sequence_indices())
        aln.free()
    want, want_idx = _plain(ctx, path, np.uint8, 255, True)
    for lt, idx in got.values():
        np.testing.assert_array_equal(lt, want)
        np.testing.assert_array_equal(idx, want_idx)
