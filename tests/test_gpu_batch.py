"""The persistent engine on batches of independent matrices, its CUDA-graph
replay, every kernel configuration the autotuner can pick, and
from_fasta_batch against per-file from_fasta. All checks are bit-exact
against the oracle or the single-matrix path."""
import json
import os

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


def _mixed_inputs():
    shapes = [(1, 40), (2, 17), (50, 1000), (129, 257), (300, 5000), (700, 333), (64, 65),
              (1000, 2999)]
    out = []
    for k, (n, L) in enumerate(shapes):
        seqs = synth.random_strings(n, L, b"ACGT-N", seed=500 + k)
        out.append(seqs)
    return out


def test_batch_matches_single_and_oracle(ctx):
    import torch

    inputs = _mixed_inputs()
    alns = [ctx.alignment_from_sequences(s) for s in inputs]
    b = ctx.batch()
    specs = []
    for k, (a, seqs) in enumerate(zip(alns, inputs)):
        dt = np.uint16 if k % 2 else np.uint8
        md = [255, 65535, 3, 89, 0, 497, 255, 65535][k]
        specs.append((dt, md))
        b.add(a, dtype=dt, max_distance=md)
    # one job with a device output
    n_dev = alns[5].n_rows
    d_out = torch.zeros(n_dev * (n_dev - 1) // 2 * 2, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    b.add(alns[5], dtype=np.uint16, max_distance=777, out=d_out.data_ptr(), out_on_device=True)
    for rep in range(2):  # second run replays the captured graph
        outs = b.run()
        for k, seqs in enumerate(inputs):
            dt, md = specs[k]
            want = o.lt_dense(seqs, max_distance=md, dtype=dt) if len(seqs) > 1 else np.zeros(0, dt)
            np.testing.assert_array_equal(outs[k], want, err_msg=f"job {k} rep {rep}")
            np.testing.assert_array_equal(ctx.pairwise_lt(alns[k], dtype=dt, max_distance=md), want)
        got = d_out.cpu().numpy().view(np.uint16)
        np.testing.assert_array_equal(got, o.lt_dense(inputs[5], max_distance=777, dtype=np.uint16))
    ms, launches, tiles = b.timing()
    assert ms > 0 and launches >= 1 and tiles > 0
    b.free()


def test_batch_sparse_rule_jobs(ctx):
    from hammingdist_gb300 import abi

    rows, _, _ = synth.alignment(150, 3000, p=1e-4, seed=61, dash_max=5)
    rows[::30, ::300] = ord("X")
    seqs = [r.tobytes() for r in rows]
    # the reference heuristic (restated by the oracle) picks the rule
    assert o.lt_cpu(seqs, include_x=False)[1], "input meant to be low-diversity"
    b = ctx.batch()
    a_x = ctx.alignment_from_sequences(seqs, include_x=True, semantics=abi.SEM_CPU)
    a_s = ctx.alignment_from_sequences(seqs, include_x=False, semantics=abi.SEM_CPU)
    assert a_x.rule == "sparse_x" and a_s.rule == "sparse"
    b.add(a_x, dtype=np.uint8, max_distance=255)
    b.add(a_s, dtype=np.uint16, max_distance=65535)
    outs = b.run()
    np.testing.assert_array_equal(outs[0], o.lt_cpu(seqs, include_x=True, max_distance=255)[0])
    np.testing.assert_array_equal(outs[1], o.lt_cpu(seqs, include_x=False, max_distance=65535,
                                                    dtype=np.uint16)[0])


@pytest.mark.parametrize("tile,stages", [(128, 3), (128, 2), (128, 4), (64, 3), (64, 4)])
def test_every_kernel_configuration(ctx, tmp_path, tile, stages):
    """A tuning table that maps every bucket to one configuration: results are
    the same bit for bit."""
    entries = [{"n_bucket": nb, "L_bucket": lb, "dtype": dt, "tile": tile, "stages": stages}
               for nb in range(7) for lb in range(4) for dt in (1, 2)]
    path = str(tmp_path / "tune.json")
    with open(path, "w") as f:
        json.dump({"device": "test", "entries": entries}, f)
    ctx.tune_load(path)
    try:
        assert ctx.tune_lookup(300, 1000, np.uint8) == (tile, stages)
        for k, (n, L) in enumerate([(2, 5), (65, 300), (200, 4097), (513, 64)]):
            seqs = synth.random_strings(n, L, b"ACGT-NX", seed=900 + k)
            aln = ctx.alignment_from_sequences(seqs)
            for dt, md in ((np.uint8, 255), (np.uint16, 40)):
                np.testing.assert_array_equal(ctx.pairwise_lt(aln, dtype=dt, max_distance=md),
                                              o.lt_dense(seqs, max_distance=md, dtype=dt))
    finally:
        with open(path, "w") as f:
            json.dump({"entries": []}, f)
        ctx.tune_load(path)  # back to the built-in choice


@pytest.mark.parametrize("band,rows", [(8, 2), (16, 2), (32, 2), (16, 1), (2, 1)])
def test_every_tensor_core_configuration(ctx, tmp_path, band, rows):
    """A table that maps every bucket to one tensor-core configuration and
    sends every launch to that engine: results are the same bit for bit, on
    single matrices and on a batch."""
    entries = [{"n_bucket": nb, "L_bucket": lb, "dtype": dt, "tile": 128, "stages": 3,
                "mma_band": band, "mma_rows": rows}
               for nb in range(7) for lb in range(4) for dt in (1, 2)]
    path = str(tmp_path / "tune.json")
    with open(path, "w") as f:
        json.dump({"device": "test", "mma_min_items": [1, 1, 1, 1], "entries": entries}, f)
    ctx.tune_load(path)
    try:
        assert ctx.tune_lookup_mma(300, 1000, np.uint8) == (band, rows, 1)
        inputs = [synth.random_strings(n, L, b"ACGT-N", seed=910 + k)
                  for k, (n, L) in enumerate([(2, 5), (300, 300), (600, 4097), (1100, 64)])]
        alns = [ctx.alignment_from_sequences(s) for s in inputs]
        b = ctx.batch()
        for a, seqs in zip(alns, inputs):
            want = o.lt_dense(seqs, max_distance=40, dtype=np.uint16)
            np.testing.assert_array_equal(ctx.pairwise_lt(a, dtype=np.uint16, max_distance=40), want)
            b.add(a, dtype=np.uint16, max_distance=40)
        for got, seqs in zip(b.run(), inputs):
            np.testing.assert_array_equal(got, o.lt_dense(seqs, max_distance=40, dtype=np.uint16))
        b.free()
    finally:
        with open(path, "w") as f:
            json.dump({"entries": []}, f)
        ctx.tune_load(path)  # back to the built-in choice
    assert ctx.tune_lookup_mma(300, 1000, np.uint8) == (16, 2, 48)


def test_autotune_small_buckets(ctx, tmp_path):
    ctx.autotune(max_n_bucket=1)
    path = str(tmp_path / "t.json")
    ctx.tune_save(path)
    table = json.load(open(path))
    assert len(table["entries"]) == 2 * 4 * 2
    for e in table["entries"]:
        assert (e["tile"], e["stages"]) in {(128, 3), (128, 2), (128, 4), (64, 3), (64, 4)}
        assert (e["mma_band"], e["mma_rows"]) in {(16, 2), (8, 2), (32, 2), (16, 1)}
    assert len(table["mma_min_items"]) == 4 and all(m >= 0 for m in table["mma_min_items"])
    ctx.tune_load(path)
    e = table["entries"][0]
    band, rows, _ = ctx.tune_lookup_mma(60, 1000, np.uint8)
    assert (band, rows) == (e["mma_band"], e["mma_rows"])
    seqs = synth.random_strings(150, 1500, b"ACGT-", seed=3)
    aln = ctx.alignment_from_sequences(seqs)
    np.testing.assert_array_equal(ctx.pairwise_lt(aln), o.lt_dense(seqs))


def test_from_fasta_batch_matches_per_file_calls(tmp_path):
    rng = np.random.default_rng(8)
    files, large = [], []
    for k in range(12):
        n = int(np.exp(rng.uniform(np.log(20), np.log(600))))
        L = int(rng.choice([100, 1000, 2999]))
        rows, _, _ = synth.alignment(n, L, p=float(rng.uniform(1e-4, 1e-2)), seed=100 + k,
                                     dup_frac=0.2)
        files.append(write(tmp_path, f"f{k}.fasta", synth.to_fasta(rows)))
        large.append(bool(k % 3 == 0))
    for dedup in (False, True):
        got = hd.from_fasta_batch(files, remove_duplicates=dedup, large=large)
        assert len(got) == len(files)
        for f, big, ds in zip(files, large, got):
            ref = (hd.from_fasta_large if big else hd.from_fasta)(f, remove_duplicates=dedup,
                                                                  use_gpu=True)
            assert type(ds) is type(ref)
            np.testing.assert_array_equal(np.asarray(ds.lt_array), np.asarray(ref.lt_array))
            np.testing.assert_array_equal(seqidx_of(ds, tmp_path), seqidx_of(ref, tmp_path))
    bad = write(tmp_path, "bad.fasta", b">a\nACGT\n>b\nAC\n")
    with pytest.raises(RuntimeError, match="same length"):
        hd.from_fasta_batch(files[:2] + [bad])


def test_pipelined_file_batch_abi(ctx, tmp_path):
    # many files of uneven size, some tiny (0 or 1 row after dedupe), through
    # hd_pairwise_lt_files: every matrix and every sequence index vs the oracle
    from hammingdist_gb300 import abi

    rng = np.random.default_rng(21)
    paths, dts, mds, fastas = [], [], [], []
    for k in range(40):
        n = int(np.exp(rng.uniform(np.log(1), np.log(1500))))
        L = int(rng.choice([1, 33, 1000, 5000]))
        rows, _, _ = synth.alignment(n, L, p=float(rng.uniform(1e-4, 1e-2)), seed=300 + k,
                                     dup_frac=0.25, dash_max=min(200, L // 4))
        fa = synth.to_fasta(rows)
        paths.append(write(tmp_path, f"p{k}.fasta", fa))
        fastas.append(fa)
        big = k % 4 == 0
        dts.append(np.uint16 if big else np.uint8)
        mds.append(int(rng.integers(0, 300)) if not big else 65535)
    outs, idx = ctx.pairwise_lt_files(paths, dtypes=dts, max_distances=mds, remove_duplicates=True)
    for fa, out, ix, dt, md in zip(fastas, outs, idx, dts, mds):
        want, want_idx = o.from_fasta_dense(fa, remove_duplicates=True, max_distance=md, dtype=dt)
        np.testing.assert_array_equal(out, want)
        np.testing.assert_array_equal(ix, want_idx)
    # an empty file among the others is reported, and the context stays usable
    empty = write(tmp_path, "empty.fasta", b"")
    with pytest.raises(abi.HDError, match="Empty sequence"):
        ctx.pairwise_lt_files(paths[:3] + [empty] + paths[3:6])
    outs, _ = ctx.pairwise_lt_files(paths[:2], dtypes=dts[:2], max_distances=mds[:2],
                                    remove_duplicates=True)
    for fa, out, dt, md in zip(fastas[:2], outs, dts[:2], mds[:2]):
        np.testing.assert_array_equal(
            out, o.from_fasta_dense(fa, remove_duplicates=True, max_distance=md, dtype=dt)[0])


def test_pipelined_file_batch_errors(ctx, tmp_path):
    from hammingdist_gb300 import abi

    good = write(tmp_path, "g.fasta", b">a\nACGT\n>b\nACGA\n")
    with pytest.raises(abi.HDError, match="Failed to open file"):
        ctx.pairwise_lt_files([good, str(tmp_path / "nope.fasta"), good])
    bad = write(tmp_path, "bad2.fasta", b">a\nACGT\n>b\nAC\n")
    with pytest.raises(abi.HDError, match="same length"):
        ctx.pairwise_lt_files([good] * 5 + [bad] + [good] * 5)
    # the context stays usable
    outs, _ = ctx.pairwise_lt_files([good, good])
    assert [list(x) for x in outs] == [[1], [1]]


def test_file_batch_cpu_semantics(tmp_path):
    # use_gpu=False semantics through the pipelined batch: low-diversity files
    # take the sparse rule (5/6-plane kernels), others the dense rule; every
    # matrix equals the per-file call and the oracle's CPU semantics
    rng = np.random.default_rng(77)
    files, fastas = [], []
    for k in range(10):
        n = int(rng.integers(20, 400))
        L = int(rng.choice([500, 2000, 3001]))
        p = 1e-4 if k % 2 else 2e-2
        rows, _, _ = synth.alignment(n, L, p=p, seed=700 + k, dup_frac=0.2, dash_max=20)
        fa = synth.to_fasta(rows)
        files.append(write(tmp_path, f"c{k}.fasta", fa))
        fastas.append(fa)
    for incl_x in (False, True):
        got = hd.from_fasta_batch(files, use_gpu=False, include_x=incl_x, remove_duplicates=True)
        for f, fa, ds in zip(files, fastas, got):
            ref = hd.from_fasta(f, use_gpu=False, include_x=incl_x, remove_duplicates=True)
            np.testing.assert_array_equal(np.asarray(ds.lt_array), np.asarray(ref.lt_array))
            seqs, _ = o.read_fasta(fa, remove_duplicates=True)
            want, _ = o.lt_cpu(seqs, include_x=incl_x)
            np.testing.assert_array_equal(np.asarray(ds.lt_array), want)


def test_file_batch_read_modes(tmp_path, monkeypatch):
    # the file batch's two read orders give the same matrices: the files'
    # page-cache mappings copied into a device arena (where the device reads
    # pageable memory through the host's page tables), and
    # HAMMINGDIST_READ_MODE=pread (readers pread into pinned staging)
    from hammingdist_gb300 import abi

    rng = np.random.default_rng(33)
    paths, fastas = [], []
    for k in range(12):
        n = int(rng.integers(2, 700))
        L = int(rng.choice([7, 1000, 29903]))
        rows, _, _ = synth.alignment(n, L, p=1e-3, seed=900 + k, dup_frac=0.2)
        fa = synth.to_fasta(rows)
        paths.append(write(tmp_path, f"m{k}.fasta", fa))
        fastas.append(fa)
    got = {}
    for mode in ("map", "pread"):
        if mode == "pread":
            monkeypatch.setenv("HAMMINGDIST_READ_MODE", "pread")
        else:
            monkeypatch.delenv("HAMMINGDIST_READ_MODE", raising=False)
        c = abi.Context(0)
        try:
            got[mode] = c.pairwise_lt_files(paths, remove_duplicates=True)
            empty = write(tmp_path, "e.fasta", b"")
            with pytest.raises(abi.HDError, match="Empty sequence"):
                c.pairwise_lt_files(paths[:4] + [empty] + paths[4:])
        finally:
            c.close()
    for fa, a, b, ia, ib in zip(fastas, got["map"][0], got["pread"][0], got["map"][1],
                                got["pread"][1]):
        want, want_idx = o.from_fasta_dense(fa, remove_duplicates=True)
        np.testing.assert_array_equal(a, want)
        np.testing.assert_array_equal(b, want)
        np.testing.assert_array_equal(ia, want_idx)
        np.testing.assert_array_equal(ib, want_idx)
