"""Serving: resident alignments, requests folded into waves of the
persistent engine. Each result must be the same in the mix, alone, and from
the plain per-request call (bit-exact); the synthetic device generator must
match its host mirror."""
import numpy as np
import pytest

from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    from hammingdist_gb300 import abi

    c = abi.Context(0)
    yield c
    c.close()


def _device_alignment(ctx, n, L, seed, p=1e-3, dedup=False):
    nb = ctx.synthetic_fasta(n, L, p=p, seed=seed)
    buf = torch.empty(nb, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    ctx.synthetic_fasta(n, L, p=p, seed=seed, out=buf.data_ptr())
    aln = ctx.alignment_from_fasta(buf.data_ptr(), nb, on_device=True, remove_duplicates=dedup)
    host = buf.cpu().numpy().tobytes()
    del buf
    return aln, host


def test_device_generator_matches_host_mirror(ctx):
    n, L, seed = 300, 2999, 77
    aln, fa = _device_alignment(ctx, n, L, seed, p=1e-2)
    assert len(fa) == synth.device_fasta_bytes(n, L)
    seqs, _ = o.read_fasta(fa)
    assert len(seqs) == n and all(len(s) == L for s in seqs)
    root = synth.device_root(seed, L).tobytes()
    assert set(b"".join(seqs)) <= set(b"ACGTN-")
    # away from the dash runs most sites equal the root
    mid = [s[300:-300] for s in seqs]
    same = np.mean([np.mean(np.frombuffer(m, np.uint8) == np.frombuffer(root[300:-300], np.uint8))
                    for m in mid])
    assert same > 0.95
    assert fa.startswith(b">s000000000\n") and b">s000000299\n" in fa
    # the ingest of device-resident bytes equals the oracle on the same bytes
    np.testing.assert_array_equal(ctx.pairwise_lt(aln), o.lt_dense(seqs))


def _plain(ctx, aln, kind, args):
    if kind == "ref":
        return ctx.alignment_reference_distances(aln, args[0])
    row0, n = args[0], args[1]
    view = aln.view(row0, n)
    if kind == "pair":
        out = ctx.pairwise_lt(view, dtype=args[2], max_distance=args[3])
    else:
        lt = ctx.pairwise_lt(view, dtype=np.uint8, max_distance=255)
        out = o.format_sparse(lt, n, args[2])
    view.free()
    return out


def test_served_mix_equals_alone_and_plain(ctx):
    a0, fa0 = _device_alignment(ctx, 2500, 2999, seed=5, dedup=True)
    a1, _ = _device_alignment(ctx, 900, 29903, seed=6)
    alns = [a0, a1]
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(60):
        which = int(rng.integers(0, 2))
        a = alns[which]
        kind = ["ref", "pair", "sparse"][int(rng.choice(3, p=[0.5, 0.3, 0.2]))]
        if kind == "ref":
            q = bytearray(synth.device_root(5 if which == 0 else 6, a.length).tobytes())
            for s in rng.integers(0, a.length, 20):
                q[s] = ord("ACGTN"[int(rng.integers(0, 5))])
            reqs.append((which, kind, (bytes(q),)))
        else:
            n = int(rng.integers(2, min(a.n_rows, 700)))
            r0 = int(rng.integers(0, a.n_rows - n + 1))
            if kind == "pair":
                dt = np.uint16 if rng.integers(0, 2) else np.uint8
                reqs.append((which, kind, (r0, n, dt, int(rng.choice([3, 255, 65535])))))
            else:
                reqs.append((which, kind, (r0, n, int(rng.integers(1, 6)) * 40)))
    srv = ctx.server(output_budget_bytes=64 << 20, max_waves=3)
    ids = [srv.add(a) for a in alns]

    def submit(which, kind, args):
        if kind == "ref":
            return srv.reference(ids[which], args[0])
        if kind == "pair":
            return srv.pairwise(ids[which], args[0], args[1], dtype=args[2], max_distance=args[3])
        return srv.sparse(ids[which], args[0], args[1], args[2])

    tickets = [submit(*r) for r in reqs]  # all at once: folded into shared waves
    mix = []
    for t in tickets:
        srv.wait(t, 120)
        mix.append(srv.result(t)[0])
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["waves"] < len(reqs)
    for (which, kind, args), got in zip(reqs, mix):
        want = _plain(ctx, alns[which], kind, args)
        if kind == "sparse":
            assert got == want
        else:
            np.testing.assert_array_equal(got, want)
        t = submit(which, kind, args)  # alone
        srv.wait(t, 120)
        alone = srv.result(t)[0]
        assert (alone == got) if kind == "sparse" else np.array_equal(alone, got)
    # queries against the deduplicated set give one distance per input record
    for (which, kind, args), got in zip(reqs, mix):
        if kind == "ref" and which == 0:
            np.testing.assert_array_equal(got, o.reference_distances(args[0], fa0))
    srv.free()


def test_budget_admission_and_errors(ctx):
    from hammingdist_gb300 import abi

    a, _ = _device_alignment(ctx, 600, 1000, seed=9)
    srv = ctx.server(output_budget_bytes=1 << 16, max_waves=2)  # 64 KB: one 300-row matrix at a time
    i = srv.add(a)
    tickets = [srv.pairwise(i, 10 * k, 300) for k in range(6)]
    outs = []
    for t in tickets:
        srv.wait(t, 120)
        outs.append(srv.result(t))
    for k, (val, cnt, lat, queue) in enumerate(outs):
        np.testing.assert_array_equal(val, _plain(ctx, a, "pair", (10 * k, 300, np.uint8, 255)))
        assert cnt == 300 * 299 // 2 and lat >= queue >= 0
    assert srv.stats()["waves"] >= 3  # the budget kept the matrices apart
    with pytest.raises(abi.HDError):
        srv.pairwise(i, 500, 200)  # window out of range
    with pytest.raises(abi.HDError):
        srv.reference(i, b"ACGT")  # wrong length
    srv.free()
