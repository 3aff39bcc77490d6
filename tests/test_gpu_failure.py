"""Failure detection without a GPU fault: a bounded device wait that is made
to run out reports a status and leaves the context usable; a server wait
times out and the request still completes; a queued request can be
cancelled; bad inputs fail on the host with the reference's messages."""
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


def test_bounded_wait_runs_out_and_context_survives(ctx):
    status, waited = ctx.selftest_wait_timeout(limit_ns=2_000_000)  # 2 ms, never completed
    assert status == 1
    assert waited >= 2.0 - 1e-3
    seqs = synth.random_strings(150, 500, b"ACGT-N", seed=1)
    aln = ctx.alignment_from_sequences(seqs)
    np.testing.assert_array_equal(ctx.pairwise_lt(aln), o.lt_dense(seqs))


def _resident(ctx, n, L, seed):
    nb = ctx.synthetic_fasta(n, L, seed=seed)
    buf = torch.empty(nb, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    ctx.synthetic_fasta(n, L, seed=seed, out=buf.data_ptr())
    a = ctx.alignment_from_fasta(buf.data_ptr(), nb, on_device=True)
    del buf
    return a


def test_server_wait_timeout_then_result(ctx):
    from hammingdist_gb300 import abi

    a = _resident(ctx, 6000, 29903, seed=3)
    srv = ctx.server(max_waves=1)
    i = srv.add(a)
    t = srv.pairwise(i, 0, 6000)  # ~5e11 pair-sites: several ms
    with pytest.raises(abi.HDError) as e:
        srv.wait(t, 1e-5)
    assert e.value.code == -7
    srv.wait(t, 120)
    val, cnt, lat, _ = srv.result(t)
    assert cnt == 6000 * 5999 // 2
    v = a.view(0, 6000)
    np.testing.assert_array_equal(val, ctx.pairwise_lt(v))
    v.free()
    srv.free()


def test_server_cancel_queued_request(ctx):
    from hammingdist_gb300 import abi

    a = _resident(ctx, 6000, 29903, seed=4)
    srv = ctx.server(output_budget_bytes=20 << 20, max_waves=1)
    i = srv.add(a)
    first = srv.pairwise(i, 0, 6000)       # 18 MB: occupies the only wave slot
    second = srv.pairwise(i, 100, 5000)    # queued behind it
    try:
        srv.cancel(second)
        cancelled = True
    except abi.HDError:
        cancelled = False  # already admitted: it must then complete normally
    srv.wait(first, 120)
    srv.result(first)
    if cancelled:
        with pytest.raises(abi.HDError, match="cancelled"):
            srv.wait(second, 5)
    else:
        srv.wait(second, 120)
        assert srv.result(second)[1] == 5000 * 4999 // 2
    srv.free()


def test_host_side_input_errors(ctx, tmp_path):
    import hammingdist_gb300 as hd

    p = tmp_path / "x.fasta"
    p.write_bytes(b">a\nACGT\n>b\nACGTT\n")
    with pytest.raises(RuntimeError, match="Sequences do not all have the same length"):
        hd.from_fasta(str(p))
    p.write_bytes(b">a\n\n>b\n\n")
    with pytest.raises(RuntimeError, match="Empty sequence"):
        hd.from_fasta(str(p))
    with pytest.raises(RuntimeError, match="Failed to open file"):
        hd.from_fasta_batch([str(tmp_path / "missing.fasta")])
