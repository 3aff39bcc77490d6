"""Phase tracing: with tracing on, each traced call reports its phases with
stream times read from CUDA events; results are unchanged; off by default."""
import re

import numpy as np
import pytest

from hammingdist_gb300 import synth
from oracle import hd_oracle as o

pytestmark = pytest.mark.gpu


def _phases(text):
    return {k: float(v) for k, v in re.findall(r"([a-z][a-z ]*?) ([0-9.]+) ms", text)}


def test_trace_phases_and_results():
    from hammingdist_gb300 import abi

    ctx = abi.Context(0)
    try:
        seqs = synth.random_strings(300, 2000, b"ACGT-N", seed=5)
        fa = b"".join(b">s%d\n" % k + s + b"\n" for k, s in enumerate(seqs + seqs[:40]))
        assert ctx.trace_last() == ""
        a0 = ctx.alignment_from_fasta(fa, remove_duplicates=True)
        assert ctx.trace_last() == ""  # off by default
        want = ctx.pairwise_lt(a0)
        ctx.trace(True)
        a = ctx.alignment_from_fasta(fa, remove_duplicates=True)
        t = ctx.trace_last()
        assert t.startswith("hd_alignment_from_fasta:")
        ph = _phases(t)
        for name in ("upload", "parse", "dedupe", "pack", "stream time"):
            assert name in ph, t
        assert abs(sum(v for k, v in ph.items() if k != "stream time") - ph["stream time"]) < 0.01
        got = ctx.pairwise_lt(a)
        t2 = ctx.trace_last()
        assert t2.startswith("hd_pairwise_lt:") and "pairwise" in _phases(t2), t2
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(got, o.lt_dense(seqs))
        ctx.trace(False)
        assert ctx.trace_last() == ""
        a.free()
        a0.free()
    finally:
        ctx.close()
