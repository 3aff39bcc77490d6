"""The seeded alignment generator used by the benchmark and the tests."""
import numpy as np

from hammingdist_gb300 import synth


def test_shapes_duplicates_and_runs():
    rows, root, nu = synth.alignment(500, 3000, p=1e-3, seed=3, dup_frac=0.3)
    assert rows.shape == (500, 3000) and root.shape == (3000,)
    assert nu == 350
    assert len({r.tobytes() for r in rows}) == 350
    assert set(np.unique(rows).tolist()) <= set(b"ACGTN-")
    assert set(np.unique(root).tolist()) <= set(b"ACGT")
    # leading and trailing '-' runs are at most 200 long
    lead = np.argmax(rows != ord("-"), axis=1)
    assert lead.max() <= 200
    # the first row is never a copy
    assert rows[0].tobytes() != b""


def test_seeded_and_fasta_format():
    a, _, _ = synth.alignment(20, 100, seed=5, dup_frac=0.2)
    b, _, _ = synth.alignment(20, 100, seed=5, dup_frac=0.2)
    assert np.array_equal(a, b)
    fa = synth.to_fasta(a)
    lines = fa.split(b"\n")
    assert lines[0] == b">s0" and lines[1] == a[0].tobytes() and fa.endswith(b"\n")
    assert fa.count(b">") == 20
