"""The reference's Python API tests (python/tests/test_hammingdist.py:39-204),
restated against the drop-in import name `hammingdist` with the same
parametrisations:

- from_fasta / from_fasta_large x use_gpu: every writer's output size and the
  dedupe indices, with n limits, include_x and remove_duplicates (:39-87);
- reference distances against the matrix and against distance(), for every
  character set x include_x x max_distance (:90-136);
- distance() known answers and its length error (:139-146);
- the exact lower-triangular file [[1], [2, 1]] of
  from_fasta_to_lower_triangular for every max_distance (:149-174);
- the dump_sparse round trip of a random lower-triangular file for every
  sample count x threshold (:177-204).

The inputs are this file's own, built to have the same structure (which
records repeat, which distances result). Beyond the reference's checks, the
matrices are compared with the oracle bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
hammingdist = pytest.importorskip("hammingdist")


def _fasta(path, seqs):
    with open(path, "w") as f:
        for k, s in enumerate(seqs):
            f.write(">r%d\n%s\n" % (k, s))
    return path


def _sizes_ok(ds, n_in, n_out, out, indices=None):
    """lt_array, dump, dump_lower_triangular and dump_sequence_indices agree
    with n_in input records and n_out matrix rows."""
    assert ds.lt_array.shape == (n_out * (n_out - 1) // 2,)
    ds.dump(out)
    full = np.loadtxt(out, delimiter=",", ndmin=2)
    assert full.shape == (n_out, n_out)
    ds.dump_lower_triangular(out)
    lines = open(out).read().splitlines()
    assert len(lines) == n_out - 1
    assert len(lines[0].split(",")) == 1
    assert len(lines[-1].split(",")) == n_out - 1
    ds.dump_sequence_indices(out)
    idx = np.loadtxt(out, dtype=np.uint64, ndmin=1)
    assert idx.size == n_in and idx[0] == 0
    if indices is not None:
        np.testing.assert_array_equal(idx, indices)


def _oracle_lt(raw, use_gpu, include_x, dedupe, n, large):
    from oracle import hd_oracle as o

    dt = np.uint16 if large else np.uint8
    md = 65535 if large else 255
    if use_gpu:
        return o.from_fasta_dense(raw, remove_duplicates=dedupe, n=n, max_distance=md, dtype=dt)[0]
    seqs, _ = o.read_fasta(raw, remove_duplicates=dedupe, n=n)
    return o.lt_cpu(seqs, include_x=include_x, max_distance=md, dtype=dt)[0]


# six records: the second to fourth are equal, the sixth holds an X, so that
# dedupe keeps 4 rows of 6, 3 of the first 5 and 2 of the first 3
SIX = [
    "TTGACGGATCCATGCAAGTCA",
    "TTGACGCATCCATGGAAGTCA",
    "TTGACGCATCCATGGAAGTCA",
    "TTGACGCATCCATGGAAGTCA",
    "TTGACGGATCCTTGCAAGTCA",
    "TTGAXGGATCCATGCAAGTCA",
]


@pytest.mark.parametrize("large", [False, True], ids=["from_fasta", "from_fasta_large"])
@pytest.mark.parametrize("use_gpu", [False, True])
def test_from_fasta_outputs(large, use_gpu, tmp_path):
    fn = hammingdist.from_fasta_large if large else hammingdist.from_fasta
    fa = _fasta(str(tmp_path / "six.fasta"), SIX)
    out = str(tmp_path / "out.txt")
    raw = open(fa, "rb").read()
    # (kwargs, n_in, n_out, with indices, use_gpu allowed)
    cases = [
        (dict(), 6, 6, False, True),
        (dict(n=5), 5, 5, False, True),
        (dict(include_x=True), 6, 6, False, False),
        (dict(remove_duplicates=True), 6, 4, True, True),
        (dict(remove_duplicates=True, include_x=True), 6, 4, True, False),
        (dict(include_x=True, n=2), 2, 2, True, False),
        (dict(remove_duplicates=True, n=3), 3, 2, True, True),
        (dict(remove_duplicates=True, n=5, include_x=True), 5, 3, True, False),
    ]
    for kw, n_in, n_out, with_idx, gpu_ok in cases:
        ug = use_gpu and gpu_ok
        ds = fn(fa, use_gpu=ug, **kw)
        idx = hammingdist.fasta_sequence_indices(fa, n=kw.get("n", 0)) if with_idx else None
        _sizes_ok(ds, n_in, n_out, out, idx)
        want = _oracle_lt(raw, ug, kw.get("include_x", False), kw.get("remove_duplicates", False),
                          kw.get("n", 0), large)
        np.testing.assert_array_equal(np.asarray(ds.lt_array), want)


@pytest.mark.parametrize("chars,include_x", [
    ("A", False),
    ("ACGT-", False),
    ("ACGT-", True),
    ("ACGT-X", False),
    ("ACGT-X", True),
])
@pytest.mark.parametrize("max_distance", [0, 1, 2, 3, 89, 497, 9999999])
def test_reference_distances_match_matrix(chars, include_x, max_distance, tmp_path):
    n_seq, n_sites = 50, 25
    rng = np.random.default_rng(len(chars) * 7919 + int(include_x) * 101 + max_distance)
    pool = np.frombuffer(chars.encode(), np.uint8)
    seqs = [pool[rng.integers(0, len(pool), n_sites)].tobytes().decode() for _ in range(n_seq)]
    fa = _fasta(str(tmp_path / "r.fasta"), seqs)
    ds = hammingdist.from_fasta(fa, remove_duplicates=False, include_x=include_x,
                                max_distance=max_distance)
    lt = np.asarray(ds.lt_array)
    assert lt.shape == (n_seq * (n_seq - 1) // 2,)
    mat = np.zeros((n_seq, n_seq), dtype=np.uint8)
    mat[np.tril_indices(n_seq, -1)] = lt
    for i, s in enumerate(seqs):
        vec = hammingdist.fasta_reference_distances(s, fa, include_x=include_x)
        assert vec.dtype == np.uint32 and len(vec) == n_seq
        for j, d in enumerate(vec):
            # without include_x an invalid symbol differs from itself, while
            # the matrix diagonal is 0 by construction
            if include_x or i != j:
                assert ds[i, j] == min(max_distance, d)
                assert mat[max(i, j), min(i, j)] == min(max_distance, d)
            assert d == hammingdist.distance(seqs[i], seqs[j], include_x=include_x)


def test_distance_known_answers():
    assert hammingdist.distance("GATC", "GTTC") == 1
    # X is an invalid symbol unless include_x: it differs from itself
    assert hammingdist.distance("GATCX", "GTTCX") == 2
    assert hammingdist.distance("GATCX", "GTTCX", include_x=True) == 1
    with pytest.raises(RuntimeError):
        hammingdist.distance("GATC", "GAT")


# three records with distances d(1,0) = 1, d(2,0) = 2, d(2,1) = 1; the '-'
# sites match every base
TRIPLE = [
    "TGCATGCAATCGGATCCATGACTGACCATGGTCAAGCTTGCAGTCA",
    "AGCATGCAATCGGATCCATGACTGA-CATGGTCAAGCTTGCAGTCA",
    "AGCATG-AATCGGATCCATGACTGACCATGGTCAAGCTTGC--TCC",
]


@pytest.mark.parametrize("max_distance", [0, 1, 2, 3, 89, 497, 9999999])
def test_lower_triangular_file_exact(max_distance, tmp_path):
    fa = _fasta(str(tmp_path / "t.fasta"), TRIPLE)
    out = str(tmp_path / "lt.txt")
    hammingdist.from_fasta_to_lower_triangular(fa, out, max_distance=max_distance)
    lines = open(out).read().splitlines()
    assert len(lines) == 2
    assert [int(x) for x in lines[0].split(",")] == [min(1, max_distance)]
    assert [int(x) for x in lines[1].split(",")] == [min(2, max_distance), min(1, max_distance)]


@pytest.mark.parametrize("samples", [2, 3, 5, 11, 54, 120, 532, 981, 1568])
@pytest.mark.parametrize("threshold", [0, 1, 2, 3, 4, 9, 89, 497])
def test_dump_sparse_round_trip(samples, threshold, tmp_path):
    rng = np.random.default_rng(samples * 1000 + threshold)
    lt_file = str(tmp_path / "lt.txt")
    with open(lt_file, "w") as f:
        for i in range(1, samples):
            f.write(",".join(str(v) for v in rng.integers(0, 256, i)) + "\n")
    ds = hammingdist.from_lower_triangular(lt_file)
    vals = np.asarray(ds._distances)
    below = int(np.sum(vals <= threshold))
    if below == 0:
        return
    sp = str(tmp_path / "sparse.txt")
    ds.dump_sparse(sp, threshold)
    got = np.loadtxt(sp, delimiter=" ", dtype=np.int64, ndmin=2)
    assert got.shape == (below, 3)
    assert np.all(got[:, 2] <= threshold)
    i, j = np.maximum(got[:, 0], got[:, 1]), np.minimum(got[:, 0], got[:, 1])
    np.testing.assert_array_equal(vals[i * (i - 1) // 2 + j], got[:, 2])
    for e in got[:: max(1, len(got) // 50)]:  # spot checks through DataSet.__getitem__
        assert ds[int(e[0]), int(e[1])] == e[2]
