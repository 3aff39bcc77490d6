"""Seeded synthetic alignments for tests and benchmarks.

The generator produces SARS-CoV-2-like aligned FASTA text: a root sequence
uniform over ACGT; each sequence copies the root with per-site substitution
(probability ``p``, new base uniform over ACGT, which may equal the old one),
leading and trailing '-' runs of uniform length 0..``dash_max``, and internal
'N' runs that start at a site with probability ``n_rate`` and last 1..50
sites. Exact duplicates of earlier unique sequences can be inserted at random
positions (``dup_frac`` of the output). Records are written as
``>s{i}\\n{seq}\\n``. No public dataset is involved.
"""
from __future__ import annotations

import numpy as np

_ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def _batch(rng, root, k, p, dash_max, n_rate, n_run_max):
    """k mutated copies of root, generated together."""
    L = root.size
    s = np.broadcast_to(root, (k, L)).copy()
    if p > 0:
        m = rng.random((k, L)) < p
        c = int(m.sum())
        if c:
            s[m] = _ACGT[rng.integers(0, 4, c)]
    if n_rate > 0:
        rr, cc = np.nonzero(rng.random((k, L)) < n_rate)
        for r, st in zip(rr, cc):
            s[r, st:st + int(rng.integers(1, n_run_max + 1))] = ord("N")
    if dash_max > 0:
        a = rng.integers(0, dash_max + 1, k)
        b = rng.integers(0, dash_max + 1, k)
        col = np.arange(L)
        s[col[None, :] < a[:, None]] = ord("-")
        s[col[None, :] >= (L - b)[:, None]] = ord("-")
    return s


def alignment(n: int, L: int, p: float = 1e-3, seed: int = 0, dup_frac: float = 0.0,
              dash_max: int = 200, n_rate: float = 1e-4, n_run_max: int = 50,
              root: np.ndarray | None = None):
    """Returns (rows uint8 [n, L], root uint8 [L], n_unique). n_unique is the
    number of generated (not copied) rows; two generated rows may still be
    equal by chance, which deduplication then merges."""
    rng = np.random.default_rng(seed)
    if root is None:
        root = _ACGT[rng.integers(0, 4, L)]
    n_dup = int(round(n * dup_frac))
    n_unique = n - n_dup
    uniq = np.empty((n_unique, L), dtype=np.uint8)
    for b0 in range(0, n_unique, 256):
        k = min(256, n_unique - b0)
        uniq[b0:b0 + k] = _batch(rng, root, k, p, dash_max, n_rate, n_run_max)
    # duplicates sit at random positions (never the first) and copy a random
    # earlier generated row
    is_dup = np.zeros(n, dtype=bool)
    if n_dup:
        is_dup[rng.choice(np.arange(1, n), size=n_dup, replace=False)] = True
    rows = np.empty((n, L), dtype=np.uint8)
    u = 0
    for i in range(n):
        if is_dup[i]:
            rows[i] = uniq[int(rng.integers(0, u))]
        else:
            rows[i] = uniq[u]
            u += 1
    return rows, root, n_unique


def to_fasta(rows: np.ndarray, names=None) -> bytes:
    """Writes rows as '>s{i}\\n{seq}\\n' records."""
    n, L = rows.shape
    parts = []
    for i in range(n):
        parts.append(b">s%d\n" % i if names is None else b">" + names[i] + b"\n")
        parts.append(rows[i].tobytes())
        parts.append(b"\n")
    return b"".join(parts)


def random_strings(n: int, L: int, chars: bytes, seed: int) -> list[bytes]:
    """n strings of length L drawn uniformly from `chars` (the shape of the
    reference tests' make_test_string helper)."""
    rng = np.random.default_rng(seed)
    pool = np.frombuffer(chars, dtype=np.uint8)
    m = pool[rng.integers(0, len(pool), size=(n, L))]
    return [m[i].tobytes() for i in range(n)]


# ---------------------------------------------------------------------------
# Host mirror of the device generator (hd_synthetic_fasta, csrc/hd_synth.cu):
# every byte is a function of (seed, record, site), so a host caller can
# rebuild a root or a record of a resident set generated on the device.
_M = (1 << 64) - 1


def _mix(x):
    x = np.asarray(x, dtype=np.uint64)
    x = x ^ (x >> np.uint64(30))
    x = x * np.uint64(0xBF58476D1CE4E5B9)
    x = x ^ (x >> np.uint64(27))
    x = x * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _hash(seed, a, b):
    with np.errstate(over="ignore"):
        a = np.asarray(a, dtype=np.uint64)
        b = np.asarray(b, dtype=np.uint64)
        return _mix(np.uint64(seed & _M) + a * np.uint64(0x9E3779B97F4A7C15)
                    + b * np.uint64(0xD1B54A32D192ED03))


def device_root(seed: int, L: int) -> np.ndarray:
    """Root sequence of hd_synthetic_fasta(seed, ..., L)."""
    s = np.arange(L, dtype=np.uint64)
    return _ACGT[(_hash(seed, 0xFFFFFFFF, s) & np.uint64(3)).astype(np.intp)]


def device_fasta_bytes(n: int, L: int) -> int:
    return n * (L + 13)
