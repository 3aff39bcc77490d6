"""Generates tests/golden/golden.npz + golden.json from the REFERENCE itself.

Run in a container where the reference sources exist and oracle/build_ref.sh
has built them into oracle/_ref/ (the reference's own pybind11 module
`hammingdist`, CPU build). The GPU machine never runs this script; it only reads
the committed fixtures.

    python oracle/build_ref.sh && python tests/golden/make_golden.py

Every input is generated here from fixed seeds and stored next to the
reference's outputs, so a test can replay the input through another
implementation and compare byte for byte.
"""
from __future__ import annotations

import contextlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _load_reference():
    """The reference's module `hammingdist`, built by oracle/build_ref.sh,
    loaded from its file: the repository root also holds a module of that
    name (the drop-in alias of hammingdist_gb300)."""
    import glob
    import importlib.machinery
    import importlib.util

    so = glob.glob(os.path.join(ROOT, "oracle", "_ref", "hammingdist*.so"))
    if not so:
        raise SystemExit("build the reference first: oracle/build_ref.sh")
    loader = importlib.machinery.ExtensionFileLoader("hammingdist", so[0])
    spec = importlib.util.spec_from_file_location("hammingdist", so[0], loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


ref = _load_reference()
from hammingdist_gb300 import synth  # noqa: E402

assert "oracle" in ref.__file__, ref.__file__

TMP = tempfile.mkdtemp(prefix="hd_golden_")
arrays: dict[str, np.ndarray] = {}
meta: dict = {"cases": []}


@contextlib.contextmanager
def capture_fd1():
    """Captures the reference's std::cout (file descriptor 1)."""
    sys.stdout.flush()
    path = os.path.join(TMP, "stdout.txt")
    saved = os.dup(1)
    with open(path, "w") as f:
        os.dup2(f.fileno(), 1)
        box = {}
        try:
            yield box
        finally:
            sys.stdout.flush()
            os.dup2(saved, 1)
            os.close(saved)
    box["text"] = open(path).read()


def put(key, arr):
    assert key not in arrays, key
    arrays[key] = np.asarray(arr)


def write_fasta_bytes(data: bytes) -> str:
    path = os.path.join(TMP, "in.fasta")
    with open(path, "wb") as f:
        f.write(data)
    return path


def run_from_fasta(path, large, **kw):
    fn = ref.from_fasta_large if large else ref.from_fasta
    with capture_fd1() as box:
        try:
            d = fn(path, **kw)
            err = None
        except RuntimeError as e:
            d, err = None, str(e)
    out = box["text"]
    if err is not None:
        return {"error": err}
    used = "sparse" if "sparse distance function" in out else (
        "dense" if "SIMD extensions" in out else "unknown")
    seqidx_path = os.path.join(TMP, "idx.txt")
    d.dump_sequence_indices(seqidx_path)
    seqidx = np.loadtxt(seqidx_path, dtype=np.uint64, ndmin=1)
    return {"lt": np.asarray(d.lt_array).copy(), "nsamples": d.lt_array.size,
            "seqidx": seqidx, "path": used, "ds": d}


# ---------------------------------------------------------------- truth tables
CHARS = b"ACGT-NX*?a. "
n_c = len(CHARS)
for include_x in (0, 1):
    dist = np.zeros((n_c, n_c), dtype=np.uint32)
    lt1 = np.zeros((n_c, n_c), dtype=np.uint8)
    for a in range(n_c):
        for b in range(n_c):
            s0, s1 = chr(CHARS[a]), chr(CHARS[b])
            dist[a, b] = ref.distance(s0, s1, include_x=bool(include_x))
            with capture_fd1():
                lt1[a, b] = ref.from_stringlist([s0, s1], bool(include_x), False, 255)[0, 1]
    put(f"truth/distance/x{include_x}", dist)
    put(f"truth/stringlist/x{include_x}", lt1)
meta["truth_chars"] = CHARS.decode()

# ------------------------------------------------------- known-answer pairs (2)
KAT2 = [
    ("AC", "CA"), ("AC", "TG"), ("ACG", "AGT"), ("ACG", "-TT"), ("ACG", "T-T"),
    ("ACG", "TA-"), ("ACG", "CCC"), ("ACGT", "AGGG"),
    ("ACGTGTCGTGTCGACGTGTCG", "ACGTGTCGTTTCGACGAGTCG"),
    ("ACGTGTCGTGTCGACGTGTCGT", "ACGTGTCGTTTCGACGAGTCGT"),
    ("ACGTGTCGTGTCGACGTGTCGT-", "ACGTGTCGTTTCGACGAGTCGTA"),
    ("ACGTGTCGTGTCGACGTGTCG----------", "ACGTGTCGTTTCGACGAGTCGGGG-------"),
    ("ACGTGTCGTGTCGACGTGTCG----------A", "ACGTGTCGTTTCGACGAGTCGGGG-------A"),
    ("ACGTGTCGTGTCGACGTGTCG----------AG", "ACGTGTCGTTTCGACGAGTCGGGG-------AG"),
    ("ACGTGTCGTGTCGACGTGTCG---ACGTGTCGTGTCGACGTGTCG---ACGTGTCGTGTCGACGTGTCG---",
     "ACGTGTCGTTTCGACGAGTCGGGGACGTGTCGTGTCGACGTGTCG---ACGTGTCGTGTCGACGTGTCG---"),
]
kat = []
for a, b in KAT2:
    with capture_fd1():
        d = ref.from_stringlist([a, b], False, False, 255)
    kat.append([a, b, int(d[0, 1]), int(ref.distance(a, b))])
meta["kat2"] = kat

# ------------------------------------------------------------------ saturation
sat = []
for m in (255, 256, 354, 65535, 65536, 65634):
    for md in (0, 1, 2, 3, 7, 21, 886, 2784904, 99999999):
        fa = b">a\n" + b"A" * m + b"\n>t\n" + b"T" * m + b"\n"
        path = write_fasta_bytes(fa)
        r8 = run_from_fasta(path, False, max_distance=md)
        r16 = run_from_fasta(path, True, max_distance=md)
        sat.append([m, md, int(r8["lt"][0]), int(r16["lt"][0])])
meta["saturation"] = sat

# ----------------------------------------------------- alignments (main parity)
ALIGNMENTS = []


def add_alignment(name, rows_bytes, combos, refs=()):
    ALIGNMENTS.append((name, rows_bytes, combos, refs))


def fasta_of(rows):
    return b"".join(b">s%d\n%s\n" % (i, r) for i, r in enumerate(rows))


MD_FULL = (0, 1, 2, 3, 89, 255, 497, 65535, 9999999, -1, -300)
MD_SHORT = (3, 255, 65535)

# uniform over ACGT- (the reference tests' generator shape): dense path
add_alignment("uniform5", synth.random_strings(45, 37, b"ACGT-", 1),
              {"md": MD_FULL, "x": (0, 1), "dedup": (0, 1)})
add_alignment("uniform_invalid", synth.random_strings(33, 129, b"ACGT-NX*a", 2),
              {"md": MD_SHORT, "x": (0, 1), "dedup": (0, 1)})
add_alignment("uniform_x", synth.random_strings(30, 64, b"ACGT-X", 3),
              {"md": MD_SHORT, "x": (0, 1), "dedup": (0, 1)})
for L in (1, 2, 3, 7, 8, 9, 15, 16, 17, 31, 32, 33, 63, 64, 65, 255, 256, 257, 511, 513, 1023,
          1025, 2049):
    add_alignment(f"len{L}", synth.random_strings(6, L, b"ACGT-", 100 + L),
                  {"md": (255, 65535), "x": (0,), "dedup": (0,)})
# duplicates
base = synth.random_strings(12, 50, b"ACGT-N", 5)
rng = np.random.default_rng(6)
dup_rows = [base[int(rng.integers(0, 12))] if i and rng.random() < 0.6 else base[i % 12]
            for i in range(50)]
add_alignment("dups", dup_rows, {"md": MD_SHORT, "x": (0, 1), "dedup": (0, 1)})
# low diversity: the reference takes its sparse branch
for k, (n, L, p, dash, nrate) in enumerate([(40, 3000, 1e-4, 10, 0.0), (64, 2000, 2e-4, 5, 2e-5),
                                            (25, 5000, 5e-4, 0, 0.0)]):
    rows, root, _ = synth.alignment(n, L, p=p, seed=20 + k, dash_max=dash, n_rate=nrate)
    add_alignment(f"lowdiv{k}", [r.tobytes() for r in rows],
                  {"md": (2, 255, 65535), "x": (0, 1), "dedup": (0, 1)}, refs=(root.tobytes(),))
# the benchmark generator's shape at small n: dense
rows, root, _ = synth.alignment(80, 2999, p=1e-3, seed=30, dup_frac=0.3)
add_alignment("covid_small", [r.tobytes() for r in rows],
              {"md": (0, 2, 3, 255, 65535), "x": (0, 1), "dedup": (0, 1)}, refs=(root.tobytes(),))
rows, root, _ = synth.alignment(64, 4001, p=2e-2, seed=31, dash_max=50)
add_alignment("wide", [r.tobytes() for r in rows],
              {"md": (3, 255, 400, 65535), "x": (0,), "dedup": (0,)}, refs=(root.tobytes(),))

for name, rows, combos, refs in ALIGNMENTS:
    fa = fasta_of(rows)
    path = write_fasta_bytes(fa)
    put(f"aln/{name}/fasta", np.frombuffer(fa, dtype=np.uint8))
    case = {"name": name, "runs": [], "refdist": [], "seqidx": []}
    for large in (0, 1):
        for x in combos["x"]:
            for dd in combos["dedup"]:
                for md in combos["md"]:
                    if not large and md == 65535:
                        continue
                    r = run_from_fasta(path, bool(large), include_x=bool(x),
                                       remove_duplicates=bool(dd), max_distance=md)
                    key = f"aln/{name}/L{large}x{x}d{dd}m{md}"
                    run = {"large": large, "x": x, "dedup": dd, "md": md, "key": key}
                    if "error" in r:
                        run["error"] = r["error"]
                    else:
                        put(key + "/lt", r["lt"])
                        put(key + "/seqidx", r["seqidx"])
                        run["path"] = r["path"]
                        run["nsamples"] = int(r["ds"].lt_array.size)
                    case["runs"].append(run)
    # writers on the default-max DataSets
    for large in (0, 1):
        r = run_from_fasta(path, bool(large))
        if "error" in r:
            continue
        ltf = os.path.join(TMP, "lt.txt")
        r["ds"].dump_lower_triangular(ltf)
        put(f"aln/{name}/lttext{large}", np.frombuffer(open(ltf, "rb").read(), dtype=np.uint8))
        for thr in (0, 1, 3, 20, 255):
            spf = os.path.join(TMP, "sp.txt")
            r["ds"].dump_sparse(spf, thr)
            lines = sorted(open(spf, "rb").read().splitlines(keepends=True))
            put(f"aln/{name}/sparse{large}t{thr}", np.frombuffer(b"".join(lines), dtype=np.uint8))
    # reference distances: the first row, a middle row and the given refs
    cand = [rows[0], rows[len(rows) // 2]] + list(refs)
    for k, rseq in enumerate(cand):
        for x in (0, 1):
            v = ref.fasta_reference_distances(rseq.decode(), path, include_x=bool(x))
            put(f"aln/{name}/refdist{k}x{x}", np.asarray(v))
            case["refdist"].append([k, x])
        put(f"aln/{name}/refseq{k}", np.frombuffer(rseq, dtype=np.uint8))
    for nlim in (0, 1, 2, 3, 7, 1000):
        put(f"aln/{name}/seqidx_n{nlim}", np.asarray(ref.fasta_sequence_indices(path, nlim)))
        case["seqidx"].append(nlim)
    meta["cases"].append(case)

# -------------------------------------------------------------- FASTA parsing
PARSE = {
    "multiline": b">s0\nACGTGTCGTGTCGACGTGTCG\nACGTGTCGTGTCGACGTGTCG\nACGTGTCGTGTCG\n"
                 b">s1\nACGTGTCGTTTCGACGAGTCG\nACGTGTCGTGTCGACGTGTCG\nACGTGTCGTGTCG\n",
    "dups6": b">seq0\nACGTGTCGTGTCGACGTGTCG\n>seq1\nACGTGTCGTTTCGACGAGTCG\n>seq2\n"
             b"ACGTGTCGTTTCGACGAGTCG\n>seq3\nACGTGTCGTTTCGACGAGTCG\n>seq4\n"
             b"ACGTGTCGTGTCGACGTGTCG\n>seq5\nACGTGTCGTATCGACGTGTCG\n",
    "blank_lines": b">a\nACGT\n\nAC\n\n>b\n\nACG-TA\n>c\nTTTTT\nA\n",
    "crlf": b">a\r\nACGTAC\r\n>b\r\nACGTTC\r\n>c\r\nAGGTAC\r\n",
    "no_trailing_newline": b">a\nACGTA\n>b\nACCTA",
    "trailing_header_nl": b">a\nACGTA\n>b\nACCTA\n>c\n",
    "trailing_header_eof": b">a\nACGTA\n>b\nACCTA\n>c",
    "header_only_nl": b">a\n",
    "header_only_eof": b">a",
    "empty": b"",
    "no_header": b"ACGTA\nACGTT\n>x\nACGTC\n",
    "empty_record": b">a\n>b\nACGT\n>c\nACGA\n",
    "gt_in_sequence": b">a\nAC>GT\n>b\nACCGT\n",
    "ragged": b">a\nACGT\n>b\nACG\n>c\nACGTA\n",
    "multi_dup": b">a\nAC\nGT\n>b\nACGT\n>c\nA\nCGT\n>d\nTTTT\n>e\nAC\nG\nT\n",
    "lowercase": b">a\nacgtNNAC\n>b\nACGTNNAC\n>c\nacgtnnac\n",
}
meta["parse"] = []
for name, fa in PARSE.items():
    path = write_fasta_bytes(fa)
    put(f"parse/{name}/fasta", np.frombuffer(fa, dtype=np.uint8))
    entry = {"name": name, "runs": []}
    for dd in (0, 1):
        for nlim in (0, 1, 2, 3):
            r = run_from_fasta(path, False, remove_duplicates=bool(dd), n=nlim)
            key = f"parse/{name}/d{dd}n{nlim}"
            run = {"dedup": dd, "n": nlim, "key": key}
            if "error" in r:
                run["error"] = r["error"]
            else:
                put(key + "/lt", r["lt"])
                put(key + "/seqidx", r["seqidx"])
                run["path"] = r["path"]
            entry["runs"].append(run)
    # at least as long as any record (the reference reads past a shorter one)
    maxlen = len(fa) + 1
    refseq = (b"ACGTN-" * (maxlen // 6 + 2))[:maxlen + 3]
    for x in (0, 1):
        v = ref.fasta_reference_distances(refseq.decode(), path, include_x=bool(x))
        put(f"parse/{name}/refdist{x}", np.asarray(v))
    put(f"parse/{name}/refseq", np.frombuffer(refseq, dtype=np.uint8))
    for nlim in (0, 2):
        put(f"parse/{name}/seqidx_n{nlim}", np.asarray(ref.fasta_sequence_indices(path, nlim)))
    meta["parse"].append(entry)

# ------------------------------------------------------- result file formats
# dump() (full matrix text, include/hamming/hamming.hh:63-73) of DataSets built
# from some of the alignments above; from_lower_triangular[_large]
# (hamming.hh:152-166) and from_csv (hamming.hh:34-55) on valid files and on
# malformed ones, with the exception the reference raises.
def describe(ds):
    """lt_array and the dump() text (which shows nsamples) of a reference DataSet."""
    f = os.path.join(TMP, "describe.txt")
    ds.dump(f)
    return np.asarray(ds.lt_array), open(f, "rb").read()


def try_load(fn, data: bytes):
    path = os.path.join(TMP, "load.txt")
    with open(path, "wb") as f:
        f.write(data)
    try:
        ds = fn(path)
    except Exception as e:  # noqa: BLE001  (the reference's own exception)
        return {"error_type": type(e).__name__, "error": str(e)}
    lt, text = describe(ds)
    return {"lt": lt, "dump": text}


meta["formats"] = {"dump": [], "lt": [], "csv": []}
by_name = {name: rows for name, rows, _, _ in ALIGNMENTS}
for name in ("uniform5", "dups", "covid_small", "len1", "len33", "wide", "uniform_invalid"):
    path = write_fasta_bytes(fasta_of(by_name[name]))
    for large in (0, 1):
        r = run_from_fasta(path, bool(large))
        f = os.path.join(TMP, "dump.txt")
        r["ds"].dump(f)
        put(f"fmt/dump/{name}{large}", np.frombuffer(open(f, "rb").read(), dtype=np.uint8))
        meta["formats"]["dump"].append({"name": name, "large": large})

LT_CASES = {
    "basic": b"1\n2,3\n",
    "no_final_newline": b"1\n2,3",
    "crlf": b"1\r\n2,3\r\n",
    "spaces": b" 1\n\t2, 3\n",
    "signs": b"+1\n-2,3\n",
    "saturate": b"300\n70000,5\n",
    "negative_wrap": b"-1\n-300,-70000\n",
    "trailing_comma": b"1\n2,3,\n",
    "empty_line": b"1\n\n2,3\n",
    "letters": b"1\n2,x\n",
    "out_of_range": b"1\n99999999999,3\n",
    "digits_then_text": b"12abc\n3,4z\n",
    "empty_file": b"",
    "only_newline": b"\n",
    "non_triangular4": b"1,2,3,4\n",
    "non_triangular7": b"1,2\n3,4,5\n6,7\n",
    "single": b"5\n",
    "leading_zeros": b"0007\n00,010\n",
    "sign_only": b"1\n+,3\n",
    "space_only": b"1\n ,3\n",
    "big_negative": b"1\n-99999999999,3\n",
    "int_max": b"2147483647\n-2147483648,0\n",
}
for key in ("dups", "covid_small", "wide"):
    LT_CASES[f"lttext_{key}"] = bytes(arrays[f"aln/{key}/lttext1"])
for cname, data in LT_CASES.items():
    put(f"fmt/lt/{cname}/input", np.frombuffer(data, dtype=np.uint8))
    entry = {"name": cname}
    for large, fn in ((0, ref.from_lower_triangular), (1, ref.from_lower_triangular_large)):
        res = try_load(fn, data)
        if "error" in res:
            entry[f"error{large}"] = [res["error_type"], res["error"]]
        else:
            put(f"fmt/lt/{cname}/lt{large}", res["lt"])
            put(f"fmt/lt/{cname}/dump{large}", np.frombuffer(res["dump"], dtype=np.uint8))
    meta["formats"]["lt"].append(entry)

CSV_CASES = {
    "two": b"0, 1\n1, 0\n",
    "one": b"0\n",
    "no_final_newline": b"0, 1\n1, 0",
    "wrap": b"0, 300\n300, 0\n",
    "negative": b"0, -1\n-1, 0\n",
    "short_row": b"0, 5\n\n",
    "extra_fields": b"9, 9, 9\n1, 9, 9\n2, 3, 9\n",
    "letters": b"a, b\nc, d\n",
    "row0_garbage": b"zz\n4, 0\n",
    "crlf": b"0, 1\r\n1, 0\r\n",
    "empty_file": b"",
    "too_few_in_row2": b"0\n1\n2\n",
    "out_of_range": b"0\n99999999999, 0\n",
}
for key in ("dups", "uniform5"):
    CSV_CASES[f"dump_{key}"] = bytes(arrays[f"fmt/dump/{key}0"])
for cname, data in CSV_CASES.items():
    put(f"fmt/csv/{cname}/input", np.frombuffer(data, dtype=np.uint8))
    entry = {"name": cname}
    res = try_load(ref.from_csv, data)
    if "error" in res:
        entry["error"] = [res["error_type"], res["error"]]
    else:
        put(f"fmt/csv/{cname}/lt", res["lt"])
        put(f"fmt/csv/{cname}/dump", np.frombuffer(res["dump"], dtype=np.uint8))
    meta["formats"]["csv"].append(entry)

out = os.path.join(HERE, "golden.npz")
np.savez_compressed(out, **arrays)
with open(os.path.join(HERE, "golden.json"), "w") as f:
    json.dump(meta, f, indent=1, sort_keys=True)
print("wrote", out, os.path.getsize(out), "bytes,", len(arrays), "arrays")
