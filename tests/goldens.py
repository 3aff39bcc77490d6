"""Loader for tests/golden/ (fixtures produced by the reference itself, see
tests/golden/make_golden.py)."""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class Golden:
    def __init__(self):
        self.npz = np.load(os.path.join(HERE, "golden.npz"))
        with open(os.path.join(HERE, "golden.json")) as f:
            self.meta = json.load(f)

    def __getitem__(self, key):
        return self.npz[key]

    def bytes(self, key) -> bytes:
        return self.npz[key].tobytes()

    def alignment_runs(self):
        """Yields (case name, fasta bytes, run dict) over every recorded
        from_fasta / from_fasta_large call on the alignments."""
        for case in self.meta["cases"]:
            fa = self.bytes(f"aln/{case['name']}/fasta")
            for run in case["runs"]:
                yield case["name"], fa, run

    def parse_runs(self):
        for entry in self.meta["parse"]:
            fa = self.bytes(f"parse/{entry['name']}/fasta")
            for run in entry["runs"]:
                yield entry["name"], fa, run


_CACHE = {}


def golden_meta():
    """The fixtures' metadata (json), loaded once per process."""
    if "g" not in _CACHE:
        _CACHE["g"] = Golden()
    return _CACHE["g"].meta


def golden_arrays():
    """The fixtures' arrays (npz), loaded once per process."""
    if "g" not in _CACHE:
        _CACHE["g"] = Golden()
    return _CACHE["g"].npz
