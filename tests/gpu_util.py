"""Helpers shared by the GPU tests."""
import os

import numpy as np


def write(tmp_path, name, data: bytes) -> str:
    p = os.path.join(str(tmp_path), name)
    with open(p, "wb") as f:
        f.write(data)
    return p


def seqidx_of(ds, tmp_path) -> np.ndarray:
    p = os.path.join(str(tmp_path), "idx.txt")
    ds.dump_sequence_indices(p)
    with open(p) as f:
        return np.array([int(x) for x in f.read().split()], dtype=np.uint64)


def clamp(md, large):
    tmax = 65535 if large else 255
    return tmax if md > tmax else (md & tmax)
