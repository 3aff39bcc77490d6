"""ctypes wrapper of oracle/hd_oracle.c, the CPU restatement of hammingdist's
pairwise Hamming-distance path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker. The product package
(hammingdist_gb300) never imports it.

Each wrapper names the reference function it restates; the C file cites the
reference file:line for each.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "hd_oracle.c")
_OUT = os.path.join(_HERE, "_build", "libhd_oracle.so")
_lock = threading.Lock()
_lib = None

ERRORS = {
    -1: "Error: Empty sequence",
    -2: "Error: Sequences do not all have the same length",
    -3: "oracle: out of memory",
    -4: "oracle: bad argument",
    -5: "oracle: a sequence is longer than the reference sequence",
}


def build(force: bool = False) -> str:
    """Compile hd_oracle.c into oracle/_build/libhd_oracle.so (gcc, OpenMP)."""
    import platform

    stamp = _OUT + ".arch"
    same_arch = os.path.exists(stamp) and open(stamp).read() == platform.machine()
    if force or not same_arch or not os.path.exists(_OUT) or \
            os.path.getmtime(_OUT) < os.path.getmtime(_SRC):
        os.makedirs(os.path.dirname(_OUT), exist_ok=True)
        tmp = _OUT + f".tmp{os.getpid()}"
        subprocess.check_call(
            ["gcc", "-O3", "-std=c11", "-fopenmp", "-shared", "-fPIC", _SRC, "-o", tmp, "-lm"]
        )
        os.replace(tmp, _OUT)
        with open(stamp, "w") as f:
            f.write(platform.machine())
    return _OUT


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            u64, i64, vp, cp = ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_char_p
            P = ctypes.POINTER
            L.hdo_lt_dense.argtypes = [vp, u64, u64, i64, ctypes.c_int, vp]
            L.hdo_lt_cpu.argtypes = [cp, vp, u64, ctypes.c_int, i64, ctypes.c_int, vp,
                                     P(ctypes.c_int)]
            L.hdo_read_fasta.argtypes = [cp, ctypes.c_size_t, ctypes.c_int, u64,
                                         P(vp), P(vp), P(u64), P(vp), P(u64)]
            L.hdo_fasta_sequence_indices.argtypes = [cp, ctypes.c_size_t, u64, P(vp), P(u64)]
            L.hdo_reference_distances.argtypes = [cp, u64, cp, ctypes.c_size_t, ctypes.c_int,
                                                  P(vp), P(u64)]
            L.hdo_distance.argtypes = [cp, u64, cp, u64, ctypes.c_int, P(ctypes.c_uint32)]
            L.hdo_from_fasta_dense.argtypes = [cp, ctypes.c_size_t, ctypes.c_int, u64, i64,
                                               ctypes.c_int, vp, u64, P(u64), vp, P(u64)]
            L.hdo_from_fasta_dense_once.argtypes = [cp, ctypes.c_size_t, ctypes.c_int, u64, i64,
                                                    ctypes.c_int, P(vp), P(u64), P(vp), P(u64)]
            L.hdo_format_lower_triangular.argtypes = [vp, u64, ctypes.c_int, vp]
            L.hdo_format_lower_triangular.restype = u64
            L.hdo_format_sparse.argtypes = [vp, u64, ctypes.c_int, i64, vp, P(u64)]
            L.hdo_format_sparse.restype = u64
            L.hdo_pack_row.argtypes = [cp, u64, vp]
            L.hdo_packed_row_bytes.argtypes = [u64]
            L.hdo_packed_row_bytes.restype = u64
            L.hdo_dump_full.argtypes = [vp, u64, u64, ctypes.c_int, cp]
            L.hdo_read_lower_triangular.argtypes = [cp, ctypes.c_int, P(vp), P(u64), P(u64),
                                                    P(ctypes.c_int)]
            L.hdo_read_csv.argtypes = [cp, P(vp), P(u64), P(u64), P(ctypes.c_int)]
            L.hdo_free.argtypes = [vp]
            L.hdo_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(ERRORS.get(rc, f"oracle error {rc}"))


def _take(ptr: int, n: int, dtype) -> np.ndarray:
    if n == 0 or not ptr:
        if ptr:
            lib().hdo_free(ptr)
        return np.zeros(0, dtype=dtype)
    arr = np.empty(n, dtype=dtype)
    ctypes.memmove(arr.ctypes.data, ptr, arr.nbytes)
    lib().hdo_free(ptr)
    return arr


def read_fasta(data: bytes, remove_duplicates: bool = False, n: int = 0):
    """read_fasta (src/hamming_impl.cc:200-242): (list of sequences as bytes,
    sequence_indices as uint64 array — empty without remove_duplicates)."""
    L = lib()
    seqs, offs, idx = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    nrec, nin = ctypes.c_uint64(), ctypes.c_uint64()
    _check(L.hdo_read_fasta(data, len(data), int(remove_duplicates), n, ctypes.byref(seqs),
                            ctypes.byref(offs), ctypes.byref(nrec), ctypes.byref(idx),
                            ctypes.byref(nin)))
    offsets = _take(offs.value, nrec.value + 1, np.uint64)
    total = int(offsets[-1]) if len(offsets) else 0
    raw = b""
    if seqs.value:
        # (c_char * n) copies any size; ctypes.string_at takes a C int size
        raw = bytes((ctypes.c_char * total).from_address(seqs.value)) if total else b""
        L.hdo_free(seqs.value)
    out = [raw[int(offsets[k]):int(offsets[k + 1])] for k in range(nrec.value)]
    indices = _take(idx.value, nin.value, np.uint64) if idx.value else np.zeros(0, np.uint64)
    return out, indices


def _concat(seqs):
    seqs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    offsets = np.zeros(len(seqs) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([len(s) for s in seqs]) if seqs else []
    return b"".join(seqs), offsets


def lt_cpu(seqs, include_x=False, max_distance=255, dtype=np.uint8):
    """distances<T>(use_gpu=False) (include/hamming/hamming_impl.hh:68-176):
    returns (lt array, used_sparse)."""
    raw, offsets = _concat(seqs)
    n = len(seqs)
    if n == 0:
        raise RuntimeError(ERRORS[-1])
    out = np.zeros(max(n * (n - 1) // 2, 1), dtype=dtype)
    used = ctypes.c_int(0)
    _check(lib().hdo_lt_cpu(raw, offsets.ctypes.data, n, int(include_x), int(max_distance),
                            np.dtype(dtype).itemsize, out.ctypes.data, ctypes.byref(used)))
    return out[: n * (n - 1) // 2], bool(used.value)


def pack_rows(seqs) -> np.ndarray:
    """to_dense_data / from_string (src/hamming_impl.cc:190-198, 244-267)."""
    L = lib()
    length = len(seqs[0])
    rb = L.hdo_packed_row_bytes(length)
    out = np.zeros((len(seqs), rb), dtype=np.uint8)
    for k, s in enumerate(seqs):
        s = s.encode() if isinstance(s, str) else bytes(s)
        L.hdo_pack_row(s, length, out[k].ctypes.data)
    return out


def lt_dense(seqs, max_distance=255, dtype=np.uint8) -> np.ndarray:
    """The dense AND-rule lower triangle (hamming_impl.hh:161-175; the rule of
    the reference GPU kernel src/distance_cuda.cu:57-65)."""
    if len(seqs) == 0 or len(seqs[0]) == 0:
        raise RuntimeError(ERRORS[-1])
    if any(len(s) != len(seqs[0]) for s in seqs):
        raise RuntimeError(ERRORS[-2])
    packed = pack_rows(seqs)
    n = len(seqs)
    out = np.zeros(max(n * (n - 1) // 2, 1), dtype=dtype)
    _check(lib().hdo_lt_dense(packed.ctypes.data, n, packed.shape[1], int(max_distance),
                              np.dtype(dtype).itemsize, out.ctypes.data))
    return out[: n * (n - 1) // 2]


def from_fasta_dense(data: bytes, remove_duplicates=False, n=0, max_distance=255,
                     dtype=np.uint8):
    """from_fasta(use_gpu=True) semantics on the CPU: (lt, sequence_indices).
    One pass over the text, as the reference's from_fasta
    (include/hamming/hamming.hh:168-178) reads its file once."""
    lt, nrows, idx, nin = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_void_p(), ctypes.c_uint64()
    _check(lib().hdo_from_fasta_dense_once(data, len(data), int(remove_duplicates), n,
                                           int(max_distance), np.dtype(dtype).itemsize,
                                           ctypes.byref(lt), ctypes.byref(nrows),
                                           ctypes.byref(idx), ctypes.byref(nin)))
    m = nrows.value
    out = _take(lt.value, m * (m - 1) // 2, dtype)
    ind = _take(idx.value, nin.value, np.uint64)
    return out, (ind if remove_duplicates else np.zeros(0, np.uint64))


def fasta_sequence_indices(data: bytes, n: int = 0) -> np.ndarray:
    """fasta_sequence_indices (src/hamming.cc:76-102)."""
    idx, nin = ctypes.c_void_p(), ctypes.c_uint64()
    _check(lib().hdo_fasta_sequence_indices(data, len(data), n, ctypes.byref(idx),
                                            ctypes.byref(nin)))
    return _take(idx.value, nin.value, np.uint64)


def reference_distances(ref, data: bytes, include_x=False) -> np.ndarray:
    """fasta_reference_distances (src/hamming.cc:104-141)."""
    ref = ref.encode() if isinstance(ref, str) else bytes(ref)
    out, nout = ctypes.c_void_p(), ctypes.c_uint64()
    _check(lib().hdo_reference_distances(ref, len(ref), data, len(data), int(include_x),
                                         ctypes.byref(out), ctypes.byref(nout)))
    return _take(out.value, nout.value, np.uint32)


def distance(s0, s1, include_x=False) -> int:
    """distance (src/hamming.cc:54-74)."""
    s0 = s0.encode() if isinstance(s0, str) else bytes(s0)
    s1 = s1.encode() if isinstance(s1, str) else bytes(s1)
    d = ctypes.c_uint32()
    _check(lib().hdo_distance(s0, len(s0), s1, len(s1), int(include_x), ctypes.byref(d)))
    return int(d.value)


def format_lower_triangular(lt: np.ndarray) -> bytes:
    """lower_triangular_lines (include/hamming/hamming_utils.hh:19-53)."""
    lt = np.ascontiguousarray(lt)
    L = lib()
    nb = L.hdo_format_lower_triangular(lt.ctypes.data, lt.size, lt.dtype.itemsize, None)
    buf = ctypes.create_string_buffer(max(int(nb), 1))
    L.hdo_format_lower_triangular(lt.ctypes.data, lt.size, lt.dtype.itemsize, buf)
    return buf.raw[: int(nb)]


def format_sparse(lt: np.ndarray, nsamples: int, threshold: int) -> bytes:
    """DataSet::dump_sparse (include/hamming/hamming.hh:79-114), serial order."""
    lt = np.ascontiguousarray(lt)
    L = lib()
    nl = ctypes.c_uint64()
    nb = L.hdo_format_sparse(lt.ctypes.data, nsamples, lt.dtype.itemsize, threshold, None,
                             ctypes.byref(nl))
    buf = ctypes.create_string_buffer(max(int(nb), 1))
    L.hdo_format_sparse(lt.ctypes.data, nsamples, lt.dtype.itemsize, threshold, buf,
                        ctypes.byref(nl))
    return buf.raw[: int(nb)]


def dump_full(lt: np.ndarray, nsamples: int, path: str) -> None:
    """DataSet::dump text (include/hamming/hamming.hh:63-73), one thread."""
    lt = np.ascontiguousarray(lt)
    _check(lib().hdo_dump_full(lt.ctypes.data if lt.size else None, lt.size, nsamples,
                               lt.dtype.itemsize, os.fsencode(path)))


def _read_values(fn, path, dtype, *lead):
    out, entries, n, kind = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_int()
    rc = fn(os.fsencode(path), *lead, ctypes.byref(out), ctypes.byref(entries), ctypes.byref(n),
            ctypes.byref(kind))
    if rc == -12:
        raise (IndexError if kind.value == 2 else ValueError)("stoi")
    _check(rc)
    return _take(out.value, entries.value, dtype), n.value


def read_lower_triangular(path: str, dtype=np.uint8):
    """from_lower_triangular<T> (hamming.hh:152-166), one thread: (values, nsamples)."""
    return _read_values(lib().hdo_read_lower_triangular, path, dtype, np.dtype(dtype).itemsize)


def read_csv(path: str):
    """from_csv (hamming.hh:34-55), one thread: (values, nsamples)."""
    return _read_values(lib().hdo_read_csv, path, np.uint8)


def num_threads() -> int:
    return int(lib().hdo_num_threads())
