"""ctypes binding of the libhd C ABI (include/hammingdist_gb300.h).

This is the binding a Python caller (or the reference's own bindings) would
add to reach the GPU path through plain pointers and sizes; the pybind11
module ``hammingdist_gb300._C`` is the C++ equivalent. Device pointers may be
passed as integers (e.g. ``torch.Tensor.data_ptr()``).
"""
from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np

from . import LIBHD_PATH

u64, i64, vp, cp, ci = ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int
P = ctypes.POINTER

# name -> (restype, argtypes); every function declared in the header
SIGNATURES = {
    "hd_device_available": (ci, []),
    "hd_ctx_create": (ci, [ci, P(vp)]),
    "hd_ctx_destroy": (None, [vp]),
    "hd_last_error": (cp, [vp]),
    "hd_ctx_kernel_launches": (u64, [vp]),
    "hd_host_alloc": (ci, [vp, ctypes.c_size_t, P(vp)]),
    "hd_host_free": (None, [vp, vp]),
    "hd_free": (None, [vp]),
    "hd_ctx_synchronize": (ci, [vp]),
    "hd_ctx_stream": (vp, [vp]),
    "hd_alignment_from_fasta": (ci, [vp, vp, u64, ci, ci, u64, ci, ci, P(vp)]),
    "hd_alignment_from_fasta_file": (ci, [vp, cp, ci, u64, ci, ci, P(vp)]),
    "hd_pairwise_lt_fasta_file": (ci, [vp, cp, ci, ci, i64, vp, vp, P(vp)]),
    "hd_alignment_from_sequences": (ci, [vp, vp, vp, u64, ci, ci, P(vp)]),
    "hd_alignment_info": (ci, [vp, P(u64), P(u64), P(u64), P(ci)]),
    "hd_alignment_sequence_indices": (ci, [vp, vp]),
    "hd_alignment_free": (None, [vp]),
    "hd_pairwise_lt": (ci, [vp, vp, ci, i64, vp, ci]),
    "hd_pairwise_lt_to_file": (ci, [vp, vp, i64, cp]),
    "hd_write_lower_triangular": (ci, [vp, vp, u64, ci, cp]),
    "hd_write_sparse": (ci, [vp, vp, u64, ci, i64, cp, P(u64)]),
    "hd_lower_triangular_text_noalloc": (ci, [vp, vp, u64, ci, vp, u64, P(u64)]),
    "hd_reference_distances": (ci, [vp, vp, u64, vp, u64, ci, P(vp), P(u64)]),
    "hd_reference_distances_file": (ci, [vp, vp, u64, cp, ci, P(vp), P(u64)]),
    "hd_alignment_reference_distances": (ci, [vp, vp, vp, u64, ci, vp]),
    "hd_fasta_sequence_indices": (ci, [vp, vp, u64, u64, P(vp), P(u64)]),
    "hd_fasta_sequence_indices_file": (ci, [vp, cp, u64, P(vp), P(u64)]),
    "hd_distance": (ci, [vp, vp, u64, vp, u64, ci, P(ctypes.c_uint32)]),
    "hd_batch_create": (ci, [vp, P(vp)]),
    "hd_batch_add": (ci, [vp, vp, ci, i64, vp, ci]),
    "hd_batch_run": (ci, [vp]),
    "hd_batch_timing": (ci, [vp, P(ctypes.c_double), P(u64), P(u64)]),
    "hd_batch_free": (None, [vp]),
    "hd_alignments_from_fasta_many": (ci, [vp, u64, P(vp), P(u64), ci, u64, ci, ci, P(vp)]),
    "hd_alignments_from_fasta_files": (ci, [vp, u64, P(cp), ci, u64, ci, ci, P(vp)]),
    "hd_alignment_view": (ci, [vp, u64, u64, P(vp)]),
    "hd_synthetic_fasta": (ci, [vp, u64, u64, ctypes.c_double, u64, ctypes.c_uint32,
                                ctypes.c_double, vp, u64, P(u64)]),
    "hd_server_create": (ci, [vp, u64, ci, P(vp)]),
    "hd_server_add_alignment": (ci, [vp, vp, P(ctypes.c_uint32)]),
    "hd_server_submit_reference": (ci, [vp, ctypes.c_uint32, vp, u64, P(u64)]),
    "hd_server_submit_pairwise": (ci, [vp, ctypes.c_uint32, u64, u64, ci, i64, P(u64)]),
    "hd_server_submit_sparse": (ci, [vp, ctypes.c_uint32, u64, u64, i64, P(u64)]),
    "hd_server_wait": (ci, [vp, u64, ctypes.c_double]),
    "hd_server_result": (ci, [vp, u64, P(vp), P(u64), P(u64), P(ctypes.c_double),
                              P(ctypes.c_double)]),
    "hd_server_release": (ci, [vp, u64]),
    "hd_server_cancel": (ci, [vp, u64]),
    "hd_selftest_wait_timeout": (ci, [vp, u64, P(ci), P(ctypes.c_double)]),
    "hd_server_stats": (ci, [vp, P(u64), P(u64), P(u64), P(u64)]),
    "hd_server_free": (None, [vp]),
    "hd_autotune": (ci, [vp, u64]),
    "hd_tune_lookup": (ci, [vp, u64, u64, ci, P(ci), P(ci)]),
    "hd_tune_lookup_mma": (ci, [vp, u64, u64, ci, P(ci), P(ci), P(u64)]),
    "hd_tune_save": (ci, [vp, cp]),
    "hd_tune_load": (ci, [vp, cp]),
    "hd_pairwise_lt_files": (ci, [vp, u64, vp, ci, u64, ci, ci, vp, vp, vp, vp, vp]),
    "hd_write_full_matrix": (ci, [vp, vp, u64, u64, ci, cp]),
    "hd_read_lower_triangular": (ci, [vp, cp, ci, vp, vp, P(u64), P(u64), P(ci)]),
    "hd_read_csv": (ci, [vp, cp, vp, vp, P(u64), P(u64), P(ci)]),
    "hd_trace_enable": (ci, [vp, ctypes.c_int]),
    "hd_trace_last": (ctypes.c_char_p, [vp]),
    "hd_measure_int_peaks": (ci, [vp, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]),
    "hd_measure_mma_peak": (ci, [vp, P(ctypes.c_double)]),
    "hd_last_pairwise_timing": (ci, [vp, P(ctypes.c_double), P(u64)]),
    "hd_last_pairwise_work": (ci, [vp, P(ctypes.c_double)]),
}

SEM_GPU, SEM_CPU = 0, 1
RULES = {0: "and", 1: "sparse", 2: "sparse_x"}

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIBHD_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


# void *(*hd_output_fn)(void *user, uint64_t index, uint64_t n_rows, uint64_t entries)
OUTPUT_FN = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                             ctypes.c_uint64)
# hd_pairwise_lt_fasta_file's request for a second copy of its result
OUTPUT_MIRROR = 2**64 - 1


class HDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _ptr(x):
    """Host buffer (bytes / numpy) or device pointer (int) -> c_void_p."""
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    if isinstance(x, np.ndarray):
        return ctypes.c_void_p(x.ctypes.data)
    if isinstance(x, (bytes, bytearray)):
        return ctypes.cast(ctypes.c_char_p(bytes(x)), ctypes.c_void_p)
    raise TypeError(type(x))


class Alignment:
    def __init__(self, ctx: "Context", handle):
        self.ctx, self.h = ctx, handle
        ctx._owned.add(self)
        n_rows, length, n_in, rule = u64(), u64(), u64(), ci()
        ctx._check(lib().hd_alignment_info(handle, ctypes.byref(n_rows), ctypes.byref(length),
                                           ctypes.byref(n_in), ctypes.byref(rule)))
        self.n_rows, self.length, self.n_input = n_rows.value, length.value, n_in.value
        self.rule = RULES[rule.value]

    def view(self, row0: int, n_rows: int) -> "Alignment":
        """Rows [row0, row0 + n_rows) (borrows this alignment's memory)."""
        v = vp()
        self.ctx._check(lib().hd_alignment_view(self.h, row0, n_rows, ctypes.byref(v)))
        out = Alignment(self.ctx, v)
        out._base = self  # keep the base alive while the view is
        return out

    def sequence_indices(self) -> np.ndarray:
        out = np.zeros(max(self.n_input, 1), dtype=np.uint64)
        self.ctx._check(lib().hd_alignment_sequence_indices(self.h, out.ctypes.data))
        return out[: self.n_input]

    def free(self):
        if self.h:
            lib().hd_alignment_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    def __init__(self, device: int = 0):
        h = vp()
        rc = lib().hd_ctx_create(device, ctypes.byref(h))
        if rc != 0:
            raise HDError(rc, f"hd_ctx_create failed ({rc})")
        self.h = h
        self._owned = weakref.WeakSet()  # alignments and batches made here

    def close(self):
        if self.h:
            # servers use resident alignments in flight; views borrow their bases
            def order(o):
                return (0 if isinstance(o, Server) else 1 if isinstance(o, Batch) else
                        2 if getattr(o, "_base", None) is not None else 3)
            for obj in sorted(list(self._owned), key=order):
                obj.free()
            lib().hd_ctx_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise HDError(rc, (lib().hd_last_error(self.h) or b"").decode())

    @property
    def kernel_launches(self) -> int:
        return int(lib().hd_ctx_kernel_launches(self.h))

    @property
    def stream(self) -> int:
        """cudaStream_t of the context (for torch.cuda.ExternalStream)."""
        return int(lib().hd_ctx_stream(self.h) or 0)

    def synchronize(self):
        self._check(lib().hd_ctx_synchronize(self.h))

    def alignment_from_fasta(self, data, nbytes=None, on_device=False, remove_duplicates=False,
                             n=0, include_x=False, semantics=SEM_GPU) -> Alignment:
        if nbytes is None:
            nbytes = len(data)
        a = vp()
        self._check(lib().hd_alignment_from_fasta(self.h, _ptr(data), nbytes, int(on_device),
                                                  int(remove_duplicates), n, int(include_x),
                                                  semantics, ctypes.byref(a)))
        return Alignment(self, a)

    def alignment_from_fasta_file(self, path, remove_duplicates=False, n=0, include_x=False,
                                  semantics=SEM_GPU) -> Alignment:
        a = vp()
        self._check(lib().hd_alignment_from_fasta_file(self.h, os.fsencode(path),
                                                       int(remove_duplicates), n,
                                                       int(include_x), semantics,
                                                       ctypes.byref(a)))
        return Alignment(self, a)

    def pairwise_lt_fasta_file(self, path, dtype=np.uint8, max_distance=None,
                               remove_duplicates=False, mirror=False):
        """from_fasta(use_gpu=True) of a file in one call (distances overlap
        the read for large files): (lower triangle, Alignment), and with
        mirror=True also the second copy the library writes on request
        (HD_OUTPUT_MIRROR)."""
        dt = np.dtype(dtype)
        md = np.iinfo(dt).max if max_distance is None else max_distance
        box = {}

        @OUTPUT_FN
        def alloc(user, index, n_rows, entries):
            key = "lt"
            if index == OUTPUT_MIRROR:
                if not mirror:
                    return None
                key = "mirror"
            arr = np.empty(max(int(entries), 1), dtype=dt)
            box[key] = arr[: int(entries)]
            return arr.ctypes.data

        a = vp()
        self._check(lib().hd_pairwise_lt_fasta_file(self.h, os.fsencode(path),
                                                    int(remove_duplicates), dt.itemsize, int(md),
                                                    ctypes.cast(alloc, vp), None,
                                                    ctypes.byref(a)))
        if mirror:
            return box["lt"], Alignment(self, a), box.get("mirror")
        return box["lt"], Alignment(self, a)

    def alignment_from_sequences(self, seqs, include_x=False, semantics=SEM_GPU) -> Alignment:
        seqs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        raw = b"".join(seqs)
        offs = np.zeros(len(seqs) + 1, dtype=np.uint64)
        offs[1:] = np.cumsum([len(s) for s in seqs]) if seqs else []
        a = vp()
        self._check(lib().hd_alignment_from_sequences(self.h, _ptr(raw), offs.ctypes.data,
                                                      len(seqs), int(include_x), semantics,
                                                      ctypes.byref(a)))
        return Alignment(self, a)

    def pairwise_lt(self, aln: Alignment, dtype=np.uint8, max_distance=255, out=None,
                    out_on_device=False):
        """Host numpy result, or writes to a device pointer `out` (int)."""
        dt = np.dtype(dtype)
        n = aln.n_rows
        if out is None:
            out = np.zeros(max(n * (n - 1) // 2, 1), dtype=dt)
            self._check(lib().hd_pairwise_lt(self.h, aln.h, dt.itemsize, int(max_distance),
                                             out.ctypes.data, 0))
            return out[: n * (n - 1) // 2]
        self._check(lib().hd_pairwise_lt(self.h, aln.h, dt.itemsize, int(max_distance), _ptr(out),
                                         int(out_on_device)))
        return out

    def pairwise_lt_to_file(self, aln: Alignment, max_distance: int, path: str):
        self._check(lib().hd_pairwise_lt_to_file(self.h, aln.h, int(max_distance), path.encode()))

    def write_lower_triangular(self, lt: np.ndarray, nsamples: int, path: str):
        lt = np.ascontiguousarray(lt)
        self._check(lib().hd_write_lower_triangular(self.h, lt.ctypes.data, nsamples,
                                                    lt.dtype.itemsize, path.encode()))

    def write_sparse(self, lt: np.ndarray, nsamples: int, threshold: int, path: str) -> int:
        lt = np.ascontiguousarray(lt)
        nl = u64()
        self._check(lib().hd_write_sparse(self.h, lt.ctypes.data, nsamples, lt.dtype.itemsize,
                                          threshold, path.encode(), ctypes.byref(nl)))
        return nl.value

    def lower_triangular_text_noalloc(self, d_lt: int, nsamples: int, dtype, d_text: int,
                                      capacity: int) -> int:
        """Formats a device lower triangle into a device text buffer without
        allocating device memory; returns the number of text bytes."""
        nb = u64()
        self._check(lib().hd_lower_triangular_text_noalloc(
            self.h, _ptr(d_lt), nsamples, np.dtype(dtype).itemsize, _ptr(d_text), capacity,
            ctypes.byref(nb)))
        return nb.value

    def reference_distances(self, ref, data: bytes, include_x=False) -> np.ndarray:
        ref = ref.encode() if isinstance(ref, str) else bytes(ref)
        out, n = vp(), u64()
        self._check(lib().hd_reference_distances(self.h, _ptr(ref), len(ref),
                                                 _ptr(data), len(data), int(include_x),
                                                 ctypes.byref(out), ctypes.byref(n)))
        return _take(out, n.value, np.uint32)

    def reference_distances_file(self, ref, path, include_x=False) -> np.ndarray:
        ref = ref.encode() if isinstance(ref, str) else bytes(ref)
        out, n = vp(), u64()
        self._check(lib().hd_reference_distances_file(self.h, _ptr(ref), len(ref),
                                                      os.fsencode(path), int(include_x),
                                                      ctypes.byref(out), ctypes.byref(n)))
        return _take(out, n.value, np.uint32)

    def alignment_reference_distances(self, aln: Alignment, ref) -> np.ndarray:
        ref = ref.encode() if isinstance(ref, str) else bytes(ref)
        out = np.zeros(max(aln.n_input, 1), dtype=np.uint32)
        self._check(lib().hd_alignment_reference_distances(self.h, aln.h, _ptr(ref),
                                                           len(ref), 0, out.ctypes.data))
        return out[: aln.n_input]

    def fasta_sequence_indices(self, data: bytes, n=0) -> np.ndarray:
        out, cnt = vp(), u64()
        self._check(lib().hd_fasta_sequence_indices(self.h, _ptr(data), len(data), n,
                                                    ctypes.byref(out), ctypes.byref(cnt)))
        return _take(out, cnt.value, np.uint64)

    def fasta_sequence_indices_file(self, path, n=0) -> np.ndarray:
        out, cnt = vp(), u64()
        self._check(lib().hd_fasta_sequence_indices_file(self.h, os.fsencode(path), n,
                                                         ctypes.byref(out), ctypes.byref(cnt)))
        return _take(out, cnt.value, np.uint64)

    def distance(self, s0, s1, include_x=False) -> int:
        s0 = s0.encode() if isinstance(s0, str) else bytes(s0)
        s1 = s1.encode() if isinstance(s1, str) else bytes(s1)
        d = ctypes.c_uint32()
        self._check(lib().hd_distance(self.h, _ptr(s0), len(s0), _ptr(s1), len(s1),
                                      int(include_x), ctypes.byref(d)))
        return int(d.value)

    def alignments_from_fasta_many(self, datas, remove_duplicates=False, n=0, include_x=False,
                                   semantics=SEM_GPU):
        """Several alignments ingested concurrently (one per FASTA buffer)."""
        k = len(datas)
        bufs = (vp * k)(*[ctypes.cast(ctypes.c_char_p(d), vp) for d in datas])
        sizes = (u64 * k)(*[len(d) for d in datas])
        outs = (vp * k)()
        self._check(lib().hd_alignments_from_fasta_many(self.h, k, bufs, sizes,
                                                        int(remove_duplicates), n, int(include_x),
                                                        semantics, outs))
        return [Alignment(self, vp(outs[i])) for i in range(k)]

    def alignments_from_fasta_files(self, paths, remove_duplicates=False, n=0, include_x=False,
                                    semantics=SEM_GPU):
        """Several alignments from FASTA files: reads overlap device ingest."""
        k = len(paths)
        arr = (cp * k)(*[p.encode() for p in paths])
        outs = (vp * k)()
        self._check(lib().hd_alignments_from_fasta_files(self.h, k, arr, int(remove_duplicates), n,
                                                         int(include_x), semantics, outs))
        return [Alignment(self, vp(outs[i])) for i in range(k)]

    def synthetic_fasta(self, n, L, p=1e-3, seed=0, dash_max=200, n_rate=1e-4, out=None):
        """Seeded synthetic FASTA written on the device; returns the byte count
        (and writes into the device pointer `out` when given)."""
        nb = u64()
        self._check(lib().hd_synthetic_fasta(self.h, n, L, p, seed, dash_max, n_rate,
                                             _ptr(out) if out is not None else None,
                                             (1 << 63) if out is not None else 0,
                                             ctypes.byref(nb)))
        return nb.value

    def server(self, output_budget_bytes=8 << 30, max_waves=3) -> "Server":
        return Server(self, output_budget_bytes, max_waves)

    def batch(self) -> "Batch":
        return Batch(self)

    def autotune(self, max_n_bucket=6):
        self._check(lib().hd_autotune(self.h, max_n_bucket))

    def tune_lookup(self, n_rows, length, dtype):
        t, s = ci(), ci()
        self._check(lib().hd_tune_lookup(self.h, n_rows, length, np.dtype(dtype).itemsize,
                                         ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    def tune_lookup_mma(self, n_rows, length, dtype):
        """(band, row tiles per item, minimum launch items) of the tensor-core
        engine for a matrix of n_rows x length sites."""
        b, r, m = ci(), ci(), u64()
        self._check(lib().hd_tune_lookup_mma(self.h, n_rows, length, np.dtype(dtype).itemsize,
                                             ctypes.byref(b), ctypes.byref(r), ctypes.byref(m)))
        return b.value, r.value, m.value

    def tune_save(self, path):
        self._check(lib().hd_tune_save(self.h, path.encode()))

    def tune_load(self, path):
        self._check(lib().hd_tune_load(self.h, path.encode()))

    def selftest_wait_timeout(self, limit_ns=1_000_000):
        """(status, waited_ms) of a bounded wait that is made to run out."""
        st, ms = ci(), ctypes.c_double()
        self._check(lib().hd_selftest_wait_timeout(self.h, limit_ns, ctypes.byref(st),
                                                   ctypes.byref(ms)))
        return st.value, ms.value

    def pairwise_lt_files(self, paths, dtypes=None, max_distances=None, remove_duplicates=False,
                          n=0, include_x=False, semantics=SEM_GPU):
        """Lower triangles of many FASTA files through the pipelined file
        batch (hd_pairwise_lt_files). Returns (list of arrays, list of
        sequence-index arrays)."""
        k = len(paths)
        dtypes = [np.dtype(d if d is not None else np.uint8) for d in (dtypes or [None] * k)]
        mds = max_distances or [np.iinfo(d).max for d in dtypes]
        outs = [None] * k

        @OUTPUT_FN
        def alloc(user, index, n_rows, entries):
            if index == OUTPUT_MIRROR:
                return None
            arr = np.empty(max(int(entries), 1), dtype=dtypes[index])
            outs[index] = arr[: int(entries)]
            return arr.ctypes.data

        raw = [os.fsencode(p) for p in paths]
        c_paths = (ctypes.c_char_p * k)(*raw)
        c_dt = (ctypes.c_int * k)(*[d.itemsize for d in dtypes])
        c_md = (ctypes.c_int64 * k)(*[int(m) for m in mds])
        handles = (vp * k)()
        self._check(lib().hd_pairwise_lt_files(self.h, k, ctypes.cast(c_paths, vp),
                                               int(remove_duplicates), n, int(include_x),
                                               semantics, ctypes.cast(c_dt, vp),
                                               ctypes.cast(c_md, vp),
                                               ctypes.cast(alloc, vp), None,
                                               ctypes.cast(handles, vp)))
        idx = []
        for h in handles:
            a = Alignment(self, h)
            idx.append(a.sequence_indices())
            a.free()
        return outs, idx

    def write_full_matrix(self, lt, nsamples, path):
        """DataSet::dump text of a host lower triangle (hd_write_full_matrix)."""
        lt = np.ascontiguousarray(lt)
        self._check(lib().hd_write_full_matrix(self.h, lt.ctypes.data if lt.size else None,
                                               lt.size, nsamples, lt.dtype.itemsize,
                                               os.fsencode(path)))

    def _read_values(self, fn, path, dtype, *lead):
        box = {}

        @OUTPUT_FN
        def alloc(user, index, n, entries):
            arr = np.empty(max(int(entries), 1), dtype=dtype)
            box["arr"], box["n"] = arr[: int(entries)], int(n)
            return arr.ctypes.data

        entries, n, kind = u64(), u64(), ci()
        rc = fn(self.h, os.fsencode(path), *lead, ctypes.cast(alloc, vp), None,
                ctypes.byref(entries), ctypes.byref(n), ctypes.byref(kind))
        if rc == -12:
            err = HDError(rc, "stoi")
            err.parse_error = kind.value
            raise err
        self._check(rc)
        return box["arr"], box["n"]

    def read_lower_triangular(self, path, dtype=np.uint8):
        """from_lower_triangular on the device: (values, nsamples)."""
        return self._read_values(lib().hd_read_lower_triangular, path, dtype,
                                 np.dtype(dtype).itemsize)

    def read_csv(self, path):
        """from_csv on the device: (values, nsamples)."""
        return self._read_values(lib().hd_read_csv, path, np.uint8)

    def trace(self, on=True):
        """Turns per-phase tracing of this context's calls on or off."""
        self._check(lib().hd_trace_enable(self.h, 1 if on else 0))

    def trace_last(self):
        """Text of the last traced call: phases with their stream times."""
        return (lib().hd_trace_last(self.h) or b"").decode()

    def measure_int_peaks(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(lib().hd_measure_int_peaks(self.h, ctypes.byref(a), ctypes.byref(b),
                                               ctypes.byref(c)))
        return {"lop3_per_s": a.value, "popc_per_s": b.value, "mix_pair_sites_per_s": c.value}

    def measure_mma_peak(self):
        """Dense FP4 (kind::mxf4) tensor-core FLOP/s (hd_measure_mma_peak)."""
        f = ctypes.c_double()
        self._check(lib().hd_measure_mma_peak(self.h, ctypes.byref(f)))
        return f.value

    def last_pairwise_timing(self):
        ms, tiles = ctypes.c_double(), u64()
        self._check(lib().hd_last_pairwise_timing(self.h, ctypes.byref(ms), ctypes.byref(tiles)))
        return ms.value, tiles.value

    def last_pairwise_work(self):
        """Multiply-adds of the last pairwise call's tensor-core launches."""
        m = ctypes.c_double()
        self._check(lib().hd_last_pairwise_work(self.h, ctypes.byref(m)))
        return m.value


class Batch:
    """Independent matrices computed together by the persistent engine; the
    launches are captured in a CUDA graph on the first run and replayed."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = vp()
        ctx._check(lib().hd_batch_create(ctx.h, ctypes.byref(h)))
        self.h = h
        self.outputs = []
        ctx._owned.add(self)

    def add(self, aln: Alignment, dtype=np.uint8, max_distance=255, out=None, out_on_device=False):
        dt = np.dtype(dtype)
        if out is None:
            n = aln.n_rows
            out = np.zeros(max(n * (n - 1) // 2, 1), dtype=dt)
            self.outputs.append((out, n * (n - 1) // 2))
            ptr = out.ctypes.data
        else:
            self.outputs.append((None, 0))
            ptr = _ptr(out)
        self.ctx._check(lib().hd_batch_add(self.h, aln.h, dt.itemsize, int(max_distance), ptr,
                                           int(out_on_device)))
        return len(self.outputs) - 1

    def run(self):
        self.ctx._check(lib().hd_batch_run(self.h))
        return [o[: n] if o is not None else None for o, n in self.outputs]

    def timing(self):
        ms, launches, tiles = ctypes.c_double(), u64(), u64()
        self.ctx._check(lib().hd_batch_timing(self.h, ctypes.byref(ms), ctypes.byref(launches),
                                              ctypes.byref(tiles)))
        return ms.value, launches.value, tiles.value

    def free(self):
        if self.h:
            lib().hd_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Request loop over resident alignments with continuous batching
    (hd_server_*). Results: uint32 array (reference), dtype array
    (pairwise), bytes (sparse text)."""

    KINDS = {}

    def __init__(self, ctx: Context, budget: int, max_waves: int):
        self.ctx = ctx
        h = vp()
        ctx._check(lib().hd_server_create(ctx.h, budget, max_waves, ctypes.byref(h)))
        self.h = h
        self._kind = {}
        self._keep = []
        ctx._owned.add(self)

    def add(self, aln: Alignment) -> int:
        i = ctypes.c_uint32()
        self.ctx._check(lib().hd_server_add_alignment(self.h, aln.h, ctypes.byref(i)))
        self._keep.append(aln)
        return i.value

    def reference(self, aln_id: int, query) -> int:
        q = query.encode() if isinstance(query, str) else bytes(query)
        t = u64()
        self.ctx._check(lib().hd_server_submit_reference(self.h, aln_id, _ptr(q), len(q),
                                                         ctypes.byref(t)))
        self._kind[t.value] = ("ref", np.uint32)
        return t.value

    def pairwise(self, aln_id: int, row0: int, n_rows: int, dtype=np.uint8, max_distance=255):
        t = u64()
        dt = np.dtype(dtype)
        self.ctx._check(lib().hd_server_submit_pairwise(self.h, aln_id, row0, n_rows, dt.itemsize,
                                                        int(max_distance), ctypes.byref(t)))
        self._kind[t.value] = ("pair", dt)
        return t.value

    def sparse(self, aln_id: int, row0: int, n_rows: int, threshold: int) -> int:
        t = u64()
        self.ctx._check(lib().hd_server_submit_sparse(self.h, aln_id, row0, n_rows, threshold,
                                                      ctypes.byref(t)))
        self._kind[t.value] = ("sparse", None)
        return t.value

    def wait(self, ticket: int, timeout: float = 60.0):
        self.ctx._check(lib().hd_server_wait(self.h, ticket, timeout))

    def result(self, ticket: int, release: bool = True):
        """(value, count, latency_ms, queue_ms) of a finished request."""
        data, nb, cnt = vp(), u64(), u64()
        lat, q = ctypes.c_double(), ctypes.c_double()
        self.ctx._check(lib().hd_server_result(self.h, ticket, ctypes.byref(data), ctypes.byref(nb),
                                               ctypes.byref(cnt), ctypes.byref(lat),
                                               ctypes.byref(q)))
        raw = ctypes.string_at(data.value, nb.value) if nb.value else b""
        kind, dt = self._kind.pop(ticket)
        value = raw if kind == "sparse" else np.frombuffer(raw, dtype=dt).copy()
        if release:
            lib().hd_server_release(self.h, ticket)
        return value, cnt.value, lat.value, q.value

    def cancel(self, ticket: int):
        self.ctx._check(lib().hd_server_cancel(self.h, ticket))
        self._kind.pop(ticket, None)

    def stats(self):
        w, c, m, b = u64(), u64(), u64(), u64()
        self.ctx._check(lib().hd_server_stats(self.h, ctypes.byref(w), ctypes.byref(c),
                                              ctypes.byref(m), ctypes.byref(b)))
        return {"waves": w.value, "completed": c.value, "max_inflight": m.value,
                "bytes_in_use": b.value}

    def free(self):
        if self.h:
            lib().hd_server_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _take(ptr: ctypes.c_void_p, n: int, dtype) -> np.ndarray:
    if not ptr.value:
        return np.zeros(0, dtype=dtype)
    nbytes = n * np.dtype(dtype).itemsize
    arr = np.frombuffer(ctypes.string_at(ptr.value, nbytes), dtype=dtype).copy() if n else \
        np.zeros(0, dtype=dtype)
    lib().hd_free(ptr)
    return arr
