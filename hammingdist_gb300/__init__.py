"""GB300 (sm_103a) implementation of hammingdist's pairwise Hamming-distance
path, with the reference's Python API (ssciwr/hammingdist 1.4.0,
python/hammingdist.cc).

All distances are computed by this package's CUDA kernels (libhd.so); there
is no CPU path. Importing fails loudly if the native build is missing: run
``python hammingdist_gb300/build.py`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import os as _os
import sysconfig as _sysconfig

_PKG = _os.path.dirname(_os.path.abspath(__file__))
_EXT = _os.path.join(_PKG, "_C" + _sysconfig.get_config_var("EXT_SUFFIX"))
if not _os.path.exists(_EXT) or not _os.path.exists(_os.path.join(_PKG, "libhd.so")):
    raise ImportError(
        "hammingdist_gb300: native extension not built (libhd.so / _C). "
        "Run `python hammingdist_gb300/build.py` first; there is no CPU fallback.")

# measured kernel configurations for GB300 (applied only on a matching device)
_os.environ.setdefault("HAMMINGDIST_TUNING", _os.path.join(_PKG, "tuning", "gb300.json"))

from ._C import (  # noqa: E402,F401
    DataSet,
    DataSetLarge,
    autotune,
    cuda_gpu_available,
    distance,
    fasta_reference_distances,
    fasta_sequence_indices,
    from_csv,
    from_fasta,
    from_fasta_batch,
    from_fasta_device,
    from_fasta_large,
    from_fasta_to_lower_triangular,
    from_lower_triangular,
    from_lower_triangular_large,
    from_stringlist,
    load_tuning,
    _kernel_launches,
    _stream,
)

LIBHD_PATH = _os.path.join(_PKG, "libhd.so")
