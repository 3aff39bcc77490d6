"""CPU-side checks of the boundary: libhd loads, exports every entry point the
header declares, and the product path refuses to run without a GPU (no CPU
fallback). No kernel is launched here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hammingdist_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hd_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("hd_alignment_from_fasta", "hd_pairwise_lt", "hd_pairwise_lt_to_file",
                 "hd_write_sparse", "hd_reference_distances", "hd_fasta_sequence_indices",
                 "hd_device_available", "hd_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import hammingdist_gb300
    from hammingdist_gb300 import abi

    lib = ctypes.CDLL(hammingdist_gb300.LIBHD_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name
    # the ctypes binding covers the whole header
    assert set(abi.SIGNATURES) == set(declared_functions())
    abi.lib()  # argtypes/restype assignment succeeds for every symbol


def test_extension_module_surface_matches_reference_api():
    import hammingdist_gb300 as hd

    for name in ("from_fasta", "from_fasta_large", "from_fasta_to_lower_triangular",
                 "fasta_reference_distances", "fasta_sequence_indices", "distance",
                 "from_stringlist", "from_csv", "from_lower_triangular",
                 "from_lower_triangular_large", "cuda_gpu_available", "DataSet", "DataSetLarge"):
        assert hasattr(hd, name), name
    for cls in (hd.DataSet, hd.DataSetLarge):
        for attr in ("dump", "dump_lower_triangular", "dump_sparse", "dump_sequence_indices",
                     "__getitem__", "_distances", "lt_array"):
            assert hasattr(cls, attr), attr
    def default(fn, arg):
        m = re.search(arg + r": [\w.]+ = (\w+)", fn.__doc__)
        return m.group(1) if m else None

    assert default(hd.from_fasta, "include_x") == "False"
    assert default(hd.from_fasta, "use_gpu") == "False"
    assert default(hd.from_fasta, "max_distance") == "255"
    assert default(hd.from_fasta_large, "max_distance") == "65535"
    assert default(hd.from_fasta_to_lower_triangular, "use_gpu") == "True"
    assert default(hd.from_fasta_to_lower_triangular, "max_distance") == "65535"
    assert default(hd.fasta_reference_distances, "include_x") == "False"
    assert default(hd.fasta_sequence_indices, "n") == "0"


def test_no_cpu_fallback_without_device():
    import hammingdist_gb300 as hd
    from hammingdist_gb300 import abi

    if abi.lib().hd_device_available():
        pytest.skip("a GPU is present")
    assert hd.cuda_gpu_available() is False
    with pytest.raises(RuntimeError, match="no CUDA device"):
        hd.distance("ACGT", "ACGA")
    h = ctypes.c_void_p()
    assert abi.lib().hd_ctx_create(0, ctypes.byref(h)) == -8  # HD_ERR_NO_DEVICE


def test_import_fails_loudly_without_native_build(tmp_path):
    import shutil
    import subprocess
    import sys

    pkg = tmp_path / "hammingdist_gb300"
    pkg.mkdir()
    shutil.copy(os.path.join(ROOT, "hammingdist_gb300", "__init__.py"), pkg / "__init__.py")
    r = subprocess.run([sys.executable, "-c", "import hammingdist_gb300"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode != 0 and "no CPU fallback" in r.stderr
