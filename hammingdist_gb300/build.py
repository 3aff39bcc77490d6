"""In-tree build of the native parts for sm_103a (GB300).

  libhd.so    — the CUDA kernels + the C ABI of include/hammingdist_gb300.h
                (nvcc, one -gencode, static cudart)
  _C*.so      — the pybind11 module mirroring the reference's Python API,
                linked against libhd.so (g++, pybind11 headers from torch)

Both land in this package directory. Sources are compiled in parallel and
only when newer than their outputs.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
CU_SOURCES = ["hd_ingest.cu", "hd_pairwise.cu", "hd_mma.cu", "hd_format.cu", "hd_results.cu", "hd_peak.cu", "hd_tune.cu",
              "hd_synth.cu", "hd_server.cu", "hd_api.cu"]
GENCODE = "arch=compute_103a,code=sm_103a"
LIBHD = os.path.join(PKG, "libhd.so")
EXT = os.path.join(PKG, "_C" + sysconfig.get_config_var("EXT_SUFFIX"))


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "hammingdist_gb300.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _run_all(cmds: list[list[str]], verbose: bool) -> None:
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(c), flush=True)
        procs.append((c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{o}" for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def _arch_stamp_ok() -> bool:
    """Outputs built on another machine architecture are rebuilt."""
    stamp = os.path.join(BUILD, "ARCH")
    ok = os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()
    if not ok:
        for f in [LIBHD, EXT] + [os.path.join(BUILD, x) for x in os.listdir(BUILD)]:
            if os.path.isfile(f):
                os.remove(f)
        with open(stamp, "w") as fh:
            fh.write(platform.machine())
    return ok


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    _arch_stamp_ok()
    nvcc = _nvcc()
    hdrs = _headers()
    objs, cmds = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            c = [nvcc, "-gencode", GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                 "-I", INCLUDE, "-c", s, "-o", o]
            if ptxas_verbose:
                c.insert(1, "-Xptxas=-v")
            cmds.append(c)
    _run_all(cmds, verbose)
    if _stale(LIBHD, objs):
        tmp = LIBHD + f".tmp{os.getpid()}"
        _run_all([[nvcc, "-shared", "-gencode", GENCODE, "-o", tmp] + objs], verbose)
        os.replace(tmp, LIBHD)
    mod_src = os.path.join(CSRC, "hd_module.cpp")
    if _stale(EXT, [mod_src, LIBHD] + hdrs):
        import torch  # pybind11 headers ship inside the torch wheel

        tinc = os.path.join(os.path.dirname(torch.__file__), "include")
        pyinc = sysconfig.get_paths()["include"]
        tmp = EXT + f".tmp{os.getpid()}"
        _run_all([["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
                   "-I", INCLUDE, "-isystem", tinc, "-isystem", pyinc, mod_src, "-o", tmp,
                   "-L", PKG, "-lhd", "-Wl,-rpath,$ORIGIN", "-pthread"]], verbose)
        os.replace(tmp, EXT)
    return EXT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print("built", LIBHD, EXT)
