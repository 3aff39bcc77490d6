"""Benchmark of the pairwise Hamming-distance path on one GB300.

Workload (the reference's headline matrix): n=20,000 aligned sequences of
L=29,903 sites (seeded synthetic SARS-CoV-2-like alignment: substitution
p=1e-3, '-' runs of 0-200 at both ends, N runs at rate 1e-4), 30% exact
duplicates; from_fasta(use_gpu=True, remove_duplicates=True,
max_distance=255) -> uint8 lower triangle of the ~14,000 unique rows + the
sequence indices, plus fasta_reference_distances of the root sequence
against all 20,000 records.

One step = that whole pass. Metric = unique pairs x L / step time
(Gpair-sites/s).
  value : FASTA bytes already resident in HBM; parse + dedupe + pack +
          distance kernel + reference distances, all on the device, results
          left in HBM. Timed with CUDA events on the library's stream.
  e2e   : the public API a user calls (hammingdist_gb300.from_fasta(file) +
          .lt_array + fasta_reference_distances(root, file)): file -> pinned
          host buffer -> device -> host results, every step. The file is read
          and uploaded once per step (its mtime changes before each step; the
          read and the upload overlap); the second call finds the same
          unchanged file already on the device.
Inputs are larger than L2 (598 MB of FASTA text, 209 MB of packed rows), so
no L2 flush is needed between steps.

--impl reference times the reference's CPU algorithm (the oracle: the
reference compiled from source where available, else the C restatement in
oracle/) on the host cores, on a bounded sample of the same workload.

Other workloads, each printing its own JSON line: --small (n=1,000
from_fasta vs the CPU port), --formats (dump / from_lower_triangular /
from_csv of the headline matrix vs the CPU port), --kernel-only (the pairwise kernel alone),
--batched (64 uneven alignments), --streaming (from_fasta_large n=50,000,
from_fasta_to_lower_triangular n=100,000, dump_sparse), --serve (Poisson
request stream over resident alignments).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpair-sites/s n=20k L=29903 (bit-exact)"
N, L, P_SUB, DUP, SEED = 20000, 29903, 1e-3, 0.3, 2024
WORKLOAD = "from_fasta(use_gpu=True, remove_duplicates=True, max_distance=255) + " \
           "fasta_reference_distances; n=20000 (30% duplicates), L=29903, uint8"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class quiet_stdout:
    """Silences file descriptor 1 (the library's progress lines) so that the
    JSON result is the only line on stdout."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *exc):
        sys.stdout.flush()
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_elapsed(elapsed, ws, device):
    """Replicas: every rank timed its own steps; the job's time is the max
    over ranks (all_reduce MAX on `device`: cuda under NCCL, cpu under gloo),
    followed by a barrier."""
    if ws <= 1:
        return elapsed
    import torch

    t = torch.tensor([elapsed], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def replica_value(units_per_rank, ws, elapsed):
    """Whole-job throughput: every rank processed the same units (weak
    scaling), in the max time over ranks."""
    return ws * units_per_rank / elapsed


class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.lines = device, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first_sample(self, timeout=10.0):
        t = time.perf_counter() + timeout
        while self.proc and not self.lines and time.perf_counter() < t:
            time.sleep(0.01)

    def mark(self):
        """Samples from here on are the timed region's."""
        self.first = len(self.lines)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the timed region's samples (every 50 ms), and the last one before it
        for ln in self.lines[max(0, getattr(self, "first", 0) - 1):]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def synth_module():
    """The seeded generator (hammingdist_gb300/synth.py, pure numpy), loaded
    from its file: the reference arm must not import the product package,
    whose __init__ loads the native library."""
    import importlib.util

    if "_hd_synth" not in sys.modules:
        spec = importlib.util.spec_from_file_location(
            "_hd_synth", os.path.join(ROOT, "hammingdist_gb300", "synth.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules["_hd_synth"] = mod
    return sys.modules["_hd_synth"]


def make_workload(tmpdir):
    synth = synth_module()
    rows, root, _ = synth.alignment(N, L, p=P_SUB, seed=SEED, dup_frac=DUP)
    fa = synth.to_fasta(rows)
    path = os.path.join(tmpdir, "bench.fasta")
    with open(path, "wb") as f:
        f.write(fa)
        # written back now: a writeback of the 598 MB starting during the
        # timed file-to-host steps would compete with their reads
        f.flush()
        os.fsync(f.fileno())
    return fa, root.tobytes(), path, rows


def measured_peaks():
    """The measured HBM copy and bf16 GEMM peaks of this GPU kind
    (MEASURED_PEAKS.json at the repository root), if present."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(p))
    except (OSError, ValueError):
        return {}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the distance kernel on this workload's 14,000 distinct rows at L=29,903,
# from one ncu capture (one launch, one pass):
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none
#       -k regex:k_pairwise_mma -s 1 -c 1
#       python bench.py --kernel-only --n 14000 --steps 1 --warmup 1
# bench.py cannot run ncu itself, so the figure is a constant of the kernel
# build it was measured on (KERNEL_DRAM_SOURCE).
KERNEL_DRAM_BYTES = 7_754_952_192
KERNEL_DRAM_SOURCE = ("ncu capture of k_pairwise_mma (FP4 operand, 240-column items, dash "
                      "products of marked chunks only), n=14000 L=29903, one launch: 7.658 GB "
                      "read + 0.097 GB written")


# ------------------------------------------------------------------ CPU leg
def oracle_pass(fa, root):
    """One pass of the reference's CPU algorithm over the whole workload, as
    restated by the oracle port (from_fasta(remove_duplicates=True): read +
    dedupe + pack + the dense AND-rule lower triangle on all host threads,
    include/hamming/hamming_impl.hh:161-175; then fasta_reference_distances,
    src/hamming.cc:104-141, single-threaded as in the reference). Returns
    (lt, sequence indices, reference distances, seconds)."""
    from oracle import hd_oracle as o

    t = time.perf_counter()
    lt, idx = o.from_fasta_dense(fa, remove_duplicates=True)
    rd = o.reference_distances(root, fa)
    return lt, idx, rd, time.perf_counter() - t


def run_reference(args):
    """The reference arm: the reference's CPU algorithm (the oracle port: the
    GPU machine has no reference sources to compile) on the host cores, on the
    same workload as the GPU arm: all 20,000 records (14,000 unique rows) of
    the n=20,000 file plus the reference distances, every step. The product
    package is not imported: the workload comes from the generator's file."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import hd_oracle as o

    with tempfile.TemporaryDirectory() as d:
        fa, root, path, rows = make_workload(d)
        n_u = len(dict.fromkeys(r.tobytes() for r in rows))
        del rows
        times = []
        for k in range(args.warmup + args.steps):
            _, _, _, dt = oracle_pass(fa, root)
            if k >= args.warmup:
                times.append(dt)
        ps = n_u * (n_u - 1) / 2 * L
        mean = sum(times) / len(times)
        value = ps / mean / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "Gpair-sites/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded generator; no public dataset)", "impl": "reference",
            "config": {"workload": WORKLOAD, "unique_rows": n_u,
                       "pairs": n_u * (n_u - 1) // 2, "same_config": True,
                       "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "Gpair-sites/s", "cores": o.num_threads(),
                             "kind": "port",
                             "sample": f"the whole workload every step: {N} records, {n_u} unique "
                                       f"rows, dense AND-rule lower triangle (OpenMP) + reference "
                                       f"distances (one thread)"},
            "e2e": {"value": value, "unit": "Gpair-sites/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def value_phases(ctx, d_fa, nbytes, root, d_lt):
    """One untimed traced step through the C ABI: the stream time of each
    phase (CUDA events on the library's stream)."""
    ctx.trace(True)
    a = ctx.alignment_from_fasta(d_fa.data_ptr(), nbytes, on_device=True, remove_duplicates=True)
    t1 = ctx.trace_last()
    ctx.pairwise_lt(a, dtype=np.uint8, max_distance=255, out=d_lt.data_ptr(), out_on_device=True)
    t2 = ctx.trace_last()
    ctx.alignment_reference_distances(a, root)
    a.free()
    ctx.trace(False)
    phases = {}
    for text in (t1, t2):
        body = text.split(":", 1)[1] if ":" in text else ""
        for part in body.split(","):
            part = part.strip()
            if part.endswith(" ms") and not part.startswith("stream time"):
                name, ms = part[:-3].rsplit(" ", 1)
                phases[name] = round(float(ms), 3)
    return phases


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    os.environ["HAMMINGDIST_DEVICE"] = str(local)
    import hammingdist_gb300 as hd
    from hammingdist_gb300 import abi

    dev = f"cuda:{local}"
    with tempfile.TemporaryDirectory() as d:
        fa, root, path, rows = make_workload(d)
        nbytes = len(fa)
        uniq_rows = len(dict.fromkeys(r.tobytes() for r in rows))
        del rows
        d_fa = torch.frombuffer(bytearray(fa), dtype=torch.uint8).to(dev)
        n_u = uniq_rows
        pairs = n_u * (n_u - 1) // 2
        d_lt = torch.empty(pairs, dtype=torch.uint8, device=dev)
        refq = root.decode()

        # one step = one call of the module: parse + dedupe + pack + distances
        # + reference distances on the device, results in HBM (distances) and
        # on the host (indices, reference distances)
        def step():
            return hd.from_fasta_device(d_fa.data_ptr(), nbytes, d_lt.data_ptr(), pairs,
                                        remove_duplicates=True, max_distance=255,
                                        reference_sequence=refq)

        # the clock sampler starts before the warm-up and has answered once
        # before the timed steps: nvidia-smi's start-up (NVML initialisation)
        # can hold the NVIDIA driver for tens of ms, which must not fall into them
        clocks = Clocks(local)
        clocks.start()
        clocks.wait_first_sample()
        for _ in range(args.warmup):
            r = step()
        assert r["nsamples"] == n_u, (r["nsamples"], n_u)
        stream = torch.cuda.ExternalStream(hd._stream(), device=dev)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        clocks.mark()
        launches0 = hd._kernel_launches()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        pair_ms = []
        for _ in range(args.steps):
            r = step()
            pair_ms.append(r["kernel_ms"])
        ev1.record(stream)
        torch.cuda.synchronize()
        # nvidia-smi stops here, before the e2e steps: their host-clock time
        # would include any wait behind its queries to the NVIDIA driver
        clk = clocks.stop()
        launches = hd._kernel_launches() - launches0
        elapsed = replica_elapsed(ev0.elapsed_time(ev1) / 1e3, ws, dev)
        ms_step = elapsed / args.steps * 1e3
        value = replica_value(pairs * L * args.steps, ws, elapsed) / 1e9
        lt_dev = d_lt.cpu().numpy()
        idx_dev, rd_dev = r["sequence_indices"], r["reference_distances"]

        # per-phase stream times of one more (untimed, traced) step
        ctx = abi.Context(local)
        phases = value_phases(ctx, d_fa, nbytes, root, d_lt)

        # e2e: the public API with host buffers (file -> device -> host).
        # Python's cyclic garbage collector is off while these steps run, as
        # timeit does: a collection pass over the harness's own objects would
        # otherwise land in whichever step crosses its allocation threshold
        e2e_times = []
        h2d = d2h = 0
        gc.collect()
        gc.disable()
        for k in range(args.warmup + args.steps):
            # a new modification time: from_fasta reads and uploads the file
            # again every step; fasta_reference_distances then finds the same
            # unchanged file already on the device
            stamp = time.time_ns()
            os.utime(path, ns=(stamp, stamp))
            torch.cuda.synchronize()
            with quiet_stdout():
                t = time.perf_counter()
                ds = hd.from_fasta(path, use_gpu=True, remove_duplicates=True)
                lt_arr = ds.lt_array
                rd2 = hd.fasta_reference_distances(refq, path)
                torch.cuda.synchronize()
                dt = time.perf_counter() - t
            if k >= args.warmup:
                e2e_times.append(dt)
            h2d = nbytes  # the FASTA goes up once per step
            d2h = lt_arr.nbytes + 8 * N + rd2.nbytes
        gc.enable()
        e2e_mean = sum(e2e_times) / len(e2e_times)
        e2e_value = ws * pairs * L / e2e_mean / 1e9

        # parity at full size: the oracle port computes the whole workload
        # (every one of the 97,993,000 distances, the 20,000 sequence indices
        # and reference distances) and both GPU paths must equal it byte for
        # byte; the same pass is the timed CPU baseline
        lt_o, idx_o, rd_o, cpu_s = oracle_pass(fa, root)
        checks = {
            "lt_resident": bool(np.array_equal(lt_dev, lt_o)),
            "lt_e2e": bool(np.array_equal(np.asarray(lt_arr), lt_o)),
            "sequence_indices": bool(np.array_equal(np.asarray(idx_dev), idx_o)) and
            bool(np.array_equal(np.asarray(ds_indices(ds, d)), idx_o)),
            "reference_distances": bool(np.array_equal(rd_dev, rd_o)) and
            bool(np.array_equal(rd2, rd_o)),
        }
        exact = all(checks.values())
        entries_equal = int(np.count_nonzero(lt_dev == lt_o)) if lt_dev.size == lt_o.size else 0

        # roofline of the dominant kernel, the tensor-core engine: per pair,
        # matches = <planes, planes'> - 3 <dash, dash'>, 4 multiply-adds per
        # site for the planes and 1 more per site of the 256-site chunks that
        # hold a '-' (the library reports the launch's multiply-adds), in
        # E2M1 (FP4) operands against the device's measured FP4 MMA rate
        peaks = ctx.measure_int_peaks()
        fp4_peak = ctx.measure_mma_peak()
        ctx.close()
        kern_s = statistics.mean(pair_ms) / 1e3
        flop_per_launch = 2.0 * r["mma_macs"]
        achieved = flop_per_launch / kern_s / 1e12
        peak = fp4_peak / 1e12
        bf16 = measured_peaks().get("bf16_tflops")
        busy = sum(phases.values())

        if rank == 0:
            line = {
                "metric": METRIC, "value": value, "unit": "Gpair-sites/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                "data": "synthetic (seeded generator; no public dataset)",
                "config": {"workload": WORKLOAD, "unique_rows": n_u, "pairs": pairs,
                           "nominal_value": ws * (N * (N - 1) // 2) * L * args.steps / elapsed / 1e9,
                           "l2": "inputs larger than L2 (598 MB FASTA, 209 MB packed rows); no flush",
                           "parallelism": "replicas" if ws > 1 else "single GPU",
                           "step_phases_ms": phases,
                           "step_host_gap_ms": ms_step - busy},
                "parity": ("bit-exact: %d/%d distances, %d sequence indices and %d reference "
                           "distances equal the oracle (resident and e2e results)"
                           % (entries_equal, lt_o.size, len(idx_o), len(rd_o)))
                if exact else "MISMATCH " + json.dumps(checks),
                "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                             "unit": "TFLOP/s", "frac": achieved / peak,
                             "traffic": KERNEL_DRAM_BYTES, "traffic_source": KERNEL_DRAM_SOURCE,
                             "kernel_ms": kern_s * 1e3,
                             "peak_source": "in-run FP4 (E2M1, kind::mxf4) tcgen05 MMA "
                                            "microbenchmark, M=128 N=256 K=64 "
                                            "(hd_measure_mma_peak); MEASURED_PEAKS.json has "
                                            "bf16 only",
                             "bf16_measured_TF": bf16,
                             "flop_per_pair_site": flop_per_launch / (pairs * L),
                             "kernel_pair_sites_T": pairs * L / kern_s / 1e12,
                             "hbm_write_GBs": pairs / kern_s / 1e9,
                             "lop3_engine_bound_T": min(8 * peaks["lop3_per_s"],
                                                        32 * peaks["popc_per_s"]) / 1e12,
                             "lop3_mix_ceiling_T": peaks["mix_pair_sites_per_s"] / 1e12},
                "e2e": {"value": e2e_value, "unit": "Gpair-sites/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": e2e_mean * 1e3,
                        # each timed step (host clock): the host is shared, and
                        # a step it delays shows here rather than only in the mean
                        "steps_ms": [round(t * 1e3, 3) for t in e2e_times],
                        "median_ms": statistics.median(e2e_times) * 1e3},
                "gpu_launches": launches,
                "clocks": clk,
            }
            if not args.no_cpu:
                from oracle import hd_oracle as o

                line["cpu_baseline"] = {
                    "value": pairs * L / cpu_s / 1e9, "unit": "Gpair-sites/s",
                    "cores": o.num_threads(), "kind": "port",
                    "sample": f"the whole workload once: {N} records, {n_u} unique rows, dense "
                              f"AND-rule lower triangle (OpenMP) + reference distances, "
                              f"{cpu_s:.1f} s"}
            del d_fa, d_lt
            torch.cuda.empty_cache()
            if not args.headline_only and ws == 1:
                line.update(extra_legs(args))
            print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def ds_indices(ds, tmpdir):
    """The DataSet's sequence indices through its own writer."""
    p = os.path.join(tmpdir, "idx.txt")
    ds.dump_sequence_indices(p)
    return np.loadtxt(p, dtype=np.uint64, ndmin=1)


def extra_legs(args):
    """The rest of the reference's workload list, each bounded in time and
    reported under its own key of the headline line: config 1 (n=1,000 from
    file, against the CPU port), config 4 (64 uneven alignments batched
    against a loop of plain calls) and config 5 (serving, a shorter Poisson
    stream than the --serve run's 60 s)."""
    out = {}
    legs = (("config1_small", lambda: small_leg(steps=10, warmup=3)),
            ("config4_batched", lambda: batched_leg(args, steps=5, warmup=2)),
            ("config5_serve", lambda: serve_leg(args, seconds=args.extra_serve_seconds)))
    for key, fn in legs:
        t = time.perf_counter()
        try:
            out[key] = fn()
        except Exception as e:  # reported in the line, not hidden
            out[key] = {"error": f"{type(e).__name__}: {e}"}
        out[key]["leg_seconds"] = round(time.perf_counter() - t, 1)
    return out


def run_kernel_only(args):
    """The pairwise kernel alone on n distinct rows (profiling harness):
    one alignment resident in HBM, warmup + steps launches of hd_pairwise_lt
    into a device buffer, CUDA-event time per launch."""
    import torch

    from hammingdist_gb300 import abi

    synth = synth_module()
    ctx = abi.Context(0)
    rows, _, _ = synth.alignment(args.n, args.L, p=P_SUB, seed=SEED)
    seqs = [r.tobytes() for r in rows]
    aln = ctx.alignment_from_sequences(seqs)
    n = aln.n_rows
    pairs = n * (n - 1) // 2
    dt = np.uint16 if args.dtype == "u16" else np.uint8
    out = torch.empty(pairs * np.dtype(dt).itemsize, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    ms = []
    for k in range(args.warmup + args.steps):
        ctx.pairwise_lt(aln, dtype=dt, max_distance=255, out=out.data_ptr(), out_on_device=True)
        if k >= args.warmup:
            ms.append(ctx.last_pairwise_timing()[0])
    mean = sum(ms) / len(ms)
    print(json.dumps({"mode": "kernel-only", "n": n, "L": args.L, "dtype": args.dtype,
                      "kernel_ms": mean, "pair_sites_T": pairs * args.L / (mean / 1e3) / 1e12,
                      "launches": ctx.kernel_launches}), flush=True)
    ctx.close()


def run_ingest_only(args):
    """Ingest alone (profiling harness): the workload's generator with --n
    records (30% duplicates) of L sites, the FASTA resident in HBM; warmup +
    steps of alignment_from_fasta (newline index, records, dedupe, pack) and
    the reference distances of the root against the resident rows, each
    step's phases traced (CUDA events on the library's stream)."""
    import torch

    from hammingdist_gb300 import abi

    synth = synth_module()
    rows, root, _ = synth.alignment(args.n, args.L, p=P_SUB, seed=SEED, dup_frac=DUP)
    fa = synth.to_fasta(rows)
    del rows
    ctx = abi.Context(0)
    d_fa = torch.frombuffer(bytearray(fa), dtype=torch.uint8).to("cuda:0")
    torch.cuda.synchronize()
    ctx.trace(True)
    traces = []
    for k in range(args.warmup + args.steps):
        a = ctx.alignment_from_fasta(d_fa.data_ptr(), len(fa), on_device=True,
                                     remove_duplicates=True)
        t = ctx.trace_last()
        ctx.alignment_reference_distances(a, root.tobytes())
        a.free()
        if k >= args.warmup:
            traces.append(t)
    print(json.dumps({"mode": "ingest-only", "records": args.n, "L": args.L,
                      "fasta_bytes": len(fa), "trace": traces[-1]}), flush=True)
    ctx.close()


def run_batched(args):
    print(json.dumps(batched_leg(args, args.steps, args.warmup)), flush=True)


def batched_leg(args, steps, warmup):
    """Batched alignments: 64 independent alignments, n log-uniform in
    [50, 5000], L from {1000, 5000, 10000, 29903}, substitution p uniform in
    [1e-4, 1e-2], each from its own seeded root, mixed uint8/uint16 outputs.
    Metric: matrices/s of from_fasta_batch (concurrent ingest + one
    persistent launch per kernel configuration, replayed from a CUDA graph)
    against a loop of plain from_fasta / from_fasta_large calls over the same
    files; every matrix compared."""
    import torch

    import hammingdist_gb300 as hd

    synth = synth_module()
    rng = np.random.default_rng(4242)
    k = args.batch_size
    with tempfile.TemporaryDirectory() as d:
        files, large, work = [], [], 0
        for i in range(k):
            n = int(round(np.exp(rng.uniform(np.log(50), np.log(5000)))))
            Li = int(rng.choice([1000, 5000, 10000, 29903]))
            p = float(rng.uniform(1e-4, 1e-2))
            rows, _, _ = synth.alignment(n, Li, p=p, seed=10_000 + i)
            path = os.path.join(d, f"a{i}.fasta")
            with open(path, "wb") as f:
                f.write(synth.to_fasta(rows))
            files.append(path)
            large.append(bool(rng.integers(0, 2)))
            work += n * (n - 1) // 2 * Li
        if args.tuning:
            hd.load_tuning(args.tuning)

        def plain():
            return [(hd.from_fasta_large if big else hd.from_fasta)(f, use_gpu=True)
                    for f, big in zip(files, large)]

        def batched():
            return hd.from_fasta_batch(files, use_gpu=True, large=large)

        res = {}
        for name, fn in (("plain", plain), ("batched", batched)):
            times = []
            for it in range(warmup + steps):
                with quiet_stdout():
                    torch.cuda.synchronize()
                    t = time.perf_counter()
                    out = fn()
                    torch.cuda.synchronize()
                    dt = time.perf_counter() - t
                if it >= warmup:
                    times.append(dt)
            res[name] = (out, statistics.median(times))
        same = all(np.array_equal(np.asarray(a.lt_array), np.asarray(b.lt_array))
                   for a, b in zip(res["plain"][0], res["batched"][0]))
        tp, tb = res["plain"][1], res["batched"][1]

        # the same matrices from alignments already resident in HBM: a loop of
        # hd_pairwise_lt calls against one replayed batch graph (host outputs)
        from hammingdist_gb300 import abi

        ctx = abi.Context(0)
        if args.tuning:
            ctx.tune_load(args.tuning)
        alns = [ctx.alignment_from_fasta(open(f, "rb").read()) for f in files]
        dts = [np.uint16 if big else np.uint8 for big in large]
        mds = [65535 if big else 255 for big in large]
        batch = ctx.batch()
        for a, dt, md in zip(alns, dts, mds):
            batch.add(a, dtype=dt, max_distance=md)
        r_plain, r_batch = [], []
        for it in range(warmup + steps):
            t = time.perf_counter()
            outs_p = [ctx.pairwise_lt(a, dtype=dt, max_distance=md) for a, dt, md in zip(alns, dts, mds)]
            t1 = time.perf_counter()
            outs_b = batch.run()
            t2 = time.perf_counter()
            if it >= warmup:
                r_plain.append(t1 - t)
                r_batch.append(t2 - t1)
        same_r = all(np.array_equal(x, y) for x, y in zip(outs_p, outs_b))
        rp, rb = statistics.median(r_plain), statistics.median(r_batch)
        graph_ms, n_launch, n_tiles = batch.timing()
        batch.free()
        ctx.close()
        return {
            "mode": "batched", "metric": "matrices/s (64 uneven alignments)",
            "batched_matrices_per_s": k / tb, "plain_loop_matrices_per_s": k / tp,
            "speedup": tp / tb, "batched_ms": tb * 1e3, "plain_ms": tp * 1e3,
            "pair_sites": work, "batched_Gpair_sites_per_s": work / tb / 1e9,
            "bit_exact_vs_plain": same and same_r, "steps": steps, "warmup": warmup,
            "resident": {"plain_loop_ms": rp * 1e3, "batched_ms": rb * 1e3, "speedup": rp / rb,
                         "batch_graph_ms": graph_ms, "persistent_launches": n_launch,
                         "tiles": n_tiles, "Gpair_sites_per_s": work / rb / 1e9},
            "tuning": args.tuning or "built-in"}


def _device_fasta_file(ctx, path, n, L_, p, seed):
    """Seeded synthetic FASTA generated on the device, written to `path`."""
    import torch

    nb = ctx.synthetic_fasta(n, L_, p=p, seed=seed)
    buf = torch.empty(nb, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    ctx.synthetic_fasta(n, L_, p=p, seed=seed, out=buf.data_ptr())
    host = buf.cpu().numpy()
    del buf
    with open(path, "wb") as f:
        f.write(memoryview(host))
    return nb


def run_streaming(args):
    """Wide distances and streamed outputs at full size (L=29,903):
    from_fasta_large on n=50,000 (p=2e-2, uint16, max_distance=65535);
    from_fasta_to_lower_triangular on n=100,000 (p=5e-5, max_distance=2, the
    text streamed to disk while later rows compute); dump_sparse(threshold=3)
    of the n=100,000 set built with max_distance=255. Checks: output sizes,
    the first rows against the oracle, every sparse line recomputed by the
    oracle."""
    import hammingdist_gb300 as hd
    from hammingdist_gb300 import abi
    from oracle import hd_oracle as o

    ctx = abi.Context(0)
    L_ = 29903
    res = {"mode": "streaming", "L": L_}
    with tempfile.TemporaryDirectory(dir=args.tmpdir or None) as d:
        f50 = os.path.join(d, "n50k.fasta")
        f100 = os.path.join(d, "n100k.fasta")
        _device_fasta_file(ctx, f50, args.n_wide, L_, 2e-2, 501)
        _device_fasta_file(ctx, f100, args.n_stream, L_, 5e-5, 502)
        head50 = open(f50, "rb").read(200 * (L_ + 13))
        head100 = open(f100, "rb").read(200 * (L_ + 13))
        # wide distances
        with quiet_stdout():
            t = time.perf_counter()
            ds = hd.from_fasta_large(f50, use_gpu=True)
            lt = np.asarray(ds.lt_array)
            dt = time.perf_counter() - t
        n = args.n_wide
        ref = o.from_fasta_dense(head50, dtype=np.uint16, max_distance=65535)[0]
        res["from_fasta_large"] = {
            "n": n, "seconds": dt, "Gpair_sites_per_s": n * (n - 1) / 2 * L_ / dt / 1e9,
            "max_distance_seen": int(lt.max()), "above_255": int(np.count_nonzero(lt > 255)),
            "first_200_rows_bit_exact": bool(np.array_equal(lt[: ref.size], ref))}
        del ds, lt
        # streamed lower-triangular text
        out = os.path.join(d, "lt.txt")
        with quiet_stdout():
            t = time.perf_counter()
            hd.from_fasta_to_lower_triangular(f100, out, max_distance=2)
            dt = time.perf_counter() - t
        n = args.n_stream
        size = os.path.getsize(out)
        with open(out, "rb") as f:
            head_text = f.read(4 * 200 * 200)
        want = o.format_lower_triangular(o.from_fasta_dense(head100, dtype=np.uint16,
                                                            max_distance=2)[0])
        res["from_fasta_to_lower_triangular"] = {
            "n": n, "seconds": dt, "Gpair_sites_per_s": n * (n - 1) / 2 * L_ / dt / 1e9,
            "bytes_written": size, "GB_per_s_text": size / dt / 1e9,
            "size_is_2_bytes_per_entry": size == n * (n - 1),
            "first_200_rows_bit_exact": head_text[: len(want)] == want}
        os.remove(out)
        # sparse dump of the max_distance=255 set
        sp = os.path.join(d, "sparse.txt")
        with quiet_stdout():
            t = time.perf_counter()
            ds = hd.from_fasta(f100, use_gpu=True, max_distance=255)
            t1 = time.perf_counter()
            ds.dump_sparse(sp, 3)
            dt = time.perf_counter() - t
        lines = open(sp, "rb").read().splitlines()
        ok = True
        rec_bytes = L_ + 13  # the generator writes fixed-width records
        with open(f100, "rb") as fh:
            def rec(i):
                fh.seek(i * rec_bytes + 12)
                return fh.read(L_)
            for ln in lines[: args.sparse_check]:
                i, j, dd = (int(x) for x in ln.split())
                ok &= o.lt_dense([rec(i), rec(j)], max_distance=255)[0] == dd <= 3
        res["dump_sparse"] = {
            "n": n, "threshold": 3, "seconds_total": dt, "seconds_matrix": t1 - t,
            "seconds_dump": dt - (t1 - t), "lines": len(lines),
            "lines_checked_by_oracle": min(len(lines), args.sparse_check), "lines_ok": bool(ok)}
        del ds
    print(json.dumps(res), flush=True)
    ctx.close()


def run_small(args):
    print(json.dumps(small_leg(args.steps, args.warmup)), flush=True)


def small_leg(steps, warmup):
    """The reference's config 1: from_fasta(use_gpu=True) on n=1,000 rows,
    L=29,903, p=1e-3, uint8, through the public API from the file, every step
    reading the file again (new mtime). Beside it the oracle port computes the
    same matrix from the same file on all host threads. Both must agree bit
    for bit."""
    import hammingdist_gb300 as hd
    from oracle import hd_oracle as o

    synth = synth_module()
    n, L_ = 1000, 29903
    rows, root, _ = synth.alignment(n, L_, p=1e-3, seed=11, dup_frac=0.0)
    fa = synth.to_fasta(rows)
    pairs = n * (n - 1) // 2
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "config1.fasta")
        with open(path, "wb") as f:
            f.write(fa)
        times = []
        for k in range(warmup + steps):
            st = time.time_ns()
            os.utime(path, ns=(st, st))
            with quiet_stdout():
                t = time.perf_counter()
                lt = hd.from_fasta(path, use_gpu=True).lt_array
                dt = time.perf_counter() - t
            if k >= warmup:
                times.append(dt)
        gpu_s = statistics.median(times)
        cpu_times = []
        for _ in range(3):
            t = time.perf_counter()
            want = o.from_fasta_dense(open(path, "rb").read())[0]
            cpu_times.append(time.perf_counter() - t)
        cpu_s = statistics.median(cpu_times)
    return {
        "mode": "config1", "workload": "from_fasta(use_gpu=True) n=1000 L=29903 p=1e-3 uint8, file to lt_array",
        "pairs": pairs, "gpu_e2e_ms": gpu_s * 1e3, "gpu_Gpair_sites_per_s": pairs * L_ / gpu_s / 1e9,
        "cpu_port_ms": cpu_s * 1e3, "cpu_cores": o.num_threads(),
        "cpu_Gpair_sites_per_s": pairs * L_ / cpu_s / 1e9, "speedup": cpu_s / gpu_s,
        "bit_exact": bool(np.array_equal(np.asarray(lt), want))}


def run_formats(args):
    """Result files of the headline matrix (14,000 unique rows of the n=20,000,
    L=29,903 workload, uint8): DataSet.dump (full matrix text),
    from_lower_triangular (the dump_lower_triangular text) and from_csv (the
    dump text), on the device through the public API. The CPU leg is the C
    restatement of the reference's single-threaded host code on the first
    --formats-cpu-rows rows (a prefix of the triangle is the matrix of those
    rows). Checks: the sample's dump text is byte-identical between device and
    CPU, and both readers give the matrix back at full size."""
    import hammingdist_gb300 as hd
    from oracle import hd_oracle as o

    def rate(entries, s):
        return entries / s / 1e6

    with tempfile.TemporaryDirectory(dir=args.tmpdir or None) as d:
        fa, root, path, rows = make_workload(d)
        with quiet_stdout():
            ds = hd.from_fasta(path, use_gpu=True, remove_duplicates=True)
        lt = np.asarray(ds.lt_array)
        n = int(round((1 + (1 + 8 * lt.size) ** 0.5) / 2))
        full_entries = n * n
        ltp, dmp = os.path.join(d, "lt.txt"), os.path.join(d, "dump.txt")
        ds.dump_lower_triangular(ltp)
        times = {}
        t = time.perf_counter()
        ds.dump(dmp)
        times["dump"] = time.perf_counter() - t
        for name, fn, arg in (("from_lower_triangular", hd.from_lower_triangular, ltp),
                              ("from_csv", hd.from_csv, dmp)):
            best = 1e30
            for _ in range(3):
                # a new mtime: the file is read and uploaded again every time
                stamp = time.time_ns()
                os.utime(arg, ns=(stamp, stamp))
                t = time.perf_counter()
                back = fn(arg)
                best = min(best, time.perf_counter() - t)
            times[name] = best
            got = np.asarray(back.lt_array)[: lt.size]
            assert np.array_equal(got, lt), name
        sizes = {"dump": os.path.getsize(dmp), "lt_text": os.path.getsize(ltp)}
        # CPU leg on a prefix sample
        m = args.formats_cpu_rows
        sub = np.ascontiguousarray(lt[: m * (m - 1) // 2])
        s_lt, s_dmp, c_dmp = (os.path.join(d, x) for x in ("s_lt.txt", "s_dump.txt", "c_dump.txt"))
        with open(s_lt, "wb") as fh:
            fh.write(o.format_lower_triangular(sub))
        cpu = {}
        t = time.perf_counter()
        o.dump_full(sub, m, c_dmp)
        cpu["dump"] = time.perf_counter() - t
        t = time.perf_counter()
        c_lt, _ = o.read_lower_triangular(s_lt)
        cpu["from_lower_triangular"] = time.perf_counter() - t
        t = time.perf_counter()
        c_csv, _ = o.read_csv(c_dmp)
        cpu["from_csv"] = time.perf_counter() - t
        sample_ds = hd.from_lower_triangular(s_lt)
        sample_ds.dump(s_dmp)
        parity = (open(s_dmp, "rb").read() == open(c_dmp, "rb").read()
                  and np.array_equal(c_lt, sub) and np.array_equal(c_csv[: sub.size], sub))
    entries = {"dump": full_entries, "from_lower_triangular": lt.size, "from_csv": lt.size}
    s_entries = {"dump": m * m, "from_lower_triangular": sub.size, "from_csv": sub.size}
    out = {"mode": "formats", "n": n, "dtype": "u8", "text_bytes": sizes,
           "parity": "bit-exact" if parity else "MISMATCH", "cpu_sample_rows": m, "cpu_threads": 1}
    for k in times:
        g, c = rate(entries[k], times[k]), rate(s_entries[k], cpu[k])
        out[k] = {"gpu_s": times[k], "gpu_Mentries_per_s": g, "cpu_Mentries_per_s": c,
                  "speedup": g / c}
    print(json.dumps(out), flush=True)


def run_serve(args):
    print(json.dumps(serve_leg(args, args.serve_seconds)), flush=True)


def serve_leg(args, seconds):
    """Serving: 8 alignments resident in HBM (n = 200k, 100k, 50k, 50k, 20k,
    20k, 10k, 10k at --serve-scale 1; L=29,903; generated on the device), a
    Poisson request stream (--serve-rate per s for --serve-seconds): 60%
    reference-distance queries (a new seeded query against a resident set),
    30% pairwise matrices of a window of n rows (n log-uniform 100-10,000,
    uint8/uint16), 10% sparse dumps of such a window (threshold 1-5).
    Reports p50/p99 latency at that load, the throughput of the same requests
    submitted at once (server saturated) and of serial plain calls."""
    import threading as th

    import torch

    from hammingdist_gb300 import abi

    synth = synth_module()
    ctx = abi.Context(0)
    L_ = 29903
    sizes = [int(x * args.serve_scale) for x in (200000, 100000, 50000, 50000, 20000, 20000,
                                                  10000, 10000)]
    alns, t0 = [], time.perf_counter()
    for k, n in enumerate(sizes):
        nb = ctx.synthetic_fasta(n, L_, p=1e-3, seed=900 + k)
        buf = torch.empty(nb, dtype=torch.uint8, device="cuda:0")
        torch.cuda.synchronize()
        ctx.synthetic_fasta(n, L_, p=1e-3, seed=900 + k, out=buf.data_ptr())
        alns.append(ctx.alignment_from_fasta(buf.data_ptr(), nb, on_device=True))
        del buf
    torch.cuda.empty_cache()
    load_s = time.perf_counter() - t0
    roots = [synth.device_root(900 + k, L_) for k in range(len(sizes))]

    rng = np.random.default_rng(31337)
    n_req = int(args.serve_rate * seconds)
    gaps = rng.exponential(1.0 / args.serve_rate, n_req)
    arrivals = np.cumsum(gaps)
    reqs = []
    for _ in range(n_req):
        u = rng.random()
        a = int(rng.integers(0, len(sizes)))
        if u < 0.6:
            q = roots[a].copy()
            m = rng.random(L_) < 1e-3
            q[m] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(m.sum()))]
            reqs.append(("ref", a, q.tobytes()))
        else:
            n = int(round(np.exp(rng.uniform(np.log(100), np.log(10000)))))
            cand = [i for i, s_ in enumerate(sizes) if s_ >= n]
            a = int(rng.choice(cand))
            r0 = int(rng.integers(0, sizes[a] - n + 1))
            if u < 0.9:
                reqs.append(("pair", a, r0, n, np.uint16 if rng.random() < 0.5 else np.uint8))
            else:
                reqs.append(("sparse", a, r0, n, int(rng.integers(1, 6))))

    def submit(srv, ids, r):
        if r[0] == "ref":
            return srv.reference(ids[r[1]], r[2])
        if r[0] == "pair":
            return srv.pairwise(ids[r[1]], r[2], r[3], dtype=r[4], max_distance=65535)
        return srv.sparse(ids[r[1]], r[2], r[3], r[4])

    def run_stream(paced):
        srv = ctx.server(output_budget_bytes=args.serve_budget_gb << 30, max_waves=3)
        ids = [srv.add(a) for a in alns]
        tickets = [None] * len(reqs)
        start = time.perf_counter()

        def producer():
            for i, r in enumerate(reqs):
                if paced:
                    delay = start + arrivals[i] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                tickets[i] = submit(srv, ids, r)

        thr = th.Thread(target=producer)
        thr.start()
        lat, queue, kinds = [], [], []
        for i in range(len(reqs)):
            while tickets[i] is None:
                time.sleep(0.0005)
            srv.wait(tickets[i], 600)
            _, _, l, q = srv.result(tickets[i])
            lat.append(l)
            queue.append(q)
            kinds.append(reqs[i][0])
        thr.join()
        wall = time.perf_counter() - start
        stats = srv.stats()
        srv.free()
        lat = np.array(lat)
        per_kind = {k: {"p50_ms": float(np.percentile(lat[np.array(kinds) == k], 50)),
                        "p99_ms": float(np.percentile(lat[np.array(kinds) == k], 99)),
                        "count": int(np.sum(np.array(kinds) == k))}
                    for k in ("ref", "pair", "sparse") if np.any(np.array(kinds) == k)}
        return {"req_per_s": len(reqs) / wall, "wall_s": wall,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "queue_p99_ms": float(np.percentile(queue, 99)),
                "per_kind": per_kind, "waves": stats["waves"],
                "max_waves_in_flight": stats["max_inflight"]}

    paced = run_stream(True)
    saturated = run_stream(False)
    # serial plain calls over the same requests (a bounded sample, timed)
    n_serial = min(len(reqs), args.serve_serial)
    t = time.perf_counter()
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "sparse.txt")
        for r in reqs[:n_serial]:
            a = alns[r[1]]
            if r[0] == "ref":
                ctx.alignment_reference_distances(a, r[2])
            else:
                v = a.view(r[2], r[3])
                if r[0] == "pair":
                    ctx.pairwise_lt(v, dtype=r[4], max_distance=65535)
                else:
                    lt = ctx.pairwise_lt(v, dtype=np.uint8, max_distance=255)
                    ctx.write_sparse(lt, r[3], r[4], sp)
                v.free()
    serial = n_serial / (time.perf_counter() - t)
    for a in alns:
        a.free()
    ctx.close()
    return {
        "mode": "serve", "metric": "p50/p99 ms and req/s (8 resident alignments)",
        "resident_rows": sizes, "L": L_, "requests": len(reqs), "rate_per_s": args.serve_rate,
        "seconds": seconds, "load_s": load_s, "paced": paced,
        "saturated": saturated, "serial_plain_req_per_s": serial,
        "saturated_vs_serial": saturated["req_per_s"] / serial,
        "all_results_checked": "alone == in the mix: tests/test_gpu_serve.py",
        "budget_gb": args.serve_budget_gb}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true",
                    help="leave out cpu_baseline (the full-size oracle parity pass still runs)")
    ap.add_argument("--headline-only", action="store_true",
                    help="leave out the config 1 / 4 / 5 legs of the default line")
    ap.add_argument("--extra-serve-seconds", type=float, default=15.0,
                    help="length of the paced serving stream in the default line")
    ap.add_argument("--ingest-only", action="store_true",
                    help="profiling harness: device ingest of --n records and reference distances")
    ap.add_argument("--kernel-only", action="store_true",
                    help="profiling harness: the pairwise kernel alone on --n distinct rows")
    ap.add_argument("--n", type=int, default=12000)
    ap.add_argument("--L", type=int, default=L)
    ap.add_argument("--dtype", default="u8", choices=["u8", "u16"])
    ap.add_argument("--batched", action="store_true",
                    help="batched workload: matrices/s of from_fasta_batch vs a plain loop")
    ap.add_argument("--batch-size", type=int, default=64)
    ap.add_argument("--tuning", default="", help="autotuner table (JSON) to load first")
    ap.add_argument("--streaming", action="store_true",
                    help="wide-distance and streamed-output workloads at full size")
    ap.add_argument("--n-wide", type=int, default=50000)
    ap.add_argument("--n-stream", type=int, default=100000)
    ap.add_argument("--sparse-check", type=int, default=2000)
    ap.add_argument("--tmpdir", default="")
    ap.add_argument("--formats", action="store_true",
                    help="result files (dump, from_lower_triangular, from_csv) vs the CPU port")
    ap.add_argument("--formats-cpu-rows", type=int, default=3500)
    ap.add_argument("--small", action="store_true",
                    help="n=1,000 from_fasta through the public API vs the CPU port")
    ap.add_argument("--serve", action="store_true", help="serving workload (Poisson stream)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-scale", type=float, default=1.0)
    ap.add_argument("--serve-budget-gb", type=int, default=8)
    ap.add_argument("--serve-serial", type=int, default=600)
    args = ap.parse_args()
    if args.formats:
        run_formats(args)
    elif args.small:
        run_small(args)
    elif args.streaming:
        run_streaming(args)
    elif args.serve:
        run_serve(args)
    elif args.batched:
        run_batched(args)
    elif args.kernel_only:
        run_kernel_only(args)
    elif args.ingest_only:
        run_ingest_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
