"""Benchmark of the GB300 CSR SpGEMM library (one JSON line on stdout, rank 0).

Default workload: C = A*A in FP64 on the 1,000,000-row synthetic web-like power-law graph
(the configuration the headline throughput is quoted on).  One step = one complete
SpGEMM (row classification, symbolic phase, row_ptr scan, C allocation from the
handle's pool, numeric phase) through the C ABI call ops_spgemm, inputs resident in HBM.
`value` = 2 * intermediate products / mean device time per step (GFLOPS).
`e2e`   = the same metric through the same call with host buffers: every step copies A
          (and B) from pinned host memory, multiplies, and copies all of C back; steps run
          pipelined two deep on the full-duplex host link (step i+1's upload and step i's
          download overlap the SpGEMMs).  The one-step-at-a-time latency is reported too.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload web|laplacian|stencil27|stencil27_f32]

--impl reference times the CPU baseline (OpenMP row-wise hash Gustavson, the oracle's
port; OpSparse itself has no CPU SpGEMM) on the same workload and prints its line.
Under torchrun each rank runs its own replica (weak scaling) and rank 0 prints.
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import io
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SpGEMM GFLOPS & %HBM peak; batched and fwd+bwd vs plain at matched tol"
L2_FLUSH_BYTES = 256 << 20
FALLBACK_HBM_GBS = 6800.0


# ----------------------------------------------------------------------------- inputs
def make_workload(name: str):
    from opsparse_gb300 import gen

    if name == "web":
        rpt, col, val = gen.web_powerlaw()
        desc = {"workload": "web_powerlaw_1M", "rows": 1_000_000, "row_len_exponent": 2.1, "row_len_max": 4700,
                "local_window": 512, "global_zipf_s": 1.0, "values": "U(0,1)", "op": "C=A*A", "seed": gen.SEED}
        dt = "f64"
    elif name == "laplacian":
        rpt, col, val = gen.laplacian2d(128)
        desc = {"workload": "laplacian2d_128x128", "rows": 16384, "op": "C=A*A"}
        dt = "f64"
    elif name == "powerlaw_AAt":
        a = gen.powerlaw_square(200_000, 16, 2.2)
        b = gen.transpose_pattern(a[0], a[1], 200_000)
        desc = {"workload": "powerlaw_200k_AAt", "rows": 200_000, "mean_degree": 16, "exponent": 2.2,
                "values": "N(0,1)", "op": "C=A*B, B = pattern(A^T) with fresh values", "seed": gen.SEED}
        n = 200_000
        return desc, "f64", (a, b), n
    elif name in ("stencil27", "stencil27_f32"):
        rpt, col, val = gen.stencil27(80)
        desc = {"workload": "stencil27_80^3", "rows": 512000, "values": "N(0,1)", "op": "C=A*A", "seed": gen.SEED}
        dt = "f32" if name.endswith("f32") else "f64"
    else:
        raise SystemExit(f"unknown workload {name}")
    n = len(rpt) - 1
    if dt == "f32":
        val = val.astype(np.float32)
    return desc, dt, (rpt, col, val), n


def bytes_alg(M, K, nnz_a, nnz_b, nnz_c, s):
    sym = 4 * (M + 1) + 4 * nnz_a + 4 * (K + 1) + 4 * nnz_b + 4 * M
    num = 4 * (M + 1) + (4 + s) * nnz_a + 4 * (K + 1) + (4 + s) * nnz_b + 4 * (M + 1) + (4 + s) * nnz_c
    return sym + num


def measured_traffic(workload):
    """DRAM bytes per step of a workload, from the committed ncu launch-list summary."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None, None
    t = json.loads(p.read_text()).get(workload)
    return (t["dram_bytes_per_step"], t["source"]) if t else (None, None)


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        rows = [r for r in csv.reader(io.StringIO(self.out or "")) if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def f(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [f(r[1]) for r in rows if f(r[1]) is not None]
        mx = [f(r[2]) for r in rows if f(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(value: float, world: int, device) -> float:
    """The largest of every rank's `value` (the slowest rank's time); `value` itself when
    there is one rank."""
    if world <= 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- CPU side
def _pair(data):
    """Plain workloads are C = A*A (one CSR triple) or C = A*B (a pair of triples)."""
    return (data, data) if len(data) == 3 else data


def cpu_baseline(data, n, steps=3):
    """Median time of the oracle's OpenMP port on the workload, its thread count, and the
    oracle's result (the checker of the GPU result's parity: the port keeps the plain
    ascending-j fold for every entry, the oracle folds entries of more than 2,560 products
    in blocks, as the library does)."""
    import oracle

    (ar, ac, av), (br, bc, bv) = _pair(data)
    av64, bv64 = np.asarray(av, dtype=np.float64), np.asarray(bv, dtype=np.float64)
    oracle.omp_spgemm(ar, ac, av64, br, bc, bv64)  # warm-up
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        oracle.omp_spgemm(ar, ac, av64, br, bc, bv64)
        ts.append(time.perf_counter() - t0)
    ref = oracle.spgemm(ar, ac, av64, br, bc, bv64, n)
    return statistics.median(ts), oracle.num_threads(), ref


def parity_report(gpu, ref, dt, scale_fn=None):
    """Measured error of a GPU result (row_ptr, col_idx, values) against the oracle's FP64
    result on the same inputs: whether the structure is identical, the largest absolute
    error, and the largest relative error over the entries the oracle makes nonzero.

    FP64 results are also compared bit for bit, and the entries the oracle makes zero must
    be zero.  FP32 results are rounded sums of FP32 products: an entry whose terms cancel
    carries an error of the order of 2^-24 * sum_j |a_ij b_jk| however small the entry, so
    for FP32 each error is also taken relative to max(|c_ik|, 2^-24 * sum_j |a_ij b_jk|)
    (`max_rel_err_scaled`; the sums come from scale_fn(), called only when some entry
    misses the plain relative bound), and that figure decides the tolerance."""
    g_rpt, g_col, g_val = (np.asarray(x) for x in gpu)
    o_rpt, o_col, o_val = (np.asarray(x) for x in ref)
    same = (g_rpt.shape == o_rpt.shape and np.array_equal(g_rpt.astype(np.int64), o_rpt.astype(np.int64))
            and g_col.shape == o_col.shape and np.array_equal(g_col, o_col))
    tol = 1e-12 if dt == "f64" else 1e-5
    rep = {"checked_against": "oracle (FP64, every entry folded in ascending j, in 32 blocks above 2,560 products)",
           "structure_identical": bool(same),
           "tolerance_rel": tol}
    if not same:
        return rep
    gv, ov = g_val.astype(np.float64), o_val.astype(np.float64)
    diff = np.abs(gv - ov)
    nz = ov != 0
    rep["entries"] = int(ov.size)
    rep["max_abs_err"] = float(diff.max()) if diff.size else 0.0
    rep["max_rel_err"] = float((diff[nz] / np.abs(ov[nz])).max()) if nz.any() else 0.0
    rep["zeros_exact"] = bool(np.all(gv[~nz] == 0))
    if dt == "f64":
        rep["values_bit_identical"] = bool(np.array_equal(gv.view(np.uint64), ov.view(np.uint64)))
        rep["within_tolerance"] = bool(rep["max_rel_err"] <= tol and rep["zeros_exact"])
        return rep
    plain_ok = rep["max_rel_err"] <= tol and rep["zeros_exact"]
    if plain_ok or scale_fn is None:
        rep["max_rel_err_scaled"] = rep["max_rel_err"] if rep["zeros_exact"] else None
        rep["within_tolerance"] = bool(plain_ok)
        return rep
    den = np.maximum(np.abs(ov), np.asarray(scale_fn(), dtype=np.float64) * 2.0 ** -24)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(den > 0, diff / np.where(den > 0, den, 1.0), np.where(diff > 0, np.inf, 0.0))
    rep["max_rel_err_scaled"] = float(rel.max()) if rel.size else 0.0
    rep["within_tolerance"] = bool(rep["max_rel_err_scaled"] <= tol)
    return rep


def run_reference(args, desc, dt, data, n, rank, world):
    if rank != 0:
        return
    import oracle

    (ar, ac, av), (br, bc, bv) = _pair(data)
    P = int(oracle.flop(ar, ac, br)[0])
    av64, bv64 = np.asarray(av, dtype=np.float64), np.asarray(bv, dtype=np.float64)
    for _ in range(max(0, args.warmup)):
        oracle.omp_spgemm(ar, ac, av64, br, bc, bv64)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.omp_spgemm(ar, ac, av64, br, bc, bv64)
        ts.append(time.perf_counter() - t0)
    t = statistics.mean(ts)
    gf = 2.0 * P / t / 1e9
    cores = oracle.num_threads()
    line = {"metric": METRIC, "value": gf, "unit": "GFLOPS", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": desc,
            "cpu_baseline": {"value": gf, "unit": "GFLOPS", "cores": cores, "kind": "port",
                             "sample": f"full workload, {args.steps} runs, FP64, OpenMP row-wise hash Gustavson "
                                       f"(OpSparse ships no CPU SpGEMM; this is the oracle's port)"},
            "e2e": {"value": gf, "unit": "GFLOPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU side
def cusparse_gpu(A, B, n, P, nnz_c, t_ms, flush, iters=10):
    """cuSPARSE's SpGEMM on the same device-resident inputs (torch's CSR x CSR product,
    which calls cusparseSpGEMM), timed like this library's steps: L2 flushed before each
    call, CUDA events around the call, 1 warm-up then the mean of `iters` calls.  A
    side-by-side comparison only; nothing here is on the library's path."""
    import torch

    try:
        def csr(m):
            return torch.sparse_csr_tensor(m.rpt.long(), m.col.long(), m.val, size=(m.rows, m.cols))

        a, b = csr(A), csr(B)
        ts = []
        nnz_cs = -1
        for i in range(iters + 1):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            c = torch.sparse.mm(a, b)
            e1.record()
            torch.cuda.synchronize()
            if i:
                ts.append(e0.elapsed_time(e1))
            nnz_cs = int(c._nnz())
            del c
        del a, b
    except Exception as e:  # a comparison, never the product
        return {"unavailable": f"{type(e).__name__}: {e}".splitlines()[0][:200]}
    ms = float(np.mean(ts))
    return {"impl": "cuSPARSE SpGEMM through torch.sparse.mm on CSR tensors (int64 indices, as torch requires)",
            "protocol": "1 warm-up + mean of 10 calls, CUDA events, L2 flushed before each call",
            "ms_per_call": ms, "GFLOPS": 2.0 * P / (ms * 1e-3) / 1e9, "nnz_c": nnz_cs,
            "nnz_c_equal": nnz_cs == nnz_c, "speedup_of_this_library": ms / t_ms}


def reference_gpu(A, B, n, P, nnz_c, t_ms, flush, iters=10):
    """OpSparse's own kernels on this GPU (oracle/ref_gpu), timed with its own benchmark
    protocol: 1 warm-up, then the mean of 10 calls, each wall-clocked around the whole call
    (per-call workspace, streams and C allocation included, as OpSparse does).  L2 is
    flushed before each call, as for this library's timed steps."""
    import torch

    from oracle import ref_gpu

    try:
        if not ref_gpu.build() or not ref_gpu.available():
            return {"unavailable": "the reference's cubin was not built (needs the OpSparse sources)"}
        ap, bp = A.ptrs(), B.ptrs()
        runs = []
        for i in range(iters + 1):
            flush.zero_()
            torch.cuda.synchronize()
            r = ref_gpu.spgemm(n, ap[0], ap[1], ap[2], bp[0], bp[1], bp[2])
            if i:
                runs.append(r.timings)
            nnz_ref = r.nnz
            r.free()
    except Exception as e:  # the reference path is a comparison, never the product
        return {"unavailable": f"{type(e).__name__}: {e}"}
    mean = {k: float(np.mean([t[k] for t in runs])) * 1e3 for k in runs[0]}
    kernel_ms = sum(mean[k] for k in ("symbolic_binning", "symbolic", "numeric_binning", "prefix", "numeric"))
    return {"impl": "OpSparse's kernels compiled from its sources for sm_103a, its host sequence restated",
            "protocol": "1 warm-up + mean of 10 calls, wall clock around each call",
            "ms_per_call": mean["total"], "GFLOPS": 2.0 * P / (mean["total"] * 1e-3) / 1e9,
            "phases_ms": {k: round(v, 4) for k, v in mean.items()},
            "phases_without_setup_allocate_cleanup_ms": kernel_ms,
            "nnz_c_equal": nnz_ref == nnz_c,
            "speedup_of_this_library": mean["total"] / t_ms}


def measure_plain(args, desc, dt, data, n, world, local_rank, steps, warmup, side=True):
    """One plain workload through the C-ABI call ops_spgemm: K timed steps on device-resident
    inputs, then K end-to-end steps with host buffers.  Returns the bench-line fields; with
    side=True (rank 0 of a one-GPU run) also OpSparse's kernels and cuSPARSE on the same
    inputs, the CPU baseline and the measured error of the last end-to-end result."""
    import torch

    import opsparse_gb300 as ops
    from opsparse_gb300 import capi

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    tdt = torch.float64 if dt == "f64" else torch.float32
    s = 8 if dt == "f64" else 4
    (rpt, col, val), (brpt, bcol, bval) = _pair(data)
    same = len(data) == 3
    A = ops.csr_to_device(rpt, col, val, n, n, dtype=tdt, device=str(dev))
    B = A if same else ops.csr_to_device(brpt, bcol, bval, n, n, dtype=tdt, device=str(dev))
    lib = capi.load()
    h = ops.Handle()
    h.set_one_pass(1 if args.one_pass else 0)
    stream = torch.cuda.current_stream()
    st = C.c_void_p(stream.cuda_stream)
    code = capi.OPS_F64 if dt == "f64" else capi.OPS_F32
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    ap, bp = A.ptrs(), B.ptrs()

    def step():
        rp, cp, vp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnz = C.c_int64(0)
        capi.check(lib.ops_spgemm(h.h, code, n, n, n, ap[0], ap[1], ap[2], A.nnz, bp[0], bp[1], bp[2], B.nnz,
                                  C.byref(rp), C.byref(cp), C.byref(vp), C.byref(nnz), st), h.h)
        return rp, cp, vp, int(nnz.value)

    def release(ptrs):
        for p in ptrs[:3]:
            lib.ops_free(p, st)

    # untimed warm-up; also collect phase and per-class kernel times
    for _ in range(max(warmup, 3)):
        release(step())
    h.set_timing(2)
    out = step()
    nnz_c = out[3]
    phases = h.timings()
    subclass = h.subclass_rows()
    release(out)
    h.set_timing(0)
    P = int(phases["flop"])

    # timed region: K steps, L2 flushed between steps outside the events
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(local_rank) as clk:
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            out = step()
            ev[i][1].record(stream)
            launches += h.timings()["launches"]
            release(out)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = max_over_ranks(float(np.mean(step_ms)), world, dev)
    gflops = world * 2.0 * P / (t_ms * 1e-3) / 1e9

    # end to end through the same call with host buffers
    host_in = (rpt, col, val) if same else (rpt, col, val, brpt, bcol, bval)
    pin = [torch.as_tensor(x).pin_memory() for x in host_in]
    d_in = [torch.empty_like(x, device=dev) for x in pin]
    d_b = d_in[:3] if same else d_in[3:]
    h_out = [torch.empty(n + 1, dtype=torch.int32).pin_memory(), torch.empty(max(nnz_c, 1), dtype=torch.int32).pin_memory(),
             torch.empty(max(nnz_c, 1), dtype=tdt).pin_memory()]
    h2d = sum(x.numel() * x.element_size() for x in pin)
    d2h = (n + 1) * 4 + nnz_c * (4 + s)
    # host<->device copies split over several streams so that the copy engines work on
    # them together (one stream per input array; C's columns and values in halves)
    copy_streams = [torch.cuda.Stream(device=dev) for _ in range(4)]

    def fan_out(jobs):
        """Run copy jobs on the copy streams after the work queued so far on `stream`,
        and make `stream` wait for all of them."""
        start = torch.cuda.Event()
        start.record(stream)
        for k, job in enumerate(jobs):
            cs = copy_streams[k % len(copy_streams)]
            cs.wait_event(start)
            with torch.cuda.stream(cs):
                job()
        for cs in copy_streams[:len(jobs)]:
            done = torch.cuda.Event()
            done.record(cs)
            stream.wait_event(done)

    vstr = "<f8" if dt == "f64" else "<f4"
    e2e_ms = []
    for i in range(warmup + steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fan_out([lambda d=d, p=p: d.copy_(p, non_blocking=True) for d, p in zip(d_in, pin)])
        rp2, cp2, vp2 = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnz = C.c_int64(0)
        capi.check(lib.ops_spgemm(h.h, code, n, n, n, d_in[0].data_ptr(), d_in[1].data_ptr(), d_in[2].data_ptr(),
                                  A.nnz, d_b[0].data_ptr(), d_b[1].data_ptr(), d_b[2].data_ptr(), B.nnz,
                                  C.byref(rp2), C.byref(cp2), C.byref(vp2), C.byref(nnz), st), h.h)
        jobs = []
        for hb, dp, cnt, ts in ((h_out[0], rp2, n + 1, "<i4"), (h_out[1], cp2, nnz_c, "<i4"),
                                (h_out[2], vp2, nnz_c, vstr)):
            dv = torch.as_tensor(ops._DevArray(dp.value, cnt, ts), device=dev)
            parts = 1 if cnt < (1 << 20) else 2
            cuts = [cnt * k // parts for k in range(parts + 1)]
            for a, b in zip(cuts[:-1], cuts[1:]):
                jobs.append(lambda hb=hb, dv=dv, a=a, b=b: hb[a:b].copy_(dv[a:b], non_blocking=True))
        fan_out(jobs)
        e1.record(stream)
        torch.cuda.synchronize()
        release((rp2, cp2, vp2))
        if i >= warmup:
            e2e_ms.append(e0.elapsed_time(e1))
    lat_t = max_over_ranks(float(np.mean(e2e_ms)), world, dev)
    lat_gf = world * 2.0 * P / (lat_t * 1e-3) / 1e9

    # End to end, pipelined two deep: the host link is full duplex, so step i+1's inputs go
    # up and step i's C comes down on copy streams while the SpGEMMs run on `stream` — the
    # way a serving loop keeps the device busy.  Every step's H2D of its inputs and D2H of
    # all of its C lie inside the timed region; C's device arrays are released once their
    # copy has landed.  (No L2 flush inside: the transfers stream through L2 themselves.)
    d_in2 = [d_in, [torch.empty_like(x, device=dev) for x in pin]]
    h_out2 = [h_out, [torch.empty_like(x).pin_memory() for x in h_out]]
    up = torch.cuda.Stream(device=dev)

    def issue_h2d(slot):
        ev = torch.cuda.Event()
        with torch.cuda.stream(up):
            for d, p in zip(d_in2[slot], pin):
                d.copy_(p, non_blocking=True)
        ev.record(up)
        return ev

    def issue_d2h(slot, ptrs):
        ready = torch.cuda.Event()
        ready.record(stream)
        done = []
        k = 0
        for hb, dp, cnt, ts in ((h_out2[slot][0], ptrs[0], n + 1, "<i4"), (h_out2[slot][1], ptrs[1], nnz_c, "<i4"),
                                (h_out2[slot][2], ptrs[2], nnz_c, vstr)):
            dv = torch.as_tensor(ops._DevArray(dp.value, cnt, ts), device=dev)
            parts = 1 if cnt < (1 << 20) else 2
            cuts = [cnt * q // parts for q in range(parts + 1)]
            for a, b in zip(cuts[:-1], cuts[1:]):
                cs = copy_streams[k % len(copy_streams)]
                k += 1
                cs.wait_event(ready)
                with torch.cuda.stream(cs):
                    hb[a:b].copy_(dv[a:b], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                done.append(ev)
        return done

    def pipelined(nsteps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        up.wait_event(e0)
        h2d_ev = issue_h2d(0)
        pending = None
        for i in range(nsteps):
            slot = i % 2
            stream.wait_event(h2d_ev)
            if i + 1 < nsteps:  # the next inputs go up now: their buffers were last read by step i - 1
                h2d_ev = issue_h2d(1 - slot)
            di = d_in2[slot]
            db = di[:3] if same else di[3:]
            rp3, cp3, vp3 = C.c_void_p(), C.c_void_p(), C.c_void_p()
            nz3 = C.c_int64(0)
            capi.check(lib.ops_spgemm(h.h, code, n, n, n, di[0].data_ptr(), di[1].data_ptr(), di[2].data_ptr(),
                                      A.nnz, db[0].data_ptr(), db[1].data_ptr(), db[2].data_ptr(), B.nnz,
                                      C.byref(rp3), C.byref(cp3), C.byref(vp3), C.byref(nz3), st), h.h)
            done = issue_d2h(slot, (rp3, cp3, vp3))
            if pending is not None:
                for ev in pending[1]:
                    stream.wait_event(ev)
                release(pending[0])
            pending = ((rp3, cp3, vp3), done)
        for ev in pending[1]:
            stream.wait_event(ev)
        release(pending[0])
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps

    pipelined(max(warmup, 2))
    e2e_t = max_over_ranks(pipelined(max(steps, 4)), world, dev)
    e2e_gf = world * 2.0 * P / (e2e_t * 1e-3) / 1e9

    peak, peak_kind = measured_peak()
    nnz_a = len(col)
    balg = bytes_alg(n, n, nnz_a, len(bcol), nnz_c, s)
    achieved = balg / (t_ms * 1e-3) / 1e9
    traffic, traffic_src = measured_traffic(f'{desc["workload"]}/{dt}')
    kms = phases["kernel_ms"]
    names = ["R8", "R16", "R32", "W", "E1", "E2", "D"]
    per_kernel = {f"{ph}_{names[c]}": round(kms[i][c], 4) for i, ph in enumerate(("symbolic", "numeric"))
                  for c in range(7) if kms[i][c] > 0}
    line = {
        "value": gflops, "unit": "GFLOPS", "steps": steps, "warmup": warmup, "ms_per_step": t_ms, "dtype": dt,
        "config": dict(desc, l2="flushed between steps (256 MiB write outside the timed events)",
                       products=P, nnz_a=nnz_a, nnz_c=nnz_c, parallelism=f"replica x{world}",
                       short_rows="one pass" if args.one_pass else "two passes"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": "whole SpGEMM pipeline (all launches of one C=A*B); achieved and traffic per step",
                     "algorithmic_bytes": balg, "peak_kind": peak_kind},
        "phases_ms": {k: round(phases[k] * 1e3, 4) for k in ("symbolic_binning", "symbolic", "prefix", "allocate",
                                                             "numeric", "total")},
        "kernels_ms": per_kernel,
        "class_rows": dict(zip(names, phases["class_rows"])),
        "subclass_rows": subclass,
        "e2e": {"value": e2e_gf, "unit": "GFLOPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_t, "steps": max(steps, 4),
                "mode": "pipelined two deep: step i+1's H2D and step i's D2H on copy streams overlap the "
                        "SpGEMMs; every step's copies inside the timed region",
                "latency_ms_per_step": lat_t, "latency_value": lat_gf,
                "latency_mode": "one step at a time: H2D, ops_spgemm, D2H of all of C"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if side and dt == "f64" and world == 1 and args.reference_gpu:
        line["reference_gpu"] = reference_gpu(A, B, n, P, nnz_c, t_ms, flush)
    if side and world == 1 and args.cusparse:
        line["cusparse_gpu"] = cusparse_gpu(A, B, n, P, nnz_c, t_ms, flush)
    if side and args.cpu_baseline and world == 1:
        t_cpu, cores, ref = cpu_baseline(data, n)
        line["cpu_baseline"] = {"value": 2.0 * P / t_cpu / 1e9, "unit": "GFLOPS", "cores": cores, "kind": "port",
                                "sample": "full workload, median of 3 runs after 1 warm-up, FP64, OpenMP row-wise "
                                          "hash Gustavson on the host cores"}
        # the last end-to-end step's C (in the pinned host buffers) against the baseline's
        try:
            gpu_c = (h_out[0][:n + 1].numpy(), h_out[1][:nnz_c].numpy(), h_out[2][:nnz_c].numpy())
            line["parity"] = parity_report(gpu_c, ref, dt, scale_fn=_abs_sums_fn(data))
        except Exception as exc:  # a report, never a reason to lose the measurement
            line["parity"] = {"error": f"{type(exc).__name__}: {exc}"}
    h.close()
    del A, B, flush, d_in, pin, h_out
    torch.cuda.empty_cache()
    return line


def _abs_sums_fn(data):
    """sum_j |a_ij b_jk| per output entry of a workload (the OpenMP port over |A| and |B|,
    whose output has C's structure): the scale of FP32 rounding in cancelling entries."""
    def f():
        import oracle

        (ar, ac, av), (br, bc, bv) = _pair(data)
        return oracle.omp_spgemm(ar, ac, np.abs(np.asarray(av, dtype=np.float64)), br, bc,
                                 np.abs(np.asarray(bv, dtype=np.float64)))[2]

    return f


def run_ours(args, desc, dt, data, n, rank, world, local_rank):
    line = measure_plain(args, desc, dt, data, n, world, local_rank, args.steps, args.warmup, side=(rank == 0))
    line = {"metric": METRIC, "value": line.pop("value"), "unit": line.pop("unit"), "n_gpus": world,
            "steps": line.pop("steps"), "warmup": line.pop("warmup"), "ms_per_step": line.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": line.pop("dtype"),
            "data": "synthetic (seeded stand-in for the SuiteSparse inputs)", **line}
    if world == 1 and args.configs and args.workload == "web":
        line["configs"] = other_configs(args, local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def other_configs(args, local_rank):
    """The benchmark's other configurations, measured in the same run as the headline: the
    Laplacian, the 27-point stencil in FP64 and FP32 and the A*A^T power-law forward (each
    as the headline: device and end-to-end time, roofline, CPU baseline, measured error,
    OpSparse's kernels and cuSPARSE on the same GPU), the 4,096-problem batch against the
    per-call loop, and forward + backward against the forward.  Fewer steps for the heavy
    legs; each entry states its own."""
    out = {}
    for name, wl, steps in (("C1", "laplacian", args.steps), ("C3_f64", "stencil27", max(3, args.steps // 2)),
                            ("C3_f32", "stencil27_f32", max(3, args.steps // 2)),
                            ("C5_forward_f64", "powerlaw_AAt", max(3, args.steps // 2))):
        try:
            desc, dt, data, n = make_workload(wl)
            out[name] = measure_plain(args, desc, dt, data, n, 1, local_rank, steps, 3, side=True)
        except Exception as exc:  # one configuration failing must not lose the others
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
    try:
        out["C4_batched"] = measure_batched(args, local_rank, args.batch, reps_loop=2, reps_batch=2,
                                            reps_replay=max(3, args.steps // 2))
    except Exception as exc:
        out["C4_batched"] = {"error": f"{type(exc).__name__}: {exc}"}
    for name, dtn in (("C5_fwd_bwd_f64", "f64"), ("C5_fwd_bwd_f32", "f32")):
        try:
            out[name] = measure_backward(local_rank, dtn, steps=max(3, args.steps // 2), warmup=3)
        except Exception as exc:
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="web",
                    choices=["web", "laplacian", "stencil27", "stencil27_f32", "powerlaw_AAt", "batched", "backward",
                             "backward_f32"])
    ap.add_argument("--batch", type=int, default=4096, help="problems in the batched workload")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-cusparse", dest="cusparse", action="store_false",
                    help="skip timing cuSPARSE's SpGEMM on the same inputs")
    ap.add_argument("--two-pass", dest="one_pass", action="store_false",
                    help="count and compute every row in separate passes (no staging of short rows)")
    ap.add_argument("--no-reference-gpu", dest="reference_gpu", action="store_false",
                    help="skip timing OpSparse's own kernels on the GPU (for profiling runs)")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="measure the chosen workload only (by default the headline run also measures the other "
                         "configurations, the batch and forward+backward, reported under 'configs')")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local_rank)
        dist.init_process_group(backend=backend)
    if args.workload == "batched":
        run_batched(args, rank, world, local_rank)
    elif args.workload.startswith("backward"):
        run_backward(args, rank, world, local_rank)
    else:
        desc, dt, data, n = make_workload(args.workload)
        run_plain(args, desc, dt, data, n, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


def run_plain(args, desc, dt, data, n, rank, world, local_rank):
    if args.impl == "reference":
        run_reference(args, desc, dt, data, n, rank, world)
    else:
        run_ours(args, desc, dt, data, n, rank, world, local_rank)


# ------------------------------------------------------------------- batched workload
def _timed(fn, reps, stream=None):
    """Median of `reps` CUDA-event times of fn() (synchronized on both sides)."""
    import torch

    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def measure_batched(args, local_rank, count, reps_loop, reps_batch, reps_replay, sample=8):
    """`count` independent FP32 Erdos-Renyi products (sizes log-uniform in 64..65,536, mean
    degree U(4,32), generated on the device): the per-call loop of ops_spgemm against one
    batch (ops_batch_create + ops_batch_execute, every problem planned and computed) and
    against graph replays of the planned numeric phase; a seeded sample of the batch's
    results against the oracle."""
    import torch

    import opsparse_gb300 as ops
    from opsparse_gb300 import capi, gen_device

    torch.cuda.set_device(local_rank)
    sizes, row_base, a_side, b_side = gen_device.er_batch(count, dtype=torch.float32)
    A = gen_device.problem_slices(sizes, row_base, a_side)
    B = gen_device.problem_slices(sizes, row_base, b_side)
    pairs = []
    for (ar, ac, av, an), (br, bc, bv, bn), n in zip(A, B, sizes):
        pairs.append((ops.CsrMatrix(int(n), int(n), ar, ac, av), ops.CsrMatrix(int(n), int(n), br, bc, bv)))
    lib = capi.load()
    h = ops.Handle()
    stream = torch.cuda.Stream()
    st = C.c_void_p(stream.cuda_stream)

    def loop_once():
        for Ap, Bp in pairs:
            a, b = Ap.ptrs(), Bp.ptrs()
            rp, cp, vp, nz = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_int64()
            capi.check(lib.ops_spgemm(h.h, capi.OPS_F32, Ap.rows, Ap.cols, Bp.cols, a[0], a[1], a[2], Ap.nnz, b[0],
                                      b[1], b[2], Bp.nnz, C.byref(rp), C.byref(cp), C.byref(vp), C.byref(nz), st),
                       h.h)
            for p_ in (rp, cp, vp):
                lib.ops_free(p_, st)

    with torch.cuda.stream(stream):
        loop_once()  # warm-up
        loop_ms = _timed(loop_once, reps_loop, stream)
        holder = {}

        def batched_full():
            if "b" in holder:
                holder["b"].close()
            holder["b"] = ops.Batch(h, pairs, stream=stream)
            holder["b"].execute(False)

        batched_full()
        full_ms = _timed(batched_full, reps_batch, stream)
        bt = holder["b"]
        bt.execute(True)  # records the graph
        replay_ms = _timed(lambda: bt.execute(True), reps_replay, stream)
    bt.check()
    seg, flop, nnz = bt.info()
    persistent, warp_rows, cta_rows = bt.queues()
    # measured error of a seeded sample of the batch's results
    par = {"problems_checked": 0, "structure_identical": True, "within_tolerance": True, "max_abs_err": 0.0,
           "max_rel_err_scaled": 0.0, "entries": 0, "values_bit_identical_to_fp32_oracle": True,
           "tolerance_rel": 1e-5, "checked_against": "oracle (FP64; and FP32 Dot2 for bit identity)"}
    if args.cpu_baseline and sample:
        import oracle

        for i in np.random.default_rng(20261203).choice(len(pairs), min(sample, len(pairs)), replace=False):
            Ap, Bp = pairs[int(i)]
            a = tuple(x.cpu().numpy() for x in (Ap.rpt, Ap.col, Ap.val))
            b = tuple(x.cpu().numpy() for x in (Bp.rpt, Bp.col, Bp.val))
            gpu = bt.result(int(i))
            ref32 = oracle.spgemm(*a, *b, Bp.cols, dtype=np.float32)
            ref64 = oracle.spgemm(a[0], a[1], a[2].astype(np.float64), b[0], b[1], b[2].astype(np.float64), Bp.cols)
            rep = parity_report(gpu, ref64, "f32", scale_fn=_abs_sums_fn((a, b)))
            par["problems_checked"] += 1
            par["structure_identical"] &= bool(rep["structure_identical"])
            par["within_tolerance"] &= bool(rep.get("within_tolerance", False))
            par["max_abs_err"] = max(par["max_abs_err"], rep.get("max_abs_err", float("inf")))
            par["max_rel_err_scaled"] = max(par["max_rel_err_scaled"], rep.get("max_rel_err_scaled") or 0.0)
            par["entries"] += rep.get("entries", 0)
            par["values_bit_identical_to_fp32_oracle"] &= bool(
                np.array_equal(gpu[2].view(np.uint32), ref32[2].view(np.uint32)))
    bt.close()
    h.close()
    del pairs, A, B, a_side, b_side
    torch.cuda.empty_cache()
    return {"value": 2.0 * flop / (full_ms * 1e-3) / 1e9, "unit": "GFLOPS", "dtype": "f32",
            "ms_per_step": full_ms,
            "config": {"workload": f"batched_er_{count}", "problems": count, "sizes": "log-uniform 64..65536",
                       "mean_degree": "U(4,32)", "values": "N(0,1)", "products": flop, "nnz_c": nnz,
                       "segments": seg, "data": "synthetic (device-generated Erdos-Renyi pairs)"},
            "batched": {"loop_ms": loop_ms, "batched_ms": full_ms, "speedup_vs_loop": loop_ms / full_ms,
                        "graph_replay_numeric_ms": replay_ms, "target_speedup": 3.0,
                        "plan": ("one setup kernel, then one persistent kernel per row-size queue and phase over "
                                 "every problem's rows" if persistent else "per segment"),
                        "queue_rows": {"warp": warp_rows, "cta": cta_rows},
                        "reps": {"loop": reps_loop, "batched": reps_batch, "replay": reps_replay}},
            "parity": par}


def run_batched(args, rank, world, local_rank):
    if args.impl == "reference":  # answered without touching a GPU
        if rank == 0:
            print(json.dumps({"metric": METRIC, "impl": "reference", "unavailable":
                              "OpSparse has no batched SpGEMM and no CPU SpGEMM; see the plain workloads"}))
        return
    r = measure_batched(args, local_rank, args.batch, max(1, args.steps // 4), max(1, args.steps // 4), args.steps)
    line = {"metric": METRIC, "value": r.pop("value"), "unit": r.pop("unit"), "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": r["config"].pop("data"), **r}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- backward workload
def measure_backward(local_rank, dtn, steps, warmup):
    """C = A*B with A 200,000^2 power-law (mean degree 16, exponent 2.2) and B = pattern of
    A^T with fresh values; loss = sum(W .* C).  Times the forward (numeric phase on the
    fixed pattern, and the full SpGEMM) and forward + backward (dA, dB); measures the
    gradients' error against the oracle's backward."""
    import torch

    import opsparse_gb300 as ops
    from opsparse_gb300 import gen
    from opsparse_gb300.autograd import FixedPatternSpGEMM

    torch.cuda.set_device(local_rank)
    dt = torch.float32 if dtn == "f32" else torch.float64
    n = 200_000
    a = gen.powerlaw_square(n, 16, 2.2)
    b = gen.transpose_pattern(a[0], a[1], n)
    A = ops.csr_to_device(*a, n, n, dtype=dt)
    B = ops.csr_to_device(*b, n, n, dtype=dt)
    h = ops.Handle()
    op = FixedPatternSpGEMM(A, B, h)
    w = torch.as_tensor(np.random.default_rng(3).standard_normal(op.nnz)).to(dt).cuda()
    flop = int(gen.row_flop(a[0], a[1], b[0]).sum())
    fwd = lambda: op.forward_values(A.val, B.val)  # noqa: E731
    fwdbwd = lambda: (op.forward_values(A.val, B.val), op.backward_values(A.val, B.val, w))  # noqa: E731
    full = lambda: h.spgemm_oneshot(A, B)  # noqa: E731
    for _ in range(max(warmup, 3)):
        fwdbwd()
        full()
    fwd_ms = _timed(fwd, steps)
    fwdbwd_ms = _timed(fwdbwd, steps)
    full_ms = _timed(full, steps)
    products, with_map = op.plan_info()
    # gradients against the oracle's FP64 backward on the same (rounded) inputs
    da, db = op.backward_values(A.val, B.val, w)
    grad = {}
    try:
        import oracle

        av, bv, wv = (x.cpu().numpy().astype(np.float64) for x in (A.val, B.val, w))
        crpt, ccol = op.c_rpt.cpu().numpy().astype(np.int64), op.c_col.cpu().numpy()
        oda, odb = oracle.backward(a[0], a[1], av, b[0], b[1], bv, n, crpt, ccol, wv)
        sda, sdb = oracle.backward(a[0], a[1], np.abs(av), b[0], b[1], np.abs(bv), n, crpt, ccol, np.abs(wv))
        for nm, g, o, sc in (("dA", da, oda, sda), ("dB", db, odb, sdb)):
            g = g.cpu().numpy()
            diff = np.abs(g.astype(np.float64) - o)
            den = np.maximum(np.abs(o), sc * (2.0 ** -24 if dtn == "f32" else 2.0 ** -53))
            rel = np.where(den > 0, diff / np.where(den > 0, den, 1.0), np.where(diff > 0, np.inf, 0.0))
            e = {"entries": int(o.size), "max_abs_err": float(diff.max()) if diff.size else 0.0,
                 "max_rel_err_scaled": float(rel.max()) if rel.size else 0.0,
                 "tolerance_rel": 1e-12 if dtn == "f64" else 1e-5}
            if dtn == "f64":
                e["values_bit_identical"] = bool(np.array_equal(g.view(np.uint64), o.view(np.uint64)))
            e["within_tolerance"] = bool(e["max_rel_err_scaled"] <= e["tolerance_rel"])
            grad[nm] = e
    except Exception as exc:  # a report, never a reason to lose the measurement
        grad = {"error": f"{type(exc).__name__}: {exc}"}
    nnz_c = int(op.nnz)
    h.close()
    del A, B, op, w
    torch.cuda.empty_cache()
    return {"value": 2.0 * flop / (fwdbwd_ms * 1e-3) / 1e9, "unit": "GFLOPS", "dtype": dtn, "steps": steps,
            "ms_per_step": fwdbwd_ms,
            "config": {"workload": "powerlaw_200k_AAt_fwd_bwd", "rows": n, "mean_degree": 16, "exponent": 2.2,
                       "products": flop, "nnz_c": nnz_c},
            "fwd_bwd": {"forward_numeric_ms": fwd_ms, "forward_full_ms": full_ms, "fwd_bwd_ms": fwdbwd_ms,
                        "ratio_vs_numeric_forward": fwdbwd_ms / fwd_ms,
                        "ratio_vs_full_forward": (fwdbwd_ms - fwd_ms + full_ms) / full_ms, "target_ratio": 3.0,
                        "product_map": with_map},
            "gradient_error": grad}


def run_backward(args, rank, world, local_rank):
    if args.impl == "reference":  # answered without touching a GPU
        if rank == 0:
            print(json.dumps({"metric": METRIC, "impl": "reference", "unavailable":
                              "OpSparse has no backward pass; see the plain workloads"}))
        return
    r = measure_backward(local_rank, "f32" if args.workload.endswith("f32") else "f64", args.steps, args.warmup)
    line = {"metric": METRIC, "value": r.pop("value"), "unit": r.pop("unit"), "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r.pop("dtype"), "data": "synthetic", **r}
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
