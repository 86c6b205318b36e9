#!/usr/bin/env python3
"""Benchmark of the block-tensor permute + sector-GEMM path on GB300.

Workload (one step): the iTEBD network of the spin-1/2 Heisenberg chain with
U(1) symmetry, chi = 512 over charges -8..8, d = 2: La-A-Lb-B-Lc-gate
contracted to theta[a,s1'|s2',c] through Network::launch (every pairwise
contract permutes its operands and runs all its sector GEMMs in one grouped
launch), inputs resident in HBM.  Metric: contract() TFLOP/s counted as the
FP64-equivalent sum of 2*M*N*K over the sector GEMMs the reference issues for
this network and ORDER (the same count in every precision mode).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--mode split|fp64|bf16|tf32]
  python bench.py --impl reference ...   # the reference path on the host cores

Under torchrun (N > 1) every rank runs an independent replica (no
collective); rank 0 prints the single JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from trim_gb300 import workloads as wl  # noqa: E402

METRIC = "contract() TFLOP/s (FP64-equivalent sector-GEMM flops), iTEBD chi=512 U(1) step"
WORKLOAD = "itebd_u1_chi512_d2"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2: written between timed steps


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(torch, vals, device):
    """Element-wise maximum of a list of floats over all ranks (a no-op on
    one process): the step times every rank reports are the slowest rank's."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return [float(v) for v in vals]
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def itebd_inputs():
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    return spec, els


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_samples(self, n: int, timeout: float) -> bool:
        """Blocks until n samples have arrived (nvidia-smi takes a moment to start)."""
        t0 = time.time()
        while self.proc and len(self.lines) < n and time.time() - t0 < timeout:
            time.sleep(0.02)
        return len(self.lines) >= n

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- CPU reference
def run_reference_steps(steps: int, warmup: int):
    """The reference path on the host cores: the numpy restatement of
    Network::launch with per-sector BLAS dgemm (the compiled reference does
    not run on this machine's architecture)."""
    from oracle import symtensor as st

    spec, els = itebd_inputs()
    ob = lambda bonds: [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]
    tens = {s.name: st.UniTensor(ob(s.bonds), s.labels, els[s.name]) for s in spec["tensors"]}
    shapes = []
    net = st.Network(text=spec["net"])
    for s in spec["tensors"]:
        net.put_tensor(s.name, tens[s.name])
    net.launch(gemm=lambda a, b: (shapes.append(a.shape + (b.shape[1],)), a @ b)[1])
    flops = sum(2.0 * m * k * n for m, k, n in shapes)

    def step():
        n = st.Network(text=spec["net"])
        for s in spec["tensors"]:
            n.put_tensor(s.name, tens[s.name])
        return n.launch()

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = (time.perf_counter() - t0) / steps
    return flops, dt


def reference_main(args, rank, world):
    if rank != 0:
        return
    flops, dt = run_reference_steps(args.steps, args.warmup)
    v = flops / dt / 1e12
    cores = os.cpu_count()
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "chi": 512, "sectors": 17, "flops_per_step": flops, "mode": "fp64"},
        "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full iTEBD network steps, numpy BLAS on {cores} host threads"},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ----------------------------------------------------------------- GPU arm
def _itebd_device(tu, spec, els):
    names = [s.name for s in spec["tensors"]]
    dev = {s.name: tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]}
    net = tu.Network(spec["net"])
    for n in names:
        net.put_tensor(n, dev[n])
    return names, dev, net


def measured_fp64_peak(torch, n=4096, reps=5):
    """FP64 denominator measured in this run: cuBLAS DGEMM (torch.matmul on
    float64) of n x n x n, best of `reps` after two warm-ups, CUDA events."""
    a = torch.rand(n, n, dtype=torch.float64, device="cuda")
    b = torch.rand(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        c = a @ b
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def _time_steps(torch, stream, flush, steps, fn):
    """CUDA-event time per step on the library stream, L2 flushed between steps."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))  # between timed steps, outside the events
        starts[k].record(stream)
        fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps


def _timed_with_clocks(torch, stream, flush, steps, fn, gpu, min_seconds=1.0, max_reps=400):
    """Repeats the timed region (exactly `steps` steps, CUDA events) until the
    clock sampler has seen at least 3 samples and min_seconds have passed
    (min_seconds 0: one repetition); returns the median ms per step over the
    repetitions, their count and the clocks sampled while they ran."""
    reps = []
    with ClockSampler(gpu) as clk:
        clk.wait_samples(1, 10.0)
        n0 = len(clk.lines)
        t0 = time.time()
        while len(reps) < max_reps:
            reps.append(_time_steps(torch, stream, flush, steps, fn))
            if min_seconds <= 0 or (time.time() - t0 >= min_seconds and len(clk.lines) - n0 >= 3):
                break
        clk.lines = clk.lines[n0:]
    return statistics.median(reps), len(reps), clk.summary()


def gpu_main(args, rank, local, world):
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    if args.autotune:  # FP64 GEMM policies timed per sector histogram on the first eager launch
        tu.autotune(True)
    spec, els = itebd_inputs()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    modes = ["fp64"] + ([args.mode] if args.mode != "fp64" else [])
    res = {}
    ref64 = None
    for mode in modes:
        names, dev, net = _itebd_device(tu, spec, els)
        for _ in range(args.warmup):
            th = net.launch(mode)
        vals = th.get_elem()
        if mode == "fp64":
            ref64 = vals
        err = float(np.linalg.norm(vals - ref64) / np.linalg.norm(ref64))
        net.capture(mode)  # the whole Network::launch as one CUDA graph
        out = net.output()
        for _ in range(args.warmup):
            net.replay()
        tu.sync()
        graph_ok = bool(np.array_equal(out.get_elem(), vals))
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = tu.launch_count()
        ms_graph, reps, clocks = _timed_with_clocks(torch, stream, flush, args.steps, net.replay, local,
                                                    min_seconds=args.clock_seconds)
        launches = (tu.launch_count() - l0) // (args.steps * reps)
        ms_eager = _time_steps(torch, stream, flush, args.steps, lambda: net.launch(mode))
        # per-kernel times: eager pass with events around every launch
        tu.prof_enable(True)
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            net.launch(mode)
        prof = tu.prof_read()
        tu.prof_enable(False)
        flops = sum(v["flops"] for k_, v in prof.items() if "gemm" in k_) / args.steps
        # end to end through the C ABI: the graph recaptured with the pinned
        # host inputs bound (copied into the network's tensors at its start)
        # and theta bound to a pinned host buffer (copied out at its end); a
        # step is one replay and the synchronisation that completes it
        pinned = {n: torch.from_numpy(els[n]).pin_memory() for n in names}
        out_host = torch.empty(vals.size, dtype=torch.float64).pin_memory()
        for n in names:
            net.bind_host_input(n, pinned[n].data_ptr(), els[n].size)
        net.bind_host_output(out_host.data_ptr(), vals.size)
        net.capture(mode)
        net.replay()
        tu.sync()
        e2e_ok = bool(np.array_equal(out_host.numpy(), vals))
        e2e = []
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            net.replay()
            tu.sync()
            e2e.append((time.perf_counter() - w0) * 1e3)
        res[mode] = {"ms_graph": ms_graph, "ms_eager": ms_eager, "flops": flops, "err_vs_fp64": err,
                     "graph_matches_eager": graph_ok, "launches": int(launches), "clocks": clocks, "timed_repeats": reps,
                     "e2e_ms": statistics.median(e2e), "e2e_matches_device": e2e_ok, "prof": prof,
                     "h2d": sum(8 * els[n].size for n in names), "d2h": 8 * vals.size}
    if world > 1:
        for m in res:
            res[m]["ms_graph"], res[m]["e2e_ms"] = max_over_ranks(torch, [res[m]["ms_graph"], res[m]["e2e_ms"]], "cuda")

    svd = itebd_svd_section(args, torch, tu, stream, flush, spec, els, ref64, rank, world)
    eigh = itebd_eigh_section(args, torch, tu, stream, flush, spec, els, ref64, rank, world)

    head = modes[-1]
    R = res[head]
    flops = R["flops"]
    value = world * flops / (R["ms_graph"] * 1e-3) / 1e12
    prof = R["prof"]
    # roofline of the dominant kernel of the headline mode
    dname, d = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    avg_ms = d["ms"] / d["launches"]
    if dname == "permute":
        ach = d["bytes"] / d["launches"] / (avg_ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    elif dname == "gemm_fp64":
        ach = d["flops"] / d["launches"] / (avg_ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": ach, "peak": measured_fp64_peak(torch), "unit": "TFLOP/s",
                "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5",
                "peak_nominal": 1.25}
    elif dname == "tc_slice":
        ach = d["bytes"] / d["launches"] / (avg_ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    else:  # tensor-core GEMM: tensor-pipe work = 34 BF16 digit products per FP64-equivalent flop
        pairs = 34 if "split" in dname else 1
        ach = pairs * d["flops"] / d["launches"] / (avg_ms * 1e-3) / 1e12
        peak = peaks.get("bf16_tflops", 1900.0)
        roof = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "peak_source": "measured (burst)" if "bf16_tflops" in peaks else "fallback",
                "work": "BF16 tensor flops (34 digit products per FP64-equivalent flop)" if pairs > 1 else "BF16 flops"}
    roof.update({"kernel": dname, "frac": roof["achieved"] / roof["peak"], "avg_launch_ms": avg_ms, "traffic": None})
    if dname == "gemm_fp64":
        # dram__bytes_read.sum + dram__bytes_write.sum per launch, mean over the
        # network's five gemm_fp64 launches (grids 545/593/667/762/543), from one
        # ncu capture of `bench.py --no-cpu --steps 3 --warmup 3 --clock-seconds 0`
        roof.update({"traffic": 880589.0, "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu, mean over the 5 network launches (reads 0.73-1.12 MB, writes 0: "
                                       "outputs stay in L2)",
                     "algorithmic_bytes_per_launch": d["bytes"] / d["launches"]})
    kernels = {k_: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps}
               for k_, v in prof.items()}
    pbytes = prof.get("permute", {}).get("bytes", 0.0)
    pms = prof.get("permute", {}).get("ms", 0.0)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        f_, dt1 = run_reference_steps(1, 1)
        n = max(3, int(args.cpu_seconds / max(dt1, 1e-4)))
        f_, dtc = run_reference_steps(n, 0)
        cpu = {"value": f_ / dtc / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} full iTEBD network steps (the whole workload), numpy BLAS on {os.cpu_count()} host threads"}

    if rank == 0:
        modes_out = {m: {k: v for k, v in r.items() if k != "prof"} for m, r in res.items()}
        for m, r in modes_out.items():
            r["tflops_graph"] = world * r["flops"] / (r["ms_graph"] * 1e-3) / 1e12
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": R["ms_graph"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f64 (bf16 digit slices on tcgen05)",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "chi": 512, "sectors": 17, "mode": head, "flops_per_step": flops,
                       "execution": "Network::launch captured as one CUDA graph, replayed per step",
                       "fp64_policy": "autotuned per sector histogram" if args.autotune else "default",
                       "l2": "flushed between timed steps (512 MB write)", "parallelism": f"replicas x{world}"},
            "error_vs_fp64": R["err_vs_fp64"],
            "speedup_vs_fp64_gpu": res["fp64"]["ms_graph"] / R["ms_graph"],
            "modes": modes_out,
            "permute": {"gb_s": (pbytes / (pms * 1e-3) / 1e9) if pms else None, "bytes_per_step": pbytes / args.steps},
            "kernels": kernels,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": world * flops / (R["e2e_ms"] * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": R["e2e_ms"],
                    "h2d_bytes_per_step": R["h2d"], "d2h_bytes_per_step": R["d2h"]},
            "clocks": R["clocks"],
            "gpu_launches": R["launches"],
            "svd_truncate": svd,
            "eigh": eigh,
            "itebd_step_ms": {"contract_graph": R["ms_graph"], "svd_truncate": svd["ms_gpu"],
                              "total": R["ms_graph"] + svd["ms_gpu"],
                              "cpu_port_total": (svd["ms_cpu_port"] + (flops / cpu["value"] / 1e9 if cpu else 0.0))
                              if svd["ms_cpu_port"] is not None and cpu else None},
        }))


def itebd_eigh_section(args, torch, tu, stream, flush, spec, els, theta64, rank, world):
    """Block::eigh of every (square) sector of the iTEBD theta, lower triangle
    read as dsyev 'U' reads the reference's row-major buffer: one batched call
    (scaled shift, cluster-Jacobi SVD, Rayleigh quotients).  Wall time per
    call, kernel device times, and the eigenvalue error against LAPACK dsyev
    per sector (the oracle), which is also the timed CPU port."""
    from oracle import symtensor as st

    names, dev, net = _itebd_device(tu, spec, els)
    th = net.launch("fp64")
    blocks = [b for b in th.sector_map().blocks() if b[1] == b[2]]
    secs, eo = [], 0
    for _, r, _, off in blocks:
        secs.append((r, off, eo, off))
        eo += r
    E = torch.empty(max(eo, 1), dtype=torch.float64, device="cuda")
    V = torch.empty(max(th.elem_num(), 1), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    run = lambda: tu.eigh_sectors(secs, th.device_ptr(), E.data_ptr(), V.data_ptr())
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    wall = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run()
        tu.sync()
        wall.append((time.perf_counter() - t0) * 1e3)
    tu.prof_enable(True)
    run()
    prof = tu.prof_read()
    tu.prof_enable(False)
    tu.sync()
    e = E.cpu().numpy()
    out = {"sectors": len(secs), "ms_gpu": statistics.median(wall), "kernels_ms": {k_: v["ms"] for k_, v in prof.items()}}
    cpu_ms = None
    if rank == 0 and world == 1:
        mats = [theta64[off:off + r * r].reshape(r, r) for _, r, _, off in blocks]
        t0 = time.perf_counter()
        ref = [st.block_eigh(m)[0] for m in mats]
        dt1 = time.perf_counter() - t0
        err = max(float(np.max(np.abs(e[o:o + r] - er)) / max(np.max(np.abs(er)), 1e-300))
                  for (r, _, o, _), er in zip(secs, ref))
        n = 0 if args.no_cpu else max(1, min(50, int(0.2 * args.cpu_seconds / max(dt1, 1e-3))))
        if n:
            t0 = time.perf_counter()
            for _ in range(n):
                for m in mats:
                    st.block_eigh(m)
            cpu_ms = (time.perf_counter() - t0) / n * 1e3
        out.update({"eig_max_err_rel": err,
                    "cpu_port_sample": f"{n} x {len(mats)} Block::eigh (LAPACK dsyev, numpy) on {os.cpu_count()} threads"})
    out["ms_cpu_port"] = cpu_ms
    return out


def itebd_svd_section(args, torch, tu, stream, flush, spec, els, theta64, rank, world):
    """The rest of the iTEBD step on the FP64 theta: per-sector FP64 SVD (one
    batched cluster-Jacobi launch), the global top-chi truncation and the
    normalisation (UniTensor-level svd_truncate).  Wall time per call (it ends
    with the host read of the kept counts, as the reference's step does), the
    kernels' device times, and the error of the kept singular values against
    LAPACK (the oracle)."""
    from oracle import symtensor as st

    chi = 512
    names, dev, net = _itebd_device(tu, spec, els)
    th = net.launch("fp64")
    for _ in range(args.warmup):
        th.svd_truncate(chi)
    torch.cuda.synchronize()
    wall = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        th.svd_truncate(chi)
        wall.append((time.perf_counter() - t0) * 1e3)
    tu.prof_enable(True)
    U, S, VT, norm = th.svd_truncate(chi)
    prof = tu.prof_read()
    tu.prof_enable(False)
    # accuracy against LAPACK dgesvd per sector (the oracle), same theta
    ob = lambda bonds: [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]
    tho = st.UniTensor(ob(th.bonds()), th.labels(), theta64)
    out = {"ms_gpu": statistics.median(wall), "norm": norm,
           "kernels_ms": {k_: v["ms"] for k_, v in prof.items()}}
    cpu_ms = None
    if rank == 0 and world == 1:
        t0 = time.perf_counter()
        Uo, So, VTo, norm_o = st.svd_truncate(tho, chi)
        dt1 = time.perf_counter() - t0
        n = 0 if args.no_cpu else max(1, min(50, int(0.3 * args.cpu_seconds / max(dt1, 1e-3))))
        if n:
            t0 = time.perf_counter()
            for _ in range(n):
                st.svd_truncate(tho, chi)
            cpu_ms = (time.perf_counter() - t0) / n * 1e3
        kept_same = [r[3] for r in S.bonds()[0][1]] == So.bonds[0].qdegs
        out.update({"kept_counts_match_oracle": bool(kept_same),
                    "kept_sv_max_err_rel": float(np.max(np.abs(S.get_elem() - So.elem))) if kept_same else None,
                    "norm_err_rel": abs(norm - norm_o) / norm_o,
                    "cpu_port_sample": f"{n} svd_truncate calls (LAPACK dgesvd per sector, numpy) on {os.cpu_count()} threads"})
    out["ms_cpu_port"] = cpu_ms
    return out


def permute_main(args, rank, local, world):
    """Large dense permute (HBM-bound): a chi^6 tensor, bonds (3 in | 3 out)
    permuted to (4 5 0 | 1 2 3) -- the operand permute a MERA ascending
    contraction issues.  Bit-exact check against numpy on a slice."""
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    chi = args.chi
    bonds = [wl.dense_bond(1, chi)] * 3 + [wl.dense_bond(-1, chi)] * 3
    n = chi ** 6
    c128 = args.c128  # complex (cflag) elements: 16-byte (re, im) pairs
    esz = 16 if c128 else 8
    x = torch.randn(n, dtype=torch.complex128 if c128 else torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(5))
    perm = [int(v) for v in args.perm.split(",")]
    rn = args.perm_rownum
    src_map = tu.SectorMap(bonds)
    dst_bonds = [wl.change(bonds[p], 1 if i < rn else -1) for i, p in enumerate(perm)]
    dst_map = tu.SectorMap(dst_bonds)
    y = torch.empty_like(x)
    torch.cuda.synchronize()  # x is written on torch's stream, read on the library's
    run = tu.permute_device_c128 if c128 else tu.permute_device
    for _ in range(args.warmup):
        run(src_map, dst_map, perm, x.data_ptr(), y.data_ptr())
    tu.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for s_, e_ in ev:
            s_.record(stream)
            run(src_map, dst_map, perm, x.data_ptr(), y.data_ptr())
            e_.record(stream)
        torch.cuda.synchronize()
    ms = statistics.median(s_.elapsed_time(e_) for s_, e_ in ev)
    gbs = 2.0 * esz * n / (ms * 1e-3) / 1e9
    y_keep = y.clone()
    # same-size device-to-device copy on the same stream: the plain-copy ceiling
    cev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for s_, e_ in cev:
            s_.record(stream)
            y.copy_(x)
            e_.record(stream)
    torch.cuda.synchronize()
    copy_gbs = 2.0 * esz * n / (statistics.median(s_.elapsed_time(e_) for s_, e_ in cev) * 1e-3) / 1e9
    exact = bool(torch.equal(y_keep, x.view([chi] * 6).permute(*perm).reshape(-1)))
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    if rank == 0:
        print(json.dumps({"metric": f"permute GB/s ({2 * esz} B per element)", "value": gbs, "unit": "GB/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                          "dtype": "c128" if c128 else "f64",
                          "bit_exact": exact, "copy_gb_s": copy_gbs, "config": {"workload": f"dense_rank6_chi{chi}_permute" + ("_c128" if c128 else ""),
                                                         "elements": n, "perm": perm, "l2": "inputs larger than L2"},
                          "roofline": {"kernel": "permute", "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                       "frac": gbs / peak, "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
                          "clocks": clk.summary()}))


def mera_main(args, rank, local, world):
    """Dense ternary MERA ascending superoperator, chi = args.chi: the three
    diagrams through Network::launch in FP64 and in the tensor-core modes;
    time, FP64-equivalent TFLOP/s, error of each mode against the FP64 GPU
    result and the Hermiticity of the ascended operator."""
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    spec = wl.mera(chi=args.chi)
    rng = np.random.default_rng(0)
    dev = {s.name: tu.UniTensor(s.bonds, s.labels, wl.gen_elems(s, rng)) for s in spec["tensors"]}
    nets = {d: tu.Network(t) for d, t in spec["nets"].items()}

    def run(mode):
        outs = {}
        for d, net in nets.items():
            for s in spec["tensors"]:
                net.put_tensor(s.name, dev[s.name])
            outs[d] = net.launch(mode)
        return outs

    modes = ["fp64"] + [m for m in args.modes.split(",") if m != "fp64"]
    res = {}
    ref = None
    for mode in modes:
        out = run(mode)  # warm-up: plans and workspaces
        tu.sync()
        tu.prof_enable(True)
        s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_.record(stream)
        out = run(mode)
        e_.record(stream)
        torch.cuda.synchronize()
        prof = tu.prof_read()
        tu.prof_enable(False)
        ms = s_.elapsed_time(e_)
        flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k)
        vals = {d: t.get_elem() for d, t in out.items()}
        if mode == "fp64":
            ref = vals
        err = max(float(np.linalg.norm(vals[d] - ref[d]) / np.linalg.norm(ref[d])) for d in vals)
        herm = 0.0
        chi2 = args.chi ** 2
        for d, v in vals.items():
            m = v.reshape(chi2, chi2)
            herm = max(herm, float(np.linalg.norm(m - m.T) / np.linalg.norm(m)))
        res[mode] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "flops": flops, "err_vs_fp64": err,
                     "hermiticity": herm,
                     "kernels": {k: {"ms": v["ms"], "launches": v["launches"]} for k, v in prof.items()}}
    if rank == 0:
        best = modes[-1]
        print(json.dumps({"metric": "contract() TFLOP/s (FP64-equivalent), dense ternary MERA ascend, 3 diagrams",
                          "value": res[best]["tflops"], "unit": "TFLOP/s", "n_gpus": world, "higher_is_better": True,
                          "config": {"workload": f"mera_ternary_chi{args.chi}", "modes": modes}, "modes": res,
                          "speedup_vs_fp64": {m: res["fp64"]["ms"] / res[m]["ms"] for m in modes}}))


def ipeps_device(tu, spec, rng_seed=None):
    """Device tensors of the Z2 iPEPS CTM quadrant: the double-layer site
    a.a* over p with each (x, x') pair combined, then C, T1, T2."""
    rng = np.random.default_rng(spec["seed"] if rng_seed is None else rng_seed)
    site, C_, T1, T2 = spec["tensors"]
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    a = tu.UniTensor(site.bonds, site.labels, els["a"])
    ac = a.copy()
    ac.set_label([0, 11, 12, 13, 14])
    aa = tu.contract(a, ac, mode="fp64")
    for x in (1, 2, 3, 4):
        aa.combine_bond([x, x + 10])
    aa.permute(aa.labels(), 2)
    aa.set_label([10, 20, 30, 40])
    dev = {"A2": aa}
    for s in (C_, T1, T2):
        dev[s.name] = tu.UniTensor(s.bonds, s.labels, els[s.name])
    return dev, els


def ipeps_main(args, rank, local, world):
    """Z2-symmetric iPEPS double-layer CTM quadrant, chi = 128, D = 8:
    C.T1.T2.A2 through Network::launch (ORDER (((C T1) T2) A2)) in FP64, split
    and fast BF16; time, FP64-equivalent TFLOP/s and error vs FP64."""
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    spec = wl.ipeps_ctm(chi=args.chi_ctm, D=args.D)
    dev, _ = ipeps_device(tu, spec)
    net = tu.Network(spec["net"])
    for n, t in dev.items():
        net.put_tensor(n, t)
    res, ref = {}, None
    for mode in ["fp64"] + [m for m in args.modes.split(",") if m != "fp64"]:
        net.launch(mode)
        tu.sync()
        tu.prof_enable(True)
        s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_.record(stream)
        q = net.launch(mode)
        e_.record(stream)
        torch.cuda.synchronize()
        prof = tu.prof_read()
        tu.prof_enable(False)
        ms = s_.elapsed_time(e_)
        v = q.get_elem()
        if mode == "fp64":
            ref = v
        flops = sum(x["flops"] for k, x in prof.items() if "gemm" in k)
        res[mode] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "flops": flops,
                     "err_vs_fp64": float(np.linalg.norm(v - ref) / np.linalg.norm(ref)),
                     "kernels": {k: {"ms": x["ms"], "launches": x["launches"]} for k, x in prof.items()}}
    if rank == 0:
        best = [m for m in res if m != "fp64"][0] if len(res) > 1 else "fp64"
        print(json.dumps({"metric": "contract() TFLOP/s (FP64-equivalent), Z2 iPEPS CTM quadrant",
                          "value": res[best]["tflops"], "unit": "TFLOP/s", "n_gpus": world, "higher_is_better": True,
                          "config": {"workload": f"ipeps_ctm_z2_chi{args.chi_ctm}_D{args.D}", "elements_out": int(ref.size)},
                          "modes": res, "speedup_vs_fp64": {m: res["fp64"]["ms"] / r["ms"] for m, r in res.items()}}))


def batched_main(args, rank, local, world):
    """1024 independent uneven U(1) contractions T1[x|y,z].T2[y,z|w]: one
    grouped launch (all 8k sector GEMMs) against a per-contraction loop and a
    per-sector loop (one GEMM launch per sector, as the reference issues
    them), in FP64 and split precision."""
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    spec = wl.batched(n=args.batch)
    rng = np.random.default_rng(spec["seed"])
    A, B = [], []
    for t1, t2 in spec["pairs"]:
        A.append(tu.UniTensor(t1.bonds, t1.labels, wl.gen_elems(t1, rng)))
        B.append(tu.UniTensor(t2.bonds, t2.labels, wl.gen_elems(t2, rng)))
    # the per-sector loop needs each pair's sector list (same order as contract issues it)
    sectors = []
    for t1, t2 in spec["pairs"]:
        a = {q: (r, c, 0) for q, r, c in wl.block_shapes(t1.bonds)}
        b = {q: (r, c) for q, r, c in wl.block_shapes(t2.bonds)}
        oa = ob = 0
        offa, offb = {}, {}
        for q, r, c in wl.block_shapes(t1.bonds):
            offa[q] = oa
            oa += r * c
        for q, r, c in wl.block_shapes(t2.bonds):
            offb[q] = ob
            ob += r * c
        outb = [(1, t1.bonds[0][1]), (-1, t2.bonds[2][1])]
        offc, oc = {}, 0
        for q, r, c in wl.block_shapes(outb):
            offc[q] = oc
            oc += r * c
        sectors.append([(a[q][0], b[q][1], a[q][1], offa[q], offb[q], offc[q]) for q in offa if q in offb])
    nsec = sum(len(x) for x in sectors)

    def timed(fn):
        fn()
        tu.sync()
        s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_.record(stream)
        r = fn()
        e_.record(stream)
        torch.cuda.synchronize()
        return s_.elapsed_time(e_), r

    res = {}
    ref = None
    for mode in ["fp64", args.mode] if args.mode != "fp64" else ["fp64"]:
        tu.prof_enable(True)
        ms_g, outs = timed(lambda: tu.contract_batch(A, B, mode))
        prof = tu.prof_read()
        tu.prof_enable(False)
        flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k) / 2  # prof spans warm-up + timed call
        vals = [o.get_elem() for o in outs]
        ms_c, outs_c = timed(lambda: [tu.contract(a, b, mode=mode) for a, b in zip(A, B)])
        same = max(float(np.linalg.norm(o.get_elem() - v) / max(np.linalg.norm(v), 1e-300)) for o, v in zip(outs_c, vals))
        outs_c = None
        cbuf = [o for o in outs]  # the grouped outputs are the C buffers of the per-sector loop

        def per_sector():
            for a, b, c, secs in zip(A, B, cbuf, sectors):
                for g in secs:
                    tu.contract_sectors(mode, [g], a.device_ptr(), b.device_ptr(), c.device_ptr())

        ms_s, _ = timed(per_sector)
        # the same grouped call with the FP64 GEMM autotuner (tile width and
        # K split chosen per sector-size histogram; tuned in the untimed call)
        tu.autotune(True)
        ms_t, outs_t = timed(lambda: tu.contract_batch(A, B, mode))
        tuned_same = max(float(np.linalg.norm(o.get_elem() - v) / max(np.linalg.norm(v), 1e-300))
                         for o, v in zip(outs_t, vals))
        outs_t = None
        tu.autotune(False)
        if mode == "fp64":
            ref = vals
        err = float(np.sqrt(sum(np.sum((v - r) ** 2) for v, r in zip(vals, ref)) / sum(np.sum(r ** 2) for r in ref)))
        res[mode] = {"ms_grouped": ms_g, "ms_per_contraction": ms_c, "ms_per_sector": ms_s,
                     "tflops_grouped": flops / (ms_g * 1e-3) / 1e12, "flops": flops, "err_vs_fp64": err,
                     "grouped_vs_per_contraction_rel": same,
                     "ms_grouped_autotuned": ms_t, "autotuned_vs_default_rel": tuned_same,
                     "speedup_vs_per_sector": ms_s / ms_g, "speedup_vs_per_contraction": ms_c / ms_g,
                     "kernels": {k: {"ms": v["ms"] / 2, "launches": v["launches"] // 2} for k, v in prof.items()}}
    if rank == 0:
        head = res[args.mode if args.mode in res else "fp64"]
        print(json.dumps({"metric": "contract() TFLOP/s (FP64-equivalent), 1024 uneven U(1) contractions, one grouped launch",
                          "value": head["tflops_grouped"], "unit": "TFLOP/s", "n_gpus": world, "higher_is_better": True,
                          "config": {"workload": f"batched_u1_rank3_x{args.batch}", "sector_gemms": nsec},
                          "modes": res}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="split", choices=["fp64", "split", "bf16", "split_fused", "split_tiled"],
                    help="iTEBD: the tensor-core mode timed beside FP64 (split_fused / split_tiled force that form)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--clock-seconds", type=float, default=1.0,
                    help="repeat the timed region for at least this long while SM clocks are sampled (0: once)")
    ap.add_argument("--workload", default="itebd", choices=["itebd", "permute", "mera", "batched", "ipeps"])
    ap.add_argument("--chi-ctm", type=int, default=128)
    ap.add_argument("--D", type=int, default=8)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--modes", default="split,bf16")
    ap.add_argument("--autotune", action="store_true",
                    help="iTEBD workload: FP64 GEMM tile/split policies from the autotuner")
    ap.add_argument("--chi", type=int, default=24)
    ap.add_argument("--perm", default="4,5,0,1,2,3", help="permute workload: the new bond order")
    ap.add_argument("--perm-rownum", type=int, default=2, help="permute workload: incoming bonds after the permute")
    ap.add_argument("--c128", action="store_true", help="permute workload: complex (cflag) elements, 16 bytes each")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, local, world = dist_env()
    if args.impl == "reference":
        reference_main(args, rank, world)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    if args.workload == "permute":
        permute_main(args, rank, local, world)
    elif args.workload == "mera":
        mera_main(args, rank, local, world)
    elif args.workload == "batched":
        batched_main(args, rank, local, world)
    elif args.workload == "ipeps":
        ipeps_main(args, rank, local, world)
    else:
        gpu_main(args, rank, local, world)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
