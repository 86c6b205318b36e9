#!/usr/bin/env python3
"""Benchmark of the block-tensor permute + sector-GEMM path on GB300.

Headline workload (one step): the dense ternary MERA ascending
superoperator at chi = 24 -- the three ascending diagrams (left, center,
right), each a Network::launch of seven tensors (a chi^6 = 1.9e8-element
operator O, isometries w, disentanglers u) through pairwise contract() calls
whose sector GEMMs are chi^8-sized.  Metric: contract() TFLOP/s counted as
the FP64-equivalent sum of 2*M*N*K over the sector GEMMs the reference
issues for these networks and ORDERs (the same count in every precision
mode).  The headline is the split-precision mode (FP64 operands cut into
BF16 digit slices multiplied on the tcgen05 tensor cores, FP32 accumulation,
FP64 recombination); the plain FP64 GPU form is timed beside it and every
result states its error against that FP64 output.

The same JSON line carries the other workloads as sections: the iTEBD step
(chi = 512 U(1) network + per-sector SVD/truncation), the chi = 24 rank-6
permute (GB/s, bit-exact), the 1024 uneven contractions (one grouped
launch), the rank-4 U(1) permute + contract, and the Z2 iPEPS CTM quadrant.

  python bench.py [--gpus N] [--steps K] [--warmup W]
  python bench.py --impl reference ...   # the reference path on the host cores
  python bench.py --workload mera|itebd|permute|batched|u1|ipeps   # one section alone

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

METRIC = ("contract() TFLOP/s (FP64-equivalent sector-GEMM flops), dense ternary MERA ascend chi=24, 3 diagrams; "
          "split-precision tcgen05 vs FP64 GPU at stated error")
ITEBD_METRIC = "contract() TFLOP/s (FP64-equivalent sector-GEMM flops), iTEBD chi=512 U(1) step"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2: written between timed steps of the small workloads


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


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def itebd_inputs():
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    return spec, els


def oracle_bonds(st, bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]


def kernels_dtype(names) -> str:
    """The arithmetic the kernels that ran compute in."""
    names = set(names)
    tc_split = any(n.endswith("_split") for n in names if n.startswith("tc_"))
    tc_bf16 = any(n.endswith("_bf16") for n in names if n.startswith("tc_"))
    tc_tf32 = any(n.endswith("_tf32") for n in names if n.startswith("tc_"))
    f64 = "gemm_fp64" in names
    if tc_split and f64:
        return "f64 (split: 7 bf16 digit slices on tcgen05, fp32 accumulation, fp64 recombination; thin sectors on the fp64 kernel)"
    if tc_split:
        return "f64 (split: 7 bf16 digit slices on tcgen05, fp32 accumulation, fp64 recombination)"
    if tc_bf16:
        return "bf16 (tcgen05, fp32 accumulation)"
    if tc_tf32:
        return "tf32 (tcgen05 kind::tf32, fp32 accumulation)"
    return "f64"


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


# ----------------------------------------------------------------- timing helpers
def _time_steps(torch, stream, flush, steps, fn):
    """CUDA-event time per step on the library stream; with a flush buffer,
    L2 is overwritten between timed steps (outside the events)."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
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


def roofline_of(torch, prof, steps_done, peaks, sustained):
    """Roofline of the dominant kernel (most device time) of a profiled run.
    Tensor-core GEMMs count 34 BF16 digit products per FP64-equivalent flop
    (split) and are set against the measured cuBLAS BF16 rate (sustained for
    a kernel timed inside a long step, else burst); FP64 GEMMs against a
    cuBLAS DGEMM measured in this run; permute and slicing against the
    measured HBM copy rate."""
    dname, d = max(prof.items(), key=lambda kv: kv[1]["ms"])
    avg_ms = d["ms"] / max(d["launches"], 1)
    if dname in ("permute", "tc_slice", "tc_maxima"):
        ach = d["bytes"] / d["launches"] / (avg_ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback",
                "algorithmic_bytes_per_launch": d["bytes"] / d["launches"]}
    elif dname == "gemm_fp64":
        ach = d["flops"] / d["launches"] / (avg_ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": ach, "peak": measured_fp64_peak(torch), "unit": "TFLOP/s",
                "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5",
                "peak_nominal": 1.25, "algorithmic_flops_per_launch": d["flops"] / d["launches"]}
    else:
        pairs = 34 if "split" in dname else 1
        ach = pairs * d["flops"] / d["launches"] / (avg_ms * 1e-3) / 1e12
        key = "bf16_tflops_sustained" if sustained else "bf16_tflops"
        peak = peaks.get(key, 1700.0 if sustained else 1900.0)
        roof = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "peak_source": (f"measured (MEASURED_PEAKS.json {key})" if key in peaks else "fallback"),
                "work": ("BF16 tensor flops: 34 digit products per FP64-equivalent flop" if pairs > 1 else "BF16 flops"),
                "fp64_equivalent_flops_per_launch": d["flops"] / d["launches"]}
        if "bf16_tflops" in peaks:
            roof["frac_of_burst"] = ach / peaks["bf16_tflops"]
    roof.update({"kernel": dname, "frac": roof["achieved"] / roof["peak"], "avg_launch_ms": avg_ms,
                 "launches_per_step": d["launches"] / steps_done, "traffic": None})
    return roof


# ----------------------------------------------------------------- MERA (headline)
def mera_inputs(chi):
    spec = wl.mera(chi=chi)
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    return spec, els


class MeraRefSampler:
    """The reference path on the host cores: the numpy restatement of
    Network::launch (per-sector BLAS dgemm, permutes as strided copies) over
    the three MERA diagrams, advanced one pairwise contract() at a time and
    cycling through the diagrams, so a bounded number of steps samples the
    same workload.  step() returns (flops, seconds) of one contraction (the
    last one of a diagram includes its final permute to TOUT, the first the
    next diagram's putTensor copies)."""

    def __init__(self, chi):
        from oracle import symtensor as st

        self.st = st
        spec, els = mera_inputs(chi)
        self.spec = spec
        self.tens = {s.name: st.UniTensor(oracle_bonds(st, s.bonds), s.labels, els[s.name]) for s in spec["tensors"]}
        self.gen = self._walk()

    def _merge(self, net, nd, acc):
        st = self.st
        l = (yield from self._merge(net, nd.left, acc)) if nd.left.t is None else net.tensors[nd.left.t]
        r = (yield from self._merge(net, nd.right, acc)) if nd.right.t is None else net.tensors[nd.right.t]
        out = st.contract(l, r, True, gemm=lambda a, b: (acc.append(2.0 * a.shape[0] * a.shape[1] * b.shape[1]), a @ b)[1])
        yield None
        return out

    def _walk(self):
        st = self.st
        while True:
            for d, text in self.spec["nets"].items():
                net = st.Network(text=text)
                for s in self.spec["tensors"]:
                    net.put_tensor(s.name, self.tens[s.name])
                acc = self.acc
                root = net.construct()
                out = yield from self._merge(net, root, acc)
                net.root = root
                tout = net.label_arr[-1]
                out.permute(tout, net.rnums[-1])

    def step(self):
        self.acc = getattr(self, "acc", [])
        self.acc.clear()
        t0 = time.perf_counter()
        next(self.gen)
        dt = time.perf_counter() - t0
        return sum(self.acc), dt


def mera_cpu_sample(chi, seconds, min_steps=2, threads=None):
    """Bounded sample of the MERA workload on the host cores (numpy port)."""
    threads = threads or os.cpu_count()
    s = MeraRefSampler(chi)
    fl = tm = 0.0
    n = 0
    while n < min_steps or tm < seconds:
        f, dt = s.step()
        fl += f
        tm += dt
        n += 1
    return {"value": fl / tm / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"{n} pairwise contract() calls of the chi={chi} MERA diagrams in network order "
                      f"({fl:.3g} FP64 flop, {tm:.1f} s), numpy BLAS dgemm on {threads} host thread(s)"}


def mera_cpu_sample_one_thread(chi, seconds):
    """The same sample with the BLAS pinned to one thread (a child process,
    since the thread count is fixed when numpy's BLAS loads)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
    code = f"import json, bench; print(json.dumps(bench.mera_cpu_sample({int(chi)}, {float(seconds)}, 1, 1)))"
    try:
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900,
                           cwd=os.path.dirname(os.path.abspath(__file__)))
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode == 0 and lines:
            return json.loads(lines[-1])
        return {"unavailable": f"child exited {r.returncode}: {r.stderr.strip()[-200:]}"}
    except Exception as e:  # a reported baseline only
        return {"unavailable": f"{type(e).__name__}: {str(e)[:200]}"}


def mera_section(args, torch, tu, stream, local, world, peaks):
    """The three MERA ascending diagrams through Network::launch in FP64 and
    split precision: device time per step (inputs resident), per-kernel times
    from the same timed steps, error of split against FP64, Hermiticity of
    the ascended operators, and an end-to-end step through the C ABI (pinned
    host inputs copied in, results read back)."""
    chi = args.chi
    spec, els = mera_inputs(chi)
    names = [s.name for s in spec["tensors"]]
    dev = {s.name: tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]}
    nets = {d: tu.Network(t) for d, t in spec["nets"].items()}
    outs = {}

    def step(mode):
        for d, net in nets.items():
            for n in names:
                net.put_tensor(n, dev[n])
            outs[d] = net.launch(mode)

    res, ref = {}, None
    fast = [m for m in args.fast_modes.split(",") if m and m not in (args.mode, "none")]
    for mode in ["fp64", args.mode] + fast:
        # FP64 takes ~2 s per step at chi=24: it is timed over fewer steps;
        # the fast (BF16 / TF32) modes are reported beside the headline
        nsteps = max(1, min(args.steps, 2)) if mode == "fp64" else (args.steps if mode == args.mode else
                                                                     max(1, min(args.steps, 5)))
        nwarm = 1 if mode == "fp64" else (args.warmup if mode == args.mode else 2)
        for _ in range(nwarm):
            step(mode)
        tu.sync()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = tu.launch_count()
        tu.prof_enable(True)
        ms, reps, clocks = _timed_with_clocks(torch, stream, None, nsteps, lambda: step(mode), local,
                                              min_seconds=args.clock_seconds if mode == args.mode else 0)
        prof = tu.prof_read()
        tu.prof_enable(False)
        done = nsteps * reps
        launches = (tu.launch_count() - l0) / done
        flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k) / done
        vals = {d: t.get_elem() for d, t in outs.items()}
        if mode == "fp64":
            ref = vals
        err = float(np.sqrt(sum(np.sum((vals[d] - ref[d]) ** 2) for d in vals) / sum(np.sum(ref[d] ** 2) for d in vals)))
        err_max = max(float(np.linalg.norm(vals[d] - ref[d]) / np.linalg.norm(ref[d])) for d in vals)
        herm = 0.0
        for d, v in vals.items():
            m = v.reshape(chi * chi, chi * chi)
            herm = max(herm, float(np.linalg.norm(m - m.T) / np.linalg.norm(m)))
        res[mode] = {"ms_per_step": ms, "tflops": world * flops / (ms * 1e-3) / 1e12, "flops_per_step": flops,
                     "err_vs_fp64": err, "err_vs_fp64_max_diagram": err_max, "hermiticity": herm,
                     "dtype": kernels_dtype(prof), "launches_per_step": launches, "timed_steps": done,
                     "warmup_steps": nwarm, "clocks": clocks, "prof": prof,
                     "kernels": {k: {"ms_per_step": v["ms"] / done, "launches_per_step": v["launches"] / done,
                                     "share": v["ms"] / done / ms} for k, v in prof.items()}}
        vals = None
    if world > 1:
        for m in res:
            (res[m]["ms_per_step"],) = max_over_ranks(torch, [res[m]["ms_per_step"]], "cuda")
            res[m]["tflops"] = world * res[m]["flops_per_step"] / (res[m]["ms_per_step"] * 1e-3) / 1e12

    # end to end through the C ABI: every step copies the inputs from pinned
    # host memory into the tensors (setElem), launches the three networks and
    # reads the three ascended operators back into pinned host buffers
    mode = args.mode
    pinned = {n: torch.from_numpy(els[n]).pin_memory() for n in names}
    out_host = {d: torch.empty(chi ** 4, dtype=torch.float64).pin_memory() for d in nets}
    h2d = sum(8 * els[n].size for n in names)
    d2h = sum(8 * chi ** 4 for _ in nets)

    def e2e_step():
        for n in names:
            dev[n].set_elem_host_ptr_async(pinned[n].data_ptr(), els[n].size)
        step(mode)
        for d, t in outs.items():
            t.get_elem_host_ptr(out_host[d].data_ptr(), chi ** 4)

    e2e_step()
    torch.cuda.synchronize()
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        e2e_step()
        e2e.append((time.perf_counter() - w0) * 1e3)
    e2e_ms = statistics.median(e2e)
    e2e_ok = bool(all(np.array_equal(out_host[d].numpy(), outs[d].get_elem()) for d in nets))
    if world > 1:
        (e2e_ms,) = max_over_ranks(torch, [e2e_ms], "cuda")
    R = res[mode]
    roof = roofline_of(torch, R["prof"], R["timed_steps"], peaks, sustained=True)
    if roof["kernel"] == "tc_gemm_split" and chi == 24:
        roof.update(TC_GEMM_TRAFFIC_NOTE)
    del pinned, out_host
    outs.clear()
    dev.clear()
    nets.clear()
    return res, {"value": world * R["flops_per_step"] / (e2e_ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                 "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                 "matches_device": e2e_ok}, roof


# dram__bytes_read.sum + dram__bytes_write.sum of one chi^8 tc_gemm_split
# launch of the chi=16 diagrams (ncu, 236.9 + 92.4 MB), scaled by the operand
# elements (24/16)^6 to the chi=24 launch of the same contraction
TC_GEMM_TRAFFIC_NOTE = {
    "traffic": 3.75e9, "traffic_unit": "bytes per chi^8 launch (the big-operand contractions)",
    "traffic_source": "ncu on the chi=16 diagrams (329.3 MB for one chi^8 launch: the digit images read once, "
                      "the output partly still in L2), scaled by (24/16)^6; algorithmic bytes of that launch "
                      "at chi=24: 4.2 GB (digit images 14 B + FP64 output 8 B per element)"}


# ----------------------------------------------------------------- iTEBD
def _itebd_device(tu, spec, els, diag=True):
    """The network's tensors on the device; the Lambdas are built by putBlock
    with diagonal matrices (diag=True), as the reference keeps them, so their
    contractions run as row/column scales -- or as dense block-diagonal
    tensors through sector GEMMs (diag=False)."""
    names = [s.name for s in spec["tensors"]]
    dev = {}
    for s in spec["tensors"]:
        if diag and s.kind == "diag":
            t = tu.UniTensor(s.bonds, s.labels)
            for q, r, c, d in wl.diag_blocks(s.bonds, els[s.name]):
                t.put_block(q, (r, c, d), diag=True)
            dev[s.name] = t
        else:
            dev[s.name] = tu.UniTensor(s.bonds, s.labels, els[s.name])
    net = tu.Network(spec["net"])
    for n in names:
        net.put_tensor(n, dev[n])
    return names, dev, net


def run_itebd_reference(steps: int, warmup: int):
    """The iTEBD network on the host cores: the numpy restatement of
    Network::launch with per-sector BLAS dgemm and the diagonal Lambdas as
    row/column scales."""
    from oracle import symtensor as st

    spec, els = itebd_inputs()
    tens = {}
    for s in spec["tensors"]:
        t = st.UniTensor(oracle_bonds(st, s.bonds), s.labels, els[s.name])
        if s.kind == "diag":  # Lambda as the reference keeps it: diagonal blocks (RDotR's diagonal paths)
            t = st.UniTensor(oracle_bonds(st, s.bonds), s.labels)
            for q, r, c, d in wl.diag_blocks(s.bonds, els[s.name]):
                t.put_block(st.Qnum(*q), d, diag=True, fresh=True)
        tens[s.name] = t
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


def itebd_section(args, torch, tu, stream, flush, local, rank, world):
    """The iTEBD step: La-A-Lb-B-Lc-gate contracted to theta through
    Network::launch captured as a CUDA graph (FP64 and the tensor-core mode
    the route tuner picks), an end-to-end replay with pinned host I/O, then
    the SVD/truncation and Block::eigh of that theta."""
    spec, els = itebd_inputs()
    modes = ["fp64"] + ([args.itebd_mode] if args.itebd_mode != "fp64" else [])
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
        kern = {k_: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps}
                for k_, v in prof.items()}
        res[mode] = {"ms_graph": ms_graph, "ms_eager": ms_eager, "flops": flops, "err_vs_fp64": err,
                     "dtype": kernels_dtype(prof), "graph_matches_eager": graph_ok, "launches": int(launches),
                     "clocks": clocks, "timed_repeats": reps, "e2e_ms": statistics.median(e2e),
                     "e2e_matches_device": e2e_ok, "kernels_eager": kern,
                     "h2d": sum(8 * els[n].size for n in names), "d2h": 8 * vals.size}
        if mode != "fp64" and "gemm_fp64" in prof and not any(k_.startswith("tc_") for k_ in prof):
            res[mode]["route"] = ("the route tuner kept every contraction of this network on the FP64 kernel "
                                  "(faster than the tensor-core forms at these sector sizes): same kernels as fp64")
    # the same network with the Lambdas as dense block-diagonal tensors (every
    # contraction a sector GEMM): what the diagonal scales replace
    names, dev, net = _itebd_device(tu, spec, els, diag=False)
    th = net.launch("fp64")
    dense_same = bool(np.array_equal(th.get_elem(), ref64))
    net.capture("fp64")
    for _ in range(args.warmup):
        net.replay()
    tu.sync()
    dense_ms = _time_steps(torch, stream, flush, args.steps, net.replay)
    tu.prof_enable(True)
    net.launch("fp64")
    dprof = tu.prof_read()
    tu.prof_enable(False)
    dense_lambda = {"ms_graph_fp64": dense_ms, "matches_diagonal_bitwise": dense_same,
                    "gemm_flops": sum(v["flops"] for k_, v in dprof.items() if "gemm" in k_),
                    "kernels": {k_: v["launches"] for k_, v in dprof.items()}}
    net = dev = th = None
    if world > 1:
        for m in res:
            res[m]["ms_graph"], res[m]["e2e_ms"] = max_over_ranks(torch, [res[m]["ms_graph"], res[m]["e2e_ms"]], "cuda")
    for m, r in res.items():
        r["tflops_graph"] = world * r["flops"] / (r["ms_graph"] * 1e-3) / 1e12
        r["tflops_e2e"] = world * r["flops"] / (r["e2e_ms"] * 1e-3) / 1e12
    svd = itebd_svd_section(args, torch, tu, stream, flush, spec, els, ref64, rank, world)
    eigh = itebd_eigh_section(args, torch, tu, stream, flush, spec, els, ref64, rank, world)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        f_, dt1 = run_itebd_reference(1, 1)
        n = max(3, int(args.itebd_cpu_seconds / max(dt1, 1e-4)))
        f_, dtc = run_itebd_reference(n, 0)
        cpu = {"value": f_ / dtc / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "ms_per_step": dtc * 1e3,
               "sample": f"{n} full iTEBD network steps, numpy BLAS on {os.cpu_count()} host threads"}
    head = modes[-1]
    best = min(res, key=lambda m: res[m]["ms_graph"])
    return {"workload": "itebd_u1_chi512_d2", "metric": ITEBD_METRIC, "chi": 512, "sectors": 17,
            "execution": "Network::launch captured as one CUDA graph, replayed per step",
            "lambdas": "diagonal tensors (putBlock of diagonal matrices): their contractions are row/column scales, "
                       "flops count only the A.B and gate sector GEMMs",
            "l2": "flushed between timed steps (512 MB write)", "modes": res, "dense_lambda": dense_lambda,
            "speedup_split_vs_fp64_gpu": res["fp64"]["ms_graph"] / res[head]["ms_graph"],
            "fastest_mode": best, "cpu_baseline": cpu, "svd_truncate": svd, "eigh": eigh,
            "step_ms": {"contract_graph": res[best]["ms_graph"], "svd_truncate": svd["ms_gpu"],
                        "total": res[best]["ms_graph"] + svd["ms_gpu"],
                        "cpu_port_total": (svd["ms_cpu_port"] + cpu["ms_per_step"])
                        if svd["ms_cpu_port"] is not None and cpu else None}}


def svd_section(args, torch, tu, stream, flush, rank, world):
    """The SVD / truncation of the iTEBD update alone: theta from the FP64
    network, then the batched SVD with the global truncation and Block::eigh
    of the same blocks (the eigendecomposition runs on the same solver)."""
    spec, els = itebd_inputs()
    names, dev, net = _itebd_device(tu, spec, els)
    theta64 = net.launch("fp64").get_elem()
    return {"workload": "itebd_theta_svd_truncate", "blocks": "19 sectors up to 130x130, chi 1024 -> 512",
            "svd_truncate": itebd_svd_section(args, torch, tu, stream, flush, spec, els, theta64, rank, world),
            "eigh": itebd_eigh_section(args, torch, tu, stream, flush, spec, els, theta64, rank, world)}


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
        n = 0 if args.no_cpu else max(1, min(50, int(0.2 * args.itebd_cpu_seconds / max(dt1, 1e-3))))
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
    tho = st.UniTensor(oracle_bonds(st, th.bonds()), th.labels(), theta64)
    out = {"ms_gpu": statistics.median(wall), "norm": norm,
           "kernels_ms": {k_: v["ms"] for k_, v in prof.items()}}
    cpu_ms = None
    if rank == 0 and world == 1:
        t0 = time.perf_counter()
        Uo, So, VTo, norm_o = st.svd_truncate(tho, chi)
        dt1 = time.perf_counter() - t0
        n = 0 if args.no_cpu else max(1, min(50, int(0.3 * args.itebd_cpu_seconds / max(dt1, 1e-3))))
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
    try:
        out["cusolver_baseline"] = cusolver_svd_baseline(torch, th, theta64, args.steps)
    except Exception as e:  # a library baseline only: its failure must not stop the bench
        out["cusolver_baseline"] = {"unavailable": f"{type(e).__name__}: {str(e)[:200]}"}
    return out


def cusolver_svd_baseline(torch, th, theta64, steps):
    """The library baseline for the per-sector SVD: cuSOLVER through
    torch.linalg.svd on the same theta blocks, one call per block and one
    call on the blocks zero-padded into a batch (the padding adds only zero
    singular values); wall time per set of blocks, median over steps, and the
    largest singular-value difference to LAPACK relative to the block's
    largest value."""
    blocks = [(r, c, off) for _, r, c, off in th.sector_map().blocks()]
    mats = [torch.from_numpy(theta64[off:off + r * c].reshape(r, c).copy()).cuda() for r, c, off in blocks]
    mx = max(max(r, c) for r, c, _ in blocks)
    padded = torch.zeros(len(mats), mx, mx, dtype=torch.float64, device="cuda")
    for i, m in enumerate(mats):
        padded[i, : m.shape[0], : m.shape[1]] = m
    torch.cuda.synchronize()

    def loop():
        return [torch.linalg.svd(m, full_matrices=False) for m in mats]

    def batch():
        return torch.linalg.svd(padded, full_matrices=False)

    out = {"library": "cuSOLVER via torch.linalg.svd (torch picks the routine)", "blocks": len(mats)}
    for name, fn in (("per_block", loop), ("padded_batch", batch)):
        fn()
        torch.cuda.synchronize()
        wall = []
        for _ in range(steps):
            t0 = time.perf_counter()
            r = fn()
            torch.cuda.synchronize()
            wall.append((time.perf_counter() - t0) * 1e3)
        out[f"ms_{name}"] = statistics.median(wall)
    S = [x[1].cpu().numpy() for x in loop()]
    err = 0.0
    for (r, c, off), sv in zip(blocks, S):
        ref = np.linalg.svd(theta64[off:off + r * c].reshape(r, c), compute_uv=False)
        err = max(err, float(np.max(np.abs(sv - ref)) / max(ref[0], 1e-300)))
    out["sv_max_err_rel"] = err
    return out


# ----------------------------------------------------------------- permute
def permute_section(args, torch, tu, stream, local, peaks, chi=None, perm=None, rn=None, c128=False):
    """Large dense permute (HBM-bound): a chi^6 tensor, bonds (3 in | 3 out)
    permuted to (4 5 0 | 1 2 3) -- the operand permute a MERA ascending
    contraction issues.  Bit-exact check against torch's permute."""
    chi = chi or args.chi
    perm = perm or [int(v) for v in args.perm.split(",")]
    rn = args.perm_rownum if rn is None else rn
    bonds = [wl.dense_bond(1, chi)] * 3 + [wl.dense_bond(-1, chi)] * 3
    n = chi ** 6
    esz = 16 if c128 else 8
    x = torch.randn(n, dtype=torch.complex128 if c128 else torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(5))
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
        clk.wait_samples(1, 10.0)
        reps = 0
        t0 = time.time()
        times = []
        while reps < 200:
            for s_, e_ in ev:
                s_.record(stream)
                run(src_map, dst_map, perm, x.data_ptr(), y.data_ptr())
                e_.record(stream)
            torch.cuda.synchronize()
            times += [s_.elapsed_time(e_) for s_, e_ in ev]
            reps += 1
            if time.time() - t0 >= args.clock_seconds and len(clk.lines) >= 4:
                break
    ms = statistics.median(times)
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
    peak = peaks.get("hbm_gbs", 6800.0)
    del x, y, y_keep
    return {"workload": f"dense_rank6_chi{chi}_permute" + ("_c128" if c128 else ""), "metric": f"permute GB/s ({2 * esz} B per element)",
            "gb_s": gbs, "ms_per_step": ms, "bit_exact": exact, "copy_gb_s": copy_gbs, "elements": n, "perm": perm,
            "row_bonds": rn, "dtype": "c128" if c128 else "f64", "l2": "inputs larger than L2",
            "timed_launches": len(times),
            "roofline": {"kernel": "permute", "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                         "frac": gbs / peak, "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback"},
            "clocks": clk.summary()}


# ----------------------------------------------------------------- rank-4 U(1) (workload 1)
def u1_section(args, torch, tu, stream, flush, rank, world):
    """The 64-dim U(1) rank-4 workload: permute A[a,p,q,b] to (a,p,b,q) and
    contract over (b,q) with B; bit-exact permute and <= 1e-13 contraction
    against the oracle, device time per step (a copy of A, the permute, the
    contraction), permute GB/s and contraction GFLOP/s from the same steps."""
    from oracle import symtensor as st

    spec = wl.u1_rank4()
    rng = np.random.default_rng(spec["seed"])
    A, B = spec["tensors"]
    ea, eb = wl.gen_elems(A, rng), wl.gen_elems(B, rng)
    ta = tu.UniTensor(A.bonds, A.labels, ea)
    tb = tu.UniTensor(B.bonds, B.labels, eb)
    keep = {}

    def step():
        t = ta.copy()
        t.permute([0, 1, 3, 2], 2)
        keep["p"] = t
        keep["c"] = tu.contract(t, tb, fast=True, mode="fp64")

    for _ in range(args.warmup):
        step()
    tu.sync()
    nsteps = max(args.steps, 100)
    ms = _time_steps(torch, stream, flush, nsteps, step)
    # per-kernel times from a second pass with events around every launch
    # (the events' own cost stays out of ms_per_step)
    tu.prof_enable(True)
    _time_steps(torch, stream, flush, nsteps, step)
    prof = tu.prof_read()
    tu.prof_enable(False)
    oa = st.UniTensor(oracle_bonds(st, A.bonds), A.labels, ea)
    obt = st.UniTensor(oracle_bonds(st, B.bonds), B.labels, eb)
    t0 = time.perf_counter()
    ncpu = 0
    while True:
        o = oa.copy()
        o.permute([0, 1, 3, 2], 2)
        oc = st.contract(o, obt, True)
        ncpu += 1
        if time.perf_counter() - t0 > 1.0 and ncpu >= 10:
            break
    cpu_ms = (time.perf_counter() - t0) / ncpu * 1e3
    got_p, got_c = keep["p"].get_elem(), keep["c"].get_elem()
    flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k) / nsteps
    pb = prof.get("permute", {})
    return {"workload": "u1_rank4_chi64", "ms_per_step": ms, "steps": nsteps,
            "permute_bit_exact": bool(np.array_equal(got_p, o.elem)),
            "contract_err_rel": float(np.linalg.norm(got_c - oc.elem) / np.linalg.norm(oc.elem)),
            "permute_bytes": 16.0 * ea.size, "contract_flops": flops,
            "permute_gb_s": pb["bytes"] / (pb["ms"] * 1e-3) / 1e9 if pb else None,
            "contract_gflops": flops / (ms * 1e-3) / 1e9,
            "kernels": {k: {"ms_per_step": v["ms"] / nsteps, "launches_per_step": v["launches"] / nsteps}
                        for k, v in prof.items()},
            "cpu_port_ms_per_step": cpu_ms, "cpu_port_sample": f"{ncpu} steps (numpy restatement, {os.cpu_count()} threads)",
            "execution": "eager: UniTensor copy + permute + contract per step, L2 flushed between steps"}


# ----------------------------------------------------------------- iPEPS
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


def ipeps_section(args, torch, tu, stream):
    """Z2-symmetric iPEPS double-layer CTM quadrant, chi = 128, D = 8:
    C.T1.T2.A2 through Network::launch (ORDER (((C T1) T2) A2)) in FP64, split
    and fast BF16; time per launch (median of 5 after a warm-up), FP64-equivalent
    TFLOP/s and error vs FP64."""
    spec = wl.ipeps_ctm(chi=args.chi_ctm, D=args.D)
    dev, _ = ipeps_device(tu, spec)
    net = tu.Network(spec["net"])
    for n, t in dev.items():
        net.put_tensor(n, t)
    res, ref = {}, None
    for mode in ["fp64"] + [m for m in args.modes.split(",") if m != "fp64"]:
        net.launch(mode)
        tu.sync()
        reps = 2 if mode == "fp64" else 5
        tu.prof_enable(True)
        ms = _time_steps(torch, stream, None, reps, lambda: net.launch(mode))
        prof = tu.prof_read()
        tu.prof_enable(False)
        q = net.launch(mode)
        v = q.get_elem()
        if mode == "fp64":
            ref = v
        flops = sum(x["flops"] for k, x in prof.items() if "gemm" in k) / reps
        res[mode] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "flops": flops, "dtype": kernels_dtype(prof),
                     "err_vs_fp64": float(np.linalg.norm(v - ref) / np.linalg.norm(ref)),
                     "kernels": {k: {"ms": x["ms"] / reps, "launches": x["launches"] / reps} for k, x in prof.items()}}
    return {"workload": f"ipeps_ctm_z2_chi{args.chi_ctm}_D{args.D}", "elements_out": int(ref.size), "modes": res,
            "speedup_vs_fp64": {m: res["fp64"]["ms"] / r["ms"] for m, r in res.items()}}


# ----------------------------------------------------------------- batched
def batched_section(args, torch, tu, stream, local, flush):
    """1024 independent uneven U(1) contractions T1[x|y,z].T2[y,z|w]
    (8 382 sector GEMMs of sizes 1..256).  The headline is a Batch (operands,
    outputs and the grouped work list kept on the device) captured as one
    CUDA graph and replayed, timed with clocks over >= 5 repeats; beside it
    the same Batch launched eagerly, the stateless tn_contract_batch call
    (host planning per call), a loop of contract() calls, and the
    reference's per-sector pattern -- one GEMM launch per sector, issued
    from C++ (tn_contract_sectors_loop) -- in FP64 and split precision."""
    spec = wl.batched(n=args.batch)
    rng = np.random.default_rng(spec["seed"])
    A, B = [], []
    for t1, t2 in spec["pairs"]:
        A.append(tu.UniTensor(t1.bonds, t1.labels, wl.gen_elems(t1, rng)))
        B.append(tu.UniTensor(t2.bonds, t2.labels, wl.gen_elems(t2, rng)))

    def timed(fn, reps=1):
        fn()
        tu.sync()
        ts = []
        r = None
        for k in range(reps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_.record(stream)
            r = fn()
            e_.record(stream)
            torch.cuda.synchronize()
            ts.append(s_.elapsed_time(e_))
        return statistics.median(ts), r

    res = {}
    ref = None
    for mode in ["fp64", args.mode] if args.mode != "fp64" else ["fp64"]:
        bt = tu.Batch(A, B)
        secs = bt.sectors()
        bt.launch(mode)  # plans the grouped work list
        tu.sync()
        tu.prof_enable(True)
        ms_eager, _ = timed(lambda: bt.launch(mode), reps=5)
        prof = tu.prof_read()
        tu.prof_enable(False)
        flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k) / 6  # warm-up + 5 timed launches
        vals = [bt.output(i).get_elem() for i in range(len(A))]
        bt.capture(mode)
        l0 = tu.launch_count()
        ms_graph, reps, clocks = _timed_with_clocks(torch, stream, flush, 5, bt.replay, local,
                                                    min_seconds=args.clock_seconds)
        launches = (tu.launch_count() - l0) / (5 * reps)
        graph_same = all(np.array_equal(bt.output(i).get_elem(), v) for i, v in enumerate(vals))
        ms_call, outs = timed(lambda: tu.contract_batch(A, B, mode), reps=3)
        call_same = max(float(np.linalg.norm(o.get_elem() - v) / max(np.linalg.norm(v), 1e-300))
                        for o, v in zip(outs, vals))
        outs = None
        ms_c, outs_c = timed(lambda: [tu.contract(a, b, mode=mode) for a, b in zip(A, B)])
        same = max(float(np.linalg.norm(o.get_elem() - v) / max(np.linalg.norm(v), 1e-300)) for o, v in zip(outs_c, vals))
        outs_c = None
        ms_s, _ = timed(lambda: tu.contract_sectors_loop(mode, secs, 0, 0, 0), reps=3)
        loop_same = max(float(np.linalg.norm(bt.output(i).get_elem() - v) / max(np.linalg.norm(v), 1e-300))
                        for i, v in enumerate(vals))
        # the FP64 tile policy from the autotuner (timed per sector histogram
        # at the first launch; the default is kept unless a candidate is 3 % faster)
        tu.autotune(True)
        bt2 = tu.Batch(A, B)
        bt2.launch(mode)
        bt2.capture(mode)
        ms_tuned = _time_steps(torch, stream, flush, 5, bt2.replay)
        tuned_same = max(float(np.linalg.norm(bt2.output(i).get_elem() - v) / max(np.linalg.norm(v), 1e-300))
                         for i, v in enumerate(vals))
        tu.autotune(False)
        bt = bt2 = None
        if mode == "fp64":
            ref = vals
        err = float(np.sqrt(sum(np.sum((v - r) ** 2) for v, r in zip(vals, ref)) / sum(np.sum(r ** 2) for r in ref)))
        res[mode] = {"ms_graph": ms_graph, "ms_batch_launch": ms_eager, "ms_contract_batch_call": ms_call,
                     "ms_per_contraction": ms_c, "ms_per_sector_loop_cpp": ms_s, "ms_graph_autotuned": ms_tuned,
                     "tflops_graph": flops / (ms_graph * 1e-3) / 1e12, "flops": flops, "err_vs_fp64": err,
                     "dtype": kernels_dtype(prof), "graph_matches_eager": graph_same,
                     "contract_batch_vs_batch_rel": call_same, "per_contraction_vs_batch_rel": same,
                     "per_sector_loop_vs_batch_rel": loop_same, "autotuned_vs_default_rel": tuned_same,
                     "speedup_vs_per_sector_loop": ms_s / ms_graph, "speedup_vs_per_contraction": ms_c / ms_graph,
                     "graph_launches": launches, "timed_repeats": 5 * reps, "clocks": clocks,
                     "kernels": {k: {"ms": v["ms"] / 6, "launches": v["launches"] / 6} for k, v in prof.items()}}
    return {"workload": f"batched_u1_rank3_x{args.batch}", "sector_gemms": len(secs),
            "execution": "uni10::Batch captured as one CUDA graph (operand permutes + one grouped sector-GEMM "
                         "launch), replayed per step; L2 flushed between timed steps", "modes": res}


# ----------------------------------------------------------------- reference arm
def reference_main(args, rank, world):
    """The reference path on the host cores for the headline workload: the
    numpy restatement of the MERA networks (the compiled reference does not
    build on the GPU host's architecture), each step one pairwise contract()
    of the three diagrams in network order, cycling (a bounded sample of the
    same workload)."""
    if rank != 0:
        return
    s = MeraRefSampler(args.chi)
    for _ in range(args.warmup):
        s.step()
    fl = tm = 0.0
    for _ in range(args.steps):
        f, dt = s.step()
        fl += f
        tm += dt
    v = fl / tm / 1e12
    cores = os.cpu_count()
    sample = (f"{args.steps} pairwise contract() calls of the chi={args.chi} MERA diagrams in network order after "
              f"{args.warmup} warm-up calls ({fl:.3g} FP64 flop), numpy BLAS dgemm on {cores} host threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tm / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"mera_ternary_chi{args.chi}", "chi": args.chi, "mode": "fp64",
                   "step": "one pairwise contract() (sample of the 3-diagram ascend)"},
        "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ----------------------------------------------------------------- GPU arm
def gpu_main(args, rank, local, world):
    import torch

    torch.cuda.set_device(local)
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.Stream()
    tu.set_stream(stream.cuda_stream)
    peaks = load_peaks()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    wanted = args.workload

    def emit(obj):
        if rank == 0:
            print(json.dumps(obj), flush=True)

    if wanted == "itebd":
        emit(itebd_section(args, torch, tu, stream, flush, local, rank, world))
        return
    if wanted == "permute":
        emit(permute_section(args, torch, tu, stream, local, peaks, c128=args.c128))
        return
    if wanted == "batched":
        emit(batched_section(args, torch, tu, stream, local, flush))
        return
    if wanted == "u1":
        emit(u1_section(args, torch, tu, stream, flush, rank, world))
        return
    if wanted == "ipeps":
        emit(ipeps_section(args, torch, tu, stream))
        return
    if wanted == "svd":
        emit(svd_section(args, torch, tu, stream, flush, rank, world))
        return

    # headline: MERA chi=24 split vs FP64, then the other workloads as sections
    modes, e2e, roof = mera_section(args, torch, tu, stream, local, world, peaks)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = mera_cpu_sample(args.chi, args.cpu_seconds)
        if args.cpu1_seconds > 0:
            cpu["one_thread"] = mera_cpu_sample_one_thread(args.chi, args.cpu1_seconds)
    R = modes[args.mode]
    sections = {}
    if wanted == "all":
        sections["itebd"] = itebd_section(args, torch, tu, stream, flush, local, rank, world)
        sections["permute"] = permute_section(args, torch, tu, stream, local, peaks, chi=24,
                                              perm=[4, 5, 0, 1, 2, 3], rn=2)
        sections["batched"] = batched_section(args, torch, tu, stream, local, flush)
        sections["u1_rank4"] = u1_section(args, torch, tu, stream, flush, rank, world)
        sections["ipeps"] = ipeps_section(args, torch, tu, stream)
    for m in modes.values():
        m.pop("prof", None)
    emit({
        "metric": METRIC, "value": R["tflops"], "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": R["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": R["dtype"], "data": "synthetic (seeded)",
        "config": {"workload": f"mera_ternary_chi{args.chi}", "chi": args.chi, "mode": args.mode,
                   "diagrams": ["left", "center", "right"], "flops_per_step": R["flops_per_step"],
                   "execution": "per step: putTensor x7 and Network::launch for each of the 3 diagrams (eager)",
                   "l2": "inputs larger than L2 (1.53 GB operator); no flush",
                   "fp64_arm": f"{modes['fp64']['timed_steps']} timed steps after {modes['fp64']['warmup_steps']} warm-up",
                   "parallelism": f"replicas x{world}"},
        "error_vs_fp64": R["err_vs_fp64"], "hermiticity": R["hermiticity"],
        "speedup_vs_fp64_gpu": modes["fp64"]["ms_per_step"] / R["ms_per_step"],
        "modes": modes,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": R["clocks"],
        "gpu_launches": int(round(R["launches_per_step"] * args.steps)),
        "gpu_launches_per_step": R["launches_per_step"],
        "sections": sections,
    })


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="all", choices=["all", "mera", "itebd", "permute", "batched", "ipeps", "u1", "svd"],
                    help="all: the MERA headline line with every other workload as a section; mera: the headline "
                         "alone; the others print that section alone")
    ap.add_argument("--mode", default="split", choices=["split", "bf16", "split_tiled"],
                    help="MERA and batched: the tensor-core mode timed beside FP64")
    ap.add_argument("--itebd-mode", default="split", choices=["fp64", "split", "bf16", "split_fused", "split_tiled"],
                    help="iTEBD: the tensor-core mode timed beside FP64 (split_fused / split_tiled force that form)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="MERA CPU baseline sample length")
    ap.add_argument("--itebd-cpu-seconds", type=float, default=8.0)
    ap.add_argument("--cpu1-seconds", type=float, default=8.0,
                    help="MERA CPU baseline with the BLAS on one thread (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--clock-seconds", type=float, default=1.0,
                    help="repeat the timed region for at least this long while SM clocks are sampled (0: once)")
    ap.add_argument("--chi", type=int, default=24, help="MERA / permute bond dimension")
    ap.add_argument("--chi-ctm", type=int, default=128)
    ap.add_argument("--D", type=int, default=8)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--modes", default="split,bf16,tf32", help="iPEPS: modes timed beside FP64")
    ap.add_argument("--fast-modes", default="bf16,tf32", help="MERA: fast modes reported beside the headline")
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
    gpu_main(args, rank, local, world)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
