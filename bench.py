#!/usr/bin/env python3
"""Benchmark of the per-timestep lattice Boltzmann update (MLUPS, %HBM).

Default workload: D3Q27 flow past a sphere on a 512x256x256 lattice
(513x257x257 = 33.9M nodes, sphere diameter 48 at (128,128,128), Re 200,
FP64 with the reference's rounding), the size the HBM-fraction target is
quoted on; sphere_d3q27_256x128x128 is the FP64 drop-in parity size. One bench step is one
iteration of the reference's time loop (main.f90:48-63): Monitor every
`interv` iterations, Collision, BoundaryCondition, Propagation,
PostProcessing. Synthetic input: the reference's own geometry generator and
initial state (InitUP with seeded perturbation draws).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--precision fp64|fp64fast|fix64|fp32|bf16|fp16]
                    [--lp-kernel staged|register] [--no-cpu-baseline] [--no-variants]

--precision selects the population storage: fp64 (default) is the drop-in
with the reference's rounding; fp64fast and fix64 (64-bit fixed point on the
integer pipes) agree with it within 1e-12; fp32/bf16/fp16 store the
populations narrow and collide in FP32. The FP64 line also carries the
fix64 and fp16 kinds measured on the same state (`variants`) unless
--no-variants.

--impl reference times the reference algorithm's CPU path (the C restatement
under oracle/, OpenMP over all host cores) on the same workload. With
--gpus N > 1 (torchrun) every rank advances its own independent replica
("replicas only": the path does not shard on one GPU per case).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "imexlb-1.0_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "MLUPS & %HBM peak"

# name -> dimension, lattice size, and the input.in values that produce it
WORKLOADS = {
    "sphere_d3q27_256x128x128": dict(
        dim=3, nx=256, ny=128, nz=128, charlength=0.09375, xpos=0.25, re=100.0,
        ome=1.8910741301059, dt=1.0, rho0=1.0, max_t=0.16666683, inter=0.01),
    # smaller case of the same flow for ncu captures (147 MB per population
    # buffer: still larger than L2)
    "sphere_d3q27_128x64x64": dict(
        dim=3, nx=128, ny=64, nz=64, charlength=0.09375, xpos=0.25, re=100.0,
        ome=1.8910741301059, dt=1.0, rho0=1.0, max_t=0.16666683, inter=0.01),
    # the reduced-precision study size (33.9M nodes)
    "sphere_d3q27_512x256x256": dict(
        dim=3, nx=512, ny=256, nz=256, charlength=0.09375, xpos=0.25, re=200.0,
        ome=1.8910741301059, dt=1.0, rho0=1.0, max_t=0.08333338, inter=0.01),
    "cylinder_d2q9_1024x512": dict(
        dim=2, nx=1024, ny=512, nz=0, charlength=0.0390625, xpos=0.25, re=100.0,
        ome=1.7857142857142856, dt=1.0, rho0=1.0, max_t=0.2500001, inter=0.01),
}
DEFAULT_WORKLOAD = "sphere_d3q27_512x256x256"
SM_MAX_HZ = 2.07e9  # GB300's maximum SM clock

# storage kind -> (library code, bytes per population, JSON dtype)
PRECISIONS = {"fp64": (0, 8, "f64"), "fp64fast": (1, 8, "f64"), "fp32": (2, 4, "f32"),
              "bf16": (3, 2, "bf16"), "fp16": (4, 2, "f16"), "fix64": (5, 8, "int64")}


def workload_label(wl, precision):
    """config.workload of a JSON line: the same string from both arms for the
    same lattice and storage (the reference arm always runs FP64)."""
    return "%s_%s" % (wl, precision)


def bytes_per_node(dim, precision):
    """Algorithmic bytes per lattice-node update: one read and one write of
    each population (2*Q*sizeof(storage))."""
    return 2 * (9 if dim == 2 else 27) * PRECISIONS[precision][1]

# The reference-rounding FP64 kernel is bound by GB300's FP64 pipe, not by
# HBM: its default variant issues 201 DFMA per fluid node in D3Q27 and 56 in
# D2Q9 (every addition of the reference's order; multiplications run in
# integer emulation), counted by ncu on the 128x64x64 sphere and the
# 1024x512 cylinder, against the DFMA rate of the device, measured live before the timed region
# (imexlb_fp64_fma_rate; 0.504e12 per second on this part when it cannot run).
FP64_DFMA_PER_NODE = {3: 201, 2: 56}
FP64_DFMA_PEAK = 0.504e12

# DRAM traffic per launch of the step kernel from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum), per workload.
NCU_TRAFFIC_BYTES = {
    # one-kernel capture of 3 launches of the step kernel (boundary copies
    # folded in): 1006.8 MB read + 903.3 MB written, 3% above the 1847.6 MB
    # of algorithmic traffic (the cell mask and the boundary nodes' sources)
    ("sphere_d3q27_256x128x128", "fp64"): 1910.1e6,
    # the 39 GB 512x256x256 case is not captured: the 256x128x128 figure
    # (446.6 B per lattice node) scaled to its 33,883,137 nodes
    ("sphere_d3q27_512x256x256", "fp64"): 15132.7e6,
    # the register kernel k_step_lp with the boundary copies folded in,
    # mean of 3 launches (FP16: one launch)
    ("sphere_d3q27_256x128x128", "fp16"): 454.6e6,
    ("sphere_d3q27_256x128x128", "bf16"): 453.5e6,
    ("sphere_d3q27_256x128x128", "fp32"): 927.0e6,
    # after an L2 flush the launch reads one population buffer (38.6 MB) and
    # its writes (38.5 MB) stay in L2 within the launch: 0.5 MB written
    ("cylinder_d2q9_1024x512", "fp64"): 39.1e6,
}


# The staged BF16 / FP16 kernel (D3Q27): one-kernel capture of the library's
# shape on 256x128x128, FP16 (273.2 MB read + 178.2 MB written, 98% of the
# 461.9 MB algorithmic; BF16 moves the same bytes), and that figure (105.5 B
# per node) scaled to the 33,883,137 nodes of 512x256x256, which is not
# captured. The boundary groups' kernel beside it reads ~1% more.
NCU_TRAFFIC_STAGED = {
    "sphere_d3q27_256x128x128": 451.3e6,
    "sphere_d3q27_512x256x256": 3575.5e6,
}


def _l2_bytes(device):
    """The device's L2 size (129 MB class on GB300)."""
    import torch
    props = torch.cuda.get_device_properties(device)
    return int(getattr(props, "L2_cache_size", 0) or 0) or 132 * 2 ** 20


class L2Flush:
    """Timing of iterations whose population buffers fit in L2: before each
    timed iteration a buffer twice the L2 size is written on the library's
    stream, and only the timed spans count (an event pair around each)."""

    def __init__(self, device, stream):
        import torch
        self.torch = torch
        self.stream = stream
        self.buf = torch.empty(2 * _l2_bytes(device) // 4, dtype=torch.int32, device=device)
        self.pairs = []
        self.k = 0

    def flush(self):
        with self.torch.cuda.stream(self.stream):
            self.buf.fill_(self.k & 0x7fffffff)
        self.k += 1

    def timed(self, fn):
        """Run fn between two events on the stream; returns fn's result."""
        a = self.torch.cuda.Event(enable_timing=True)
        b = self.torch.cuda.Event(enable_timing=True)
        a.record(self.stream)
        r = fn()
        b.record(self.stream)
        self.pairs.append((a, b))
        return r

    def ms(self):
        """Sum of the timed spans (after a synchronize); resets the list."""
        self.torch.cuda.synchronize()
        t = sum(a.elapsed_time(b) for a, b in self.pairs)
        self.pairs = []
        return t


def hold_stream(torch, stream, ms=50.0):
    """Keeps `stream` busy for about `ms` (torch's bounded spin kernel, a fixed
    number of clock cycles at the SM's maximum clock) ahead of a timed
    region's start event. The host then queues the region's launches while
    the device is still busy, so a pause of the host between the start event
    and the first launch (another process querying the driver, say) does
    not count as device time. The region itself is unchanged: the start
    event follows the spin kernel, and the K iterations follow the event.
    (A torch without the spin kernel times the region without the hold.)"""
    sleep = getattr(torch.cuda, "_sleep", None)
    if sleep is None:
        return
    with torch.cuda.stream(stream):
        sleep(int(ms * 1e-3 * SM_MAX_HZ))


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.th.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def _setup(wl):
    import imexlb as im
    w = dict(WORKLOADS[wl])
    dim = w.pop("dim")
    nx, ny, nz = w.pop("nx"), w.pop("ny"), w.pop("nz")
    cfg = im.make_config(dim, nx, ny, nz, **w)
    return cfg, im.Setup(cfg, seed=12345)


def cpu_reference(wl, budget_s, max_steps, threads=None, warmup=1):
    """Time the reference algorithm's CPU path (oracle, OpenMP) on the workload,
    after `warmup` untimed iterations.

    Returns (mlups, steps, seconds, threads)."""
    from oracle import orc
    w = dict(WORKLOADS[wl])
    threads = threads or os.cpu_count() or 1
    o = orc.Oracle(orc.make_input(w["dim"], w["nx"], w["ny"], w["nz"], charlength=w["charlength"],
                                  xpos=w["xpos"], re=w["re"], ome=w["ome"], dt=w["dt"],
                                  rho0=w["rho0"]), nthreads=threads)
    o.init_up(orc.r_vec(12345))
    o.init_pdf()
    o.run(0, warmup, 0)  # warm-up iterations
    nodes = (w["nx"] + 1) * (w["ny"] + 1) * ((w["nz"] + 1) if w["dim"] == 3 else 1)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        o.run(warmup + steps, 1, 0)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    o.close()
    return nodes * steps / dt / 1e6, steps, dt, threads


def _cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def whole_job(ms_local, units_local, dist, device="cpu"):
    """Whole-job timing over the ranks of a replicas run: the slowest rank's
    timed region (MPI-style max) and the units all ranks processed (sum).
    Returns (ms_max, total_units); with dist False the local values."""
    import torch
    if not dist:
        return float(ms_local), float(units_local)
    mx = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    sm = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(sm, op=torch.distributed.ReduceOp.SUM)
    return float(mx.item()), float(sm.item())


def run_reference(args, rank, world):
    if rank != 0:
        return
    wl = args.workload
    dim = WORKLOADS[wl]["dim"]
    # each bench step is one full-domain iteration; the count is bounded so
    # the run ends within a few minutes
    budget = float(os.environ.get("IMEXLB_REF_BUDGET_S", "60"))
    warmup = max(1, args.warmup)
    mlups, steps, dt, threads = cpu_reference(wl, budget, max(1, args.steps), warmup=warmup)
    sample = "%d iterations of the full %s domain after %d warm-up" % (steps, wl, warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mlups, 3), "unit": "MLUPS",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": round(dt / steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (reference geometry generator, seeded InitUP)",
        "config": {"workload": workload_label(wl, "fp64"), "lattice": "D%dQ%d" % (dim, 9 if dim == 2 else 27),
                   "implementation": "C restatement of the reference CPU path (oracle/), OpenMP"},
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads,
                         "kind": "port", "sample": sample, "cpu": _cpu_model()},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


WARMSTART_METRIC = "time-to-Cd/St(+-1%) warm-start+FP16 vs plain FP64 LBM"


def run_warmstart(args, rank, world, local_rank):
    """The learned warm start on the D2Q9 1024x512 cylinder: the network is
    trained (ensemble of 256 cylinder flows, then Adam with the library's
    tensor-core kernels), then for each of K held-out seeds the plain FP64
    run from rest (the arbiter: converged Cd and St from its last quarter) and
    the warm-started FP16 run are timed until their Cd / St stay within 1 %
    of the plain run's converged values. value = median over the seeds of
    (plain wall time to converge) / (warm wall time to converge); one bench
    step is one held-out seed."""
    import numpy as np
    import torch
    from imexlb import warmstart as ws
    torch.cuda.set_device(local_rank)
    if rank != 0:
        return
    ntrain = int(os.environ.get("IMEXLB_WS_TRAIN_STEPS", "2000"))
    net, tinfo = ws.train_network(ncases=256, nx_iters=60, train_steps=ntrain)
    t0 = time.perf_counter()
    rows = ws.evaluate(net, range(1000, 1000 + args.steps), steps=100000, every=20, nx=1024,
                       log=lambda r: None, warm=("warm16", "warm64"))
    eval_s = time.perf_counter() - t0
    summ = ws.summarize(rows)
    per_seed = []
    for r in rows:
        item = {"seed": r["seed"], "re": round(r["Re"], 1), "d": round(r["D"], 1),
                "cd": round(r["cd_ref"], 5), "st": None if not np.isfinite(r["st_ref"]) else round(r["st_ref"], 5)}
        if r["plain_its"] is not None:
            item["plain_s"] = round(r["plain_its"] * r["plain_ms_per_it"] / 1e3, 3)
        for k in ("warm16", "warm64"):
            if r[k + "_its"] is not None:
                item[k + "_s"] = round(max(r[k + "_its"], 1) * r[k + "_ms_per_it"] / 1e3, 3)
        per_seed.append(item)
    value = summ["warm16"]["median_speedup"]
    line = {
        "metric": WARMSTART_METRIC, "value": None if value is None else round(value, 3), "unit": "x",
        "n_gpus": world, "steps": args.steps, "warmup": 0, "ms_per_step": round(eval_s / max(1, args.steps) * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (seeded held-out cylinder cases, reference geometry)",
        "config": {"workload": "warmstart_d2q9_1024x512", "held_out_seeds": list(range(1000, 1000 + args.steps)),
                   "iterations_per_run": 100000, "force_every": 20,
                   "criterion": "trailing 5-period mean Cd and its St within 1% of the plain run's "
                                "converged values until the end",
                   "training": {k: round(v, 4) for k, v in tinfo.items()},
                   "network_gain_fp64_median": summ["warm64"]["median_speedup"],
                   "converged": {"warm16": summ["warm16"]["converged"], "warm64": summ["warm64"]["converged"]},
                   "per_seed": per_seed},
        "e2e": {"value": None if value is None else round(value, 3), "unit": "x",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "note": "wall-clock times through the library's API (host timers around whole runs)"},
    }
    print(json.dumps(line), flush=True)


def run_ensemble(args, rank, world, local_rank):
    """The batched D2Q9 ensemble (256 cylinder cases of different sizes, FP32
    storage, 8*nx iterations each, snapshots every 500): whole-job MLUPS."""
    import torch
    import imexlb as im
    from imexlb import ensemble
    torch.cuda.set_device(local_rank)
    n = int(args.workload.split("_")[2])
    cases = ensemble.draw_cases(n, seed=rank)
    prec = PRECISIONS[args.precision][0] if args.precision != "fp64" else im.FP32
    pname = args.precision if args.precision != "fp64" else "fp32"
    clocks = ClockSampler(local_rank)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    mode = im.BATCH_PERSISTENT if args.batch_mode == "persistent" else im.BATCH_LOCKSTEP
    res = ensemble.run(cases, prec, snapshot_every=500, log=lambda *a: None, mode=mode)
    clk = clocks.stop()
    ms_max, updates = whole_job(res["gpu_seconds"] * 1e3, res["node_updates"], world > 1,
                                "cuda:%d" % local_rank)
    if rank != 0:
        return
    peak, peak_kind = _peaks()
    achieved = res["mlups"] * 1e6 * bytes_per_node(2, pname) / 1e9
    esz = PRECISIONS[pname][1]
    pop_bytes = lambda c: (c["nx"] + 7) * (c["ny"] + 7) * 9 * esz
    last = max(c["steps"] for c in cases)
    line = {
        "metric": METRIC, "value": round(updates / (ms_max / 1e3) / 1e6, 3), "unit": "MLUPS",
        "n_gpus": world,
        "steps": int(max(c["steps"] for c in cases)), "warmup": 0,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": PRECISIONS[pname][2], "data": "synthetic (seeded case table, reference geometry)",
        "config": {"workload": workload_label(args.workload, pname), "cases": n,
                   "node_updates": res["node_updates"], "gpu_seconds": round(res["gpu_seconds"], 3),
                   "launch_shape": res["shape"], "snapshots": "every 500 iterations, 256x128",
                   "batch_mode": args.batch_mode,
                   "boundary_copies": ("fill chunks of the persistent kernel"
                                       if args.batch_mode == "persistent" else "batched fill kernel"),
                   "l2": "no flush; population buffers %.2f GB per set over all cases, "
                         "%.0f MB for the cases still running in the last 1%% of iterations "
                         "(L2 %.0f MB)" % (sum(map(pop_bytes, cases)) / 1e9,
                                           sum(pop_bytes(c) for c in cases
                                               if c["steps"] > 0.99 * last) / 1e6,
                                           _l2_bytes(local_rank) / 1e6)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "note": "whole batch incl. boundary refresh and snapshot sampling"},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def link_rates(host_t, reps=3):
    """Host<->device bandwidth of plain cudaMemcpyAsync copies between the
    pinned tensor host_t and a device buffer of its size (best of `reps` each
    way, GB/s). The copies run on a stream of torch's own: the pinned-memory
    allocator records the copy's stream with the block, so it must not be a
    stream that is destroyed before the tensor is freed."""
    import torch
    stream = torch.cuda.Stream()
    dev = torch.empty(host_t.shape, dtype=host_t.dtype, device=torch.cuda.current_device())
    nbytes = host_t.numel() * host_t.element_size()
    out = {}
    for name, dst, src in (("h2d", dev, host_t), ("d2h", host_t, dev)):
        best = None
        for _ in range(reps + 1):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                dst.copy_(src, non_blocking=True)
                b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = round(nbytes / best / 1e6, 1)
    del dev
    torch.cuda.empty_cache()
    return out


# storage kinds measured beside the FP64 headline on the same state:
# precision -> (arithmetic, step kernel)
VARIANTS = {
    "fix64": ("64-bit fixed point (Q3.60) populations, integer node update with "
              "round-to-nearest products: within 1e-12 of the reference", "k_step_fx"),
    "fp16": ("FP16 storage, FP32 node update with explicit rounding; tiles staged in shared "
             "memory by bulk copies, two cells per thread in packed f32x2 (boundary groups "
             "beside it on a second stream)", "k_step_staged + k_step_bgroups"),
}


def measure_variant(im, torch, cfg, st, hptr, precision, args, device, interv, state_bytes):
    """K timed iterations (CUDA events on the handle's stream, inputs resident)
    and the same end-to-end sequence as the headline (upload, InitPDF, K
    iterations, download through the C ABI) for another storage kind on the
    same state."""
    s = im.Solver(cfg, precision=PRECISIONS[precision][0], device=device)
    try:
        s.set_geometry(st)
        s.upload_ptr(*hptr)
        s.init_pdf()
        stream = torch.cuda.ExternalStream(s.stream(), device=device)
        s.step(0, args.warmup, interv)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        s.profile_reset(timing=True)
        hold_stream(torch, stream)
        e[0].record(stream)
        s.step(args.warmup, args.steps, interv)
        e[1].record(stream)
        torch.cuda.synchronize()
        prof = s.profile()
        s.profile_reset(timing=False)
        ms = e[0].elapsed_time(e[1])
        s.download_ptr(*hptr)  # warm
        s.upload_ptr(*hptr)
        torch.cuda.synchronize()
        e[2].record(stream)
        s.upload_ptr(*hptr)
        s.init_pdf()
        it = 0
        chunk = interv if interv > 0 else args.steps
        while it < args.steps:
            k = min(chunk, args.steps - it)
            s.step(it, k, interv)
            it += k
        s.download_ptr(*hptr)
        e[3].record(stream)
        torch.cuda.synchronize()
        e2e_ms = e[2].elapsed_time(e[3])
    finally:
        s.close()
    peak, _ = _peaks()
    step_ms = prof["ms"][im.KERNEL_STEP] / max(1, prof["launches"][im.KERNEL_STEP])
    achieved = bytes_per_node(cfg.dim, precision) * cfg.nodes / (step_ms / 1e3) / 1e9
    arithmetic, kernel = VARIANTS[precision]
    return {"precision": precision, "arithmetic": arithmetic,
            "value": round(cfg.nodes * args.steps / (ms / 1e3) / 1e6, 3), "unit": "MLUPS",
            "ms_per_step": round(ms / args.steps, 4), "kernel": kernel,
            "kernel_ms": round(step_ms, 4), "roofline_frac": round(achieved / peak, 4),
            "achieved_gbs": round(achieved, 1),
            "e2e": {"value": round(cfg.nodes * args.steps / (e2e_ms / 1e3) / 1e6, 3), "unit": "MLUPS",
                    "h2d_bytes_per_step": round(state_bytes / args.steps, 1),
                    "d2h_bytes_per_step": round(state_bytes / args.steps, 1)}}


def run_ours(args, rank, world, local_rank):
    import torch
    import imexlb as im

    dist = world > 1
    torch.cuda.set_device(local_rank)
    wl = args.workload
    cfg, st = _setup(wl)
    dim, nq, nodes = cfg.dim, cfg.nq, cfg.nodes
    interv = cfg.interv
    n = cfg.array_size

    # pinned host copies of the reference-layout state (one set: the e2e
    # region uploads from it and downloads into it; the numpy arrays are
    # dropped, which keeps the 512x256x256 case at ~17 GB of host memory)
    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64).pin_memory()
        t.numpy()[:] = a
        return t

    s = im.Solver(cfg, precision=PRECISIONS[args.precision][0], device=local_rank)
    s.set_geometry(st)
    if args.fill != "auto":
        s.set_fill_mode(im.FILL_FUSED if args.fill == "fused" else im.FILL_KERNEL)
    fill_used = s.fill_mode()
    if args.lp_kernel == "register":
        s.set_staged_kernel(False)
    host = [pinned(st.f), pinned(st.fb), pinned(st.p), pinned(st.u)]
    st.f = st.fb = st.p = st.u = None
    hptr = [t.data_ptr() for t in host]
    s.upload_ptr(*hptr)
    s.init_pdf()
    info = s.info()
    stream = torch.cuda.ExternalStream(s.stream(), device=local_rank)

    def barrier():
        if dist:
            torch.distributed.barrier()

    # the FP64 fused multiply-add rate, the bound of the reference-order kernel
    dfma_peak, dfma_src = FP64_DFMA_PEAK, "earlier measurement on this part (live measurement failed)"
    if args.precision == "fp64":
        try:
            dfma_peak, dfma_src = im.fp64_fma_rate(local_rank), "measured live (imexlb_fp64_fma_rate)"
        except Exception:
            pass
    # A population buffer no larger than L2 would stay cached from one
    # iteration to the next: then L2 is flushed before every timed iteration.
    buf_bytes = n * nq * PRECISIONS[args.precision][1]
    l2 = L2Flush(local_rank, stream) if buf_bytes <= _l2_bytes(local_rank) else None
    # warm-up iterations
    s.step(0, args.warmup, interv)
    # device-resident timed region: K iterations, inputs in HBM
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.4)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    s.profile_reset(timing=True)
    if l2 is None:
        hold_stream(torch, stream)
        e0.record(stream)
        s.step(args.warmup, args.steps, interv)
        e1.record(stream)
    else:
        # one iteration per call; imexlb_step returns after its iteration
        # completes, so the iteration's device time is taken from the
        # library's own events around each of its launches
        for it in range(args.warmup, args.warmup + args.steps):
            l2.flush()
            s.step(it, 1, interv)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    prof = s.profile()
    ms = e0.elapsed_time(e1) if l2 is None else sum(prof["ms"])
    s.profile_reset(timing=False)
    ms_max, units = whole_job(ms, nodes * args.steps, dist, "cuda:%d" % local_rank)
    value = units / (ms_max / 1e3) / 1e6

    # end-to-end through the C ABI with pinned host buffers: upload a state
    # (f, fb, p, u), InitPDF, K iterations in Monitor intervals (each call
    # returns its Monitor value to the host), download f, fb, p, u.
    s.download_ptr(*hptr)  # warm (builds the download's ghost list)
    s.upload_ptr(*hptr)    # warm: the first host copies after a large download run slower
    barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    mon_values = 0
    phases = None
    if l2 is None:
        ev[0].record(stream)
        h0 = time.perf_counter()
        s.upload_ptr(*hptr)
        h1 = time.perf_counter()
        ev[1].record(stream)
        s.init_pdf()
        it = 0
        chunk = interv if interv > 0 else args.steps
        while it < args.steps:
            k = min(chunk, args.steps - it)
            mon_values += s.step(it, k, interv).size
            it += k
        ev[2].record(stream)
        h2 = time.perf_counter()
        s.download_ptr(*hptr)
        h3 = time.perf_counter()
        ev[3].record(stream)
        torch.cuda.synchronize()
        e2e_ms = ev[0].elapsed_time(ev[3])
        phases = (ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3]), 1e3 * (h1 - h0),
                  1e3 * (h3 - h2))
    else:
        # the same calls, one iteration per step call with L2 flushed before
        # each; the flushes are outside the timed spans, the return of each
        # blocking call inside
        l2.flush()
        l2.timed(lambda: (s.upload_ptr(*hptr), s.init_pdf()))
        for it in range(args.steps):
            l2.flush()
            mon_values += l2.timed(lambda: s.step(it, 1, interv)).size
        l2.flush()
        l2.timed(lambda: s.download_ptr(*hptr))
        e2e_ms = l2.ms()
    e2e_ms, units = whole_job(e2e_ms, nodes * args.steps, dist, "cuda:%d" % local_rank)
    state_bytes = n * (2 * nq + 1 + dim) * 8
    e2e = {"value": round(units / (e2e_ms / 1e3) / 1e6, 3), "unit": "MLUPS",
           "h2d_bytes_per_step": round(state_bytes / args.steps, 1),
           "d2h_bytes_per_step": round((state_bytes + 8 * mon_values) / args.steps, 1)}
    if phases is not None:
        # the link's bound: a plain pinned cudaMemcpyAsync of the largest
        # array (f) each way, beside what the upload / download calls achieve
        # (their layout conversion included)
        link = link_rates(host[0])
        e2e["copy_gbs"] = {"h2d": round(state_bytes / phases[0] / 1e6, 1),
                           "d2h": round(state_bytes / phases[1] / 1e6, 1)}
        e2e["link_gbs"] = link
        e2e["copy_ms"] = {"upload": round(phases[0], 2), "download": round(phases[1], 2),
                          "upload_host": round(phases[2], 2), "download_host": round(phases[3], 2)}
    s.close()
    # the fixed-point kind (the drop-in's 1e-12 accuracy off the FP64 pipe)
    # and the FP16 storage kind on the same state and workload, beside the
    # bitwise headline
    variants = {}
    if args.precision == "fp64" and dim == 3 and not args.no_variants:
        for v in VARIANTS:
            variants[v] = measure_variant(im, torch, cfg, st, hptr, v, args, local_rank, interv,
                                          state_bytes)
    host = hptr = None  # release the pinned state before the CPU baseline

    if rank != 0:
        return
    peak, peak_kind = _peaks()
    L = prof["launches"]
    step_ms = prof["ms"][im.KERNEL_STEP] / max(1, L[im.KERNEL_STEP])
    alg_bytes = bytes_per_node(dim, args.precision) * nodes
    achieved = alg_bytes / (step_ms / 1e3) / 1e9
    traffic = NCU_TRAFFIC_BYTES.get((wl, args.precision))
    staged = (args.precision in ("fp16", "bf16") and dim == 3 and args.lp_kernel == "staged")
    if staged:
        traffic = NCU_TRAFFIC_STAGED.get(wl)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "kernel": ("k_step_staged + k_step_bgroups (staged pull-collide, boundary "
                           "groups beside it)"
                           if staged else
                           "%s (fused pull-collide)" % ("k_step" if args.precision == "fp64" else
                                                        "k_step_fx" if args.precision == "fix64" else
                                                        "k_step_lp")),
                "kernel_ms": round(step_ms, 4),
                "alg_bytes_per_launch": alg_bytes,
                "kernel_share": round(prof["ms"][im.KERNEL_STEP] / max(1e-9, sum(prof["ms"])), 4)}
    if args.precision == "fp64" and dim in FP64_DFMA_PER_NODE:
        dfma = FP64_DFMA_PER_NODE[dim] * int(info.size_fluid) / (step_ms / 1e3)
        roofline["fp64_pipe"] = {"unit": "DFMA/s", "achieved": round(dfma / 1e9, 1) * 1e9,
                                 "peak": round(dfma_peak / 1e9, 1) * 1e9,
                                 "frac": round(dfma / dfma_peak, 4),
                                 "per_fluid_node": FP64_DFMA_PER_NODE[dim],
                                 "peak_source": dfma_src}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": PRECISIONS[args.precision][2],
        "data": "synthetic (reference geometry generator, seeded InitUP)",
        "config": {"workload": workload_label(wl, args.precision), "lattice": "D%dQ%d" % (dim, nq),
                   "nodes": nodes,
                   "fluid_nodes": int(info.size_fluid),
                   "mlups_fluid_nodes": round(value * int(info.size_fluid) / nodes, 3),
                   "monitor_interval": interv,
                   "arithmetic": ("IEEE f64, reference evaluation order and rounding (bitwise); "
                                  "multiplications in exact integer emulation, additions as "
                                  "exact fused multiply-adds a*1+b"
                                  if args.precision == "fp64" else
                                  "IEEE f64, minimal operation count with FMA (not bitwise)"
                                  if args.precision == "fp64fast" else
                                  "64-bit fixed point (Q3.60) storage and integer arithmetic, "
                                  "round-to-nearest products (within 1e-12 of the reference)"
                                  if args.precision == "fix64" else
                                  "%s storage of the deviation f, FP32 arithmetic with explicit "
                                  "rounding, FP64 force/mass" % args.precision),
                   **({"step_kernel": ("tiles staged in shared memory by bulk copies, two "
                                       "cells per thread in packed f32x2 (k_step_staged), "
                                       "boundary groups beside it (k_step_bgroups)"
                                       if args.lp_kernel == "staged" else
                                       "populations loaded into registers (k_step_lp)")}
                      if args.precision in ("fp16", "bf16") and dim == 3 else {}),
                   "l2": ("inputs larger than L2: two %.2f GB population buffers"
                          % (buf_bytes / 1e9) if l2 is None else
                          "L2 flushed before every timed iteration (population buffers of "
                          "%.1f MB fit in L2): one iteration per call, value from CUDA events "
                          "around each launch, e2e from events around each call"
                          % (buf_bytes / 1e6)),
                   "boundary_copies": ("inside the step kernel" if fill_used == im.FILL_FUSED
                                       else "separate fill kernel"),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": int(sum(L)),
        **({"variants": variants} if variants else {}),
        "clocks": clk,
    }
    if world == 1 and not args.no_cpu_baseline:
        budget = float(os.environ.get("IMEXLB_CPU_BUDGET_S", "20"))
        mlups, steps, dt, threads = cpu_reference(wl, budget, 1000)
        line["cpu_baseline"] = {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads,
                                "kind": "port", "cpu": _cpu_model(),
                                "sample": "%d iterations of the full domain (%.1f s)" % (steps, dt)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    help="one of %s, ensemble_d2q9_<cases>, or warmstart_d2q9_1024x512 (the "
                         "learned warm start: --steps held-out seeds)" % ", ".join(sorted(WORKLOADS)))
    ap.add_argument("--precision", default="fp64", choices=sorted(PRECISIONS))
    ap.add_argument("--fill", default="auto", choices=["auto", "fused", "kernel"],
                    help="boundary copies inside the step kernel, in a separate kernel, or "
                         "the library's default for the workload")
    ap.add_argument("--batch-mode", default="lockstep", choices=["lockstep", "persistent"],
                    help="ensemble workloads: one cooperative launch per call, or one "
                         "graph-replayed launch pair per iteration")
    ap.add_argument("--lp-kernel", default="staged", choices=["staged", "register"],
                    help="BF16 / FP16 on D3Q27: the step kernel fed by bulk copies into "
                         "shared memory (the library's default) or the one that loads every "
                         "population into registers (identical results)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true",
                    help="leave out the fixed-point kind's figures beside an FP64 3D line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    try:
        if args.workload.startswith("ensemble_d2q9_"):
            run_ensemble(args, rank, world, local_rank)
        elif args.workload == "warmstart_d2q9_1024x512":
            run_warmstart(args, rank, world, local_rank)
        else:
            run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    main()
