#!/usr/bin/env python3
"""Benchmark of the physical-optics integrator on one GB300 per rank.

Workload (default `dish_eh`): paraboloid D 1000 mm, f 500 mm, uv 501x501
(251,001 source points, lambda 1 mm) radiating to a 301x301 focal-plane grid
(90,601 targets), mode EH: 2.27e10 source-target pairs. Inputs are seeded
synthetic currents with the configuration's taper and phase noise (M = 0).

A step is one forward propagation of the whole workload plus its adjoint:
the gradient of a loss on the output fields (a fixed random cotangent) with
respect to the source currents and to the normal displacement of every
source and target point. value = pairs per step / step time (each pair
counted once per forward+adjoint step).
  value  inputs resident on the device (po_run_dev + po_adjoint_dev)
  e2e    the same through the host-buffer C-ABI (po_run_d + po_adjoint_d):
         H2D of each call's inputs from pinned memory and D2H of its outputs
         inside the timed region
Also reported: the forward and adjoint accuracy against the plain FP64 GPU
path, the FP64 GPU path's own step rate, the FP32 roofline of each kernel
(CUDA events around every launch on its stream), the clocks during the timed
region, and the FP64 CPU oracle on a bounded sample.

`--workload cassegrain` benchmarks the Cassegrain chain instead: feed (201x201) -> hyperboloid (401x401, JM) -> paraboloid (1001x1001,
JM) -> far field (201x201, FF), ~2.1e11 pairs; `--workload dish_chain` the
perturbed-dish chain: feed (101x101) -> dish (301x301, JM, with its seeded
surface error) -> far field (101x101, FF). For a chain, a step is the forward chain
plus its backward pass (the currents' cotangents through every stage and the
displacement gradients of every reflector), through torch autograd on device
tensors (value) and through the host-buffer C-ABI with the chain rule applied
stage by stage (e2e). The FP64 GPU chain is timed per stage on source
subsamples and combined by pairs; the accuracy is the mixed chain against
the FP64 chain at scale 0.2.

`--impl reference` times the reference's CPU path on the host cores, on the
same workload and the same step: the FP64 C restatement of the reference's
forward (oracle/po_oracle.c, pinned to the reference's own outputs) plus the
FP64 C adjoint (the reference has none; po_oracle_adjoint states the same
formulas), over every source and a random sample of targets sized to a few
seconds a step. Its ms_per_step is that sampled step as timed; its value is
pairs per second. The arm imports only oracle/ (inputs from
oracle/workloads.py, equal to pypo_gb300/configs.py's): no product code
runs on it.

The default run (dish_eh, full size, one GPU) also measures the far-field
configuration (dish_ff: 1001x1001 dish -> 401x401 far field, 1.6e11 pairs)
and the Cassegrain chain the same way in shorter runs (3 timed steps) and
reports them under `other_configs`; --no-others skips them.

Multi-GPU: one process per GPU (torchrun); each rank runs its own replica of
the workload (targets are independent, no collective on the data path);
value = all ranks' pairs / max-over-ranks time ("scaling": "weak").
"""
import argparse
import json
import os
import pathlib
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gpairs/s fwd+adjoint, mixed-prec vs FP64 sum, 1 GB300 at ≤1e-5 rel err vs FP64"
#: algorithmic FP32 flops per pair (FMA = 2; split-precision overhead not counted)
FWD_FLOPS = {("EH", True): 234, ("EH", False): 140, ("FF", True): 61, ("FF", False): 37}
# Adjoint. Near field: the fused kernel (currents 12 rows, source displacement
# 416 flops/pair, plus 50 for the target displacement sharing the pair's
# geometry, phase, coefficients, S and Z = b x J - a x M, from which
# W.v = -v.Z for v = R_hat, n_s, n_t); sources with M add 116 (source side:
# alpha 24, M.R_hat 10, beta 8, a x M into Z 48, b.n_s 10, grad(beta).n_s 16)
# and 26 (target side: M.n_t 10, grad(beta).n_t 16). Far field: currents +
# source displacement, 99; with M, +24.
ADJ_FLOPS = {("EH", False): 466, ("EH", True): 608, ("FF", False): 99, ("FF", True): 123}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampled every 200 ms while running (started before, stopped after)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.index)], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for ln in fh:
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 8:
                    try:
                        rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[4:8]))
                    except ValueError:
                        pass
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [r[0] for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3][i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def gpu_index(local):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    parts = [p for p in vis.split(",") if p.strip()]
    if parts and len(parts) > local and parts[local].strip().isdigit():
        return int(parts[local])
    return local


#: the workloads as the JSON line names them (both arms print the same config)
DESCS = {
    "dish_eh": "paraboloid D1000 f500 uv 501x501 -> focal plane 301x301 +-50 mm, lambda 1.0 mm, EH, M=0",
    "dish_ff": "paraboloid D2000 f800 uv 1001x1001 -> far field 401x401 +-0.5 deg, lambda 1.0 mm, FF, M=0",
    "feed_dish_jm": "Gaussian feed 101x101 -> f300 D300 dish uv 101x101, lambda 3 mm, JM",
    "cassegrain": "feed 201^2 -> hyperboloid 401^2 -> paraboloid 1001^2 -> FF 201^2, lambda 1 mm",
    "dish_chain": "feed 101^2 -> dish 301^2 (+surface error) -> FF 101^2, lambda 2 mm",
}
STEP = "forward + adjoint (grad wrt currents, source and target normal displacement)"
STEP_CHAIN = "forward chain + backward (currents' cotangents, displacement of every reflector)"
L2 = ("GPU arm: flushed before every step (256 MB write inside the timed loop); CPU arm: "
      "not applicable (host caches, inputs larger than them)")


def config_of(name, scale, pairs, **extra):
    """The `config` object, identical for both arms of one workload."""
    c = {"workload": name + ("" if scale == 1.0 else f" (scale {scale})"), "desc": DESCS[name],
         "pairs_per_step": pairs, **extra}
    c["step"] = STEP_CHAIN if name in CHAINS else STEP
    c["l2"] = L2
    return c


def field_errors(got, ref, mode):
    """Relative L2 over every row, and the largest phase error over the complex
    components within 20 dB and 40 dB of the sample's largest component."""
    got, ref = np.asarray(got), np.asarray(ref)
    out = {"rel_l2": float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))}
    nc = {"scalar": 1, "JMEH": 4}.get(mode, 2)
    rc = np.concatenate([ref[6 * b:6 * b + 3] + 1j * ref[6 * b + 3:6 * b + 6] for b in range(nc)]) \
        if mode != "scalar" else ref[0:1] + 1j * ref[1:2]
    gc = np.concatenate([got[6 * b:6 * b + 3] + 1j * got[6 * b + 3:6 * b + 6] for b in range(nc)]) \
        if mode != "scalar" else got[0:1] + 1j * got[1:2]
    mag = np.abs(rc)
    for db in (20, 40):
        sel = mag >= mag.max() * 10 ** (-db / 20)
        out[f"max_phase_rad_{db}db"] = float(np.abs(np.angle(gc[sel] / rc[sel])).max()) if sel.any() else 0.0
    return out


def cot_for(mode, nt):
    """The step's cotangent: seeded, the same in both arms."""
    return np.random.default_rng(7).standard_normal((N_OUT[mode], nt))


N_OUT = {"JM": 12, "EH": 12, "JMEH": 24, "EHP": 15, "FF": 12, "scalar": 2}


def cpu_step(w, cot, idx, threads):
    """One step of the FP64 CPU path over every source and the targets `idx`:
    the oracle's forward (the reference's algorithm) and its adjoint. Returns
    (forward rows, gradients, forward seconds, adjoint seconds)."""
    from oracle import oracle as O
    t7s = np.ascontiguousarray(w["t7"][:, idx])
    cots = np.ascontiguousarray(cot[:, idx])
    grid = (w["gmode"], w["ncx"], w["ncy"])
    t0 = time.perf_counter()
    out = O.run(w["mode"], w["s7"], w["cur"], *grid, t7s, w["k"], 1.0, -1.0, nthreads=threads)
    t1 = time.perf_counter()
    g = O.adjoint(w["mode"], w["s7"], w["cur"], *grid, t7s, w["k"], cots, 1.0, -1.0, nthreads=threads)
    t2 = time.perf_counter()
    return out, g, t1 - t0, t2 - t1


def cpu_sample_size(w, cot, seconds, threads, rng):
    """Number of sampled targets for which one CPU step takes about `seconds`."""
    nt = w["t7"].shape[1]
    n0 = min(nt, max(threads, 16))
    _, _, tf, ta = cpu_step(w, cot, np.sort(rng.choice(nt, size=n0, replace=False)), threads)
    return int(min(nt, max(n0, n0 * seconds / max(tf + ta, 1e-3))))


#: chain workloads: config builder, stages (mode, source, source grid, target),
#: displaced reflectors (their normal displacement is a differentiated input)
CHAINS = {
    "cassegrain": ("cassegrain", [("JM", "feed7", "feed_grid", "sec7"), ("JM", "sec7", "sec_grid", "prim7"),
                                  ("FF", "prim7", "prim_grid", "ff7")], ["sec7", "prim7"]),
    "dish_chain": ("dish_chain", [("JM", "feed7", "feed_grid", "dish7"), ("FF", "dish7", "dish_grid", "ff7")],
                   ["dish7"]),
}


def chain_config(name, scale=1.0):
    """The product's chain configuration (the GPU arm)."""
    from pypo_gb300 import configs
    builder, stages, refl = CHAINS[name]
    c = getattr(configs, builder)(scale=scale)
    # initial normal displacement of each reflector: the configuration's surface error, if it has one
    disp = {r: (c["delta"] if "delta" in c else np.zeros(c[r].shape[1])) for r in refl}
    return c, stages, refl, disp


def chain_stage_workloads(c, stages):
    """The chain's stages as workload dicts (cpu_step's inputs) with a seeded
    cotangent each; the source currents after the feed are seeded random rows
    (the step's cost does not depend on their values)."""
    rng = np.random.default_rng(11)
    out = []
    for mode, skey, gkey, tkey in stages:
        g = c[gkey]
        cur = c["feed_cur"] if skey == "feed7" else rng.standard_normal((12, c[skey].shape[1]))
        w = dict(mode=mode, s7=c[skey], cur=cur, gmode=g[0], ncx=g[1], ncy=g[2], t7=c[tkey], k=c["k"])
        w["cot"] = rng.standard_normal((N_OUT[mode], c[tkey].shape[1]))
        out.append(w)
    return out


def cpu_chain_step(ws, frac, threads, rng):
    """One sampled step of the FP64 CPU chain: in every stage, forward and
    adjoint over all its sources and the same fraction `frac` of its targets,
    so that the sampled pairs are in the stages' proportion. Returns (pairs,
    seconds, per-stage descriptions)."""
    pairs, secs, parts = 0, 0.0, []
    for w in ws:
        nt, ns = w["t7"].shape[1], w["s7"].shape[1]
        n = int(min(nt, max(1, round(frac * nt))))
        idx = np.sort(rng.choice(nt, size=n, replace=False))
        _, _, tf, ta = cpu_step(w, w["cot"], idx, threads)
        pairs += ns * n
        secs += tf + ta
        parts.append(f"{n} targets x {ns} sources")
    return pairs, secs, parts


def cpu_chain_fraction(ws, seconds, threads, rng):
    total = sum(w["s7"].shape[1] * w["t7"].shape[1] for w in ws)
    f0 = 2e6 / total
    p, sec, _ = cpu_chain_step(ws, f0, threads, rng)
    return min(1.0, f0 * seconds / max(sec, 1e-3))


def dish_chain_fd(c, grad, cot, k, nodes=64, h_lam=1e-6):
    """The perturbed-dish chain's displacement gradient against central finite
    differences of the FP64 oracle chain (the reference's CPU algorithm) on 64
    seeded dish nodes (h = 1e-6 lambda). The loss sum(cot * far field) is a
    sum of per-node far-field terms, and a node's displacement changes only its
    own (its induced current and its position), so each difference needs that
    node alone: a one-target JM from the feed and a one-source FF."""
    from oracle import oracle as O
    f7, fcur, d7, ff7 = c["feed7"], c["feed_cur"], c["dish7"], c["ff7"]
    fg, (gm, ncx, ncy) = c["feed_grid"], c["dish_grid"]
    h = h_lam * c["lam"]
    pick = np.random.default_rng(2).choice(d7.shape[1], nodes, replace=False)
    threads = os.cpu_count() or 1

    def term(i, delta):
        p7 = d7[:, i:i + 1].copy()
        p7[:3, 0] += delta * d7[3:6, i]
        ji = O.run("JM", f7, fcur, *fg, p7, k, nthreads=1)
        xu, yv = i // ncy, i % ncy   # the dish grid's trapezoid weight of node i
        w = (0.5 if xu in (0, ncx - 1) else 1.0) * (0.5 if gm != 1 and yv in (0, ncy - 1) else 1.0)
        p7[6, 0] *= w
        return float((O.run("FF", p7, ji, -1, 0, 0, ff7, k, nthreads=threads) * cot).sum())

    fd = np.array([(term(i, c["delta"][i] + h) - term(i, c["delta"][i] - h)) / (2 * h) for i in pick])
    g = grad[pick]
    return {"rel_l2": float(np.linalg.norm(g - fd) / np.linalg.norm(fd)), "nodes": nodes,
            "h": f"{h_lam:g} lambda", "gradient": "mixed-precision autograd of the timed step",
            "against": "central differences of the FP64 CPU oracle chain (the reference's algorithm), "
                       "one node moved at a time"}


def reference_line(args, world, value, ms, timed_pairs, full_pairs, threads, sample, config):
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (the same inputs as the GPU arm)",
            "config": config, "device": "cpu", "precision": "FP64",
            "timed_pairs_per_step": timed_pairs,
            "full_step_ms_extrapolated": full_pairs / (value * 1e9) * 1e3,
            "cpu_baseline": {"value": value, "unit": "Gpairs/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}


def run_reference(args):
    """The CPU arm: the reference's algorithm (the oracle's C restatement,
    pinned to the reference's outputs) timed on the host cores on the same
    workload and step, each step a bounded sample of it. Imports only oracle/."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import workloads as OW
    threads = os.cpu_count() or 1
    per_step = max(0.2, args.cpu_seconds / max(1, args.steps + args.warmup))
    rng = np.random.default_rng(123)
    if args.workload in CHAINS:
        builder, stages, _ = CHAINS[args.workload]
        c = OW.CHAINS[builder](scale=args.scale)
        ws = chain_stage_workloads(c, stages)
        full = sum(w["s7"].shape[1] * w["t7"].shape[1] for w in ws)
        frac = cpu_chain_fraction(ws, per_step, threads, rng)
        times, pairs, parts = [], 0, []
        for i in range(args.warmup + args.steps):
            pairs, sec, parts = cpu_chain_step(ws, frac, threads, rng)
            if i >= args.warmup:
                times.append(sec)
        sec = float(np.mean(times))
        value = pairs / sec / 1e9
        sample = ("per stage " + "; ".join(parts) + f" (a fraction {frac:.2e} of every stage's targets), "
                  "forward + adjoint, FP64 oracle")
        line = reference_line(args, world, value, sec * 1e3, pairs, full, threads, sample,
                              config_of(args.workload, args.scale, full,
                                        stage_pairs=[w["s7"].shape[1] * w["t7"].shape[1] for w in ws]))
        print(json.dumps(line), flush=True)
        return
    w = OW.WORKLOADS[args.workload](scale=args.scale)   # equal to the GPU arm's inputs
    nt, ns = w["t7"].shape[1], w["s7"].shape[1]
    cot = cot_for(w["mode"], nt)
    n = cpu_sample_size(w, cot, per_step, threads, rng)
    times = []
    for i in range(args.warmup + args.steps):
        idx = np.sort(rng.choice(nt, size=n, replace=False))
        _, _, tf, ta = cpu_step(w, cot, idx, threads)
        if i >= args.warmup:
            times.append(tf + ta)
    sec = float(np.mean(times))
    value = ns * n / sec / 1e9
    sample = (f"{n} random targets x {ns} sources per step (a new sample every step), forward + adjoint, "
              "FP64 oracle")
    line = reference_line(args, world, value, sec * 1e3, ns * n, w["pairs"], threads, sample,
                          config_of(args.workload, args.scale, w["pairs"], ns=ns, nt=nt))
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    from pypo_gb300 import build as B
    B.build()
    from pypo_gb300 import configs, engine
    from pypo_gb300._lib import load

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    w = configs.WORKLOADS[args.workload](scale=args.scale)
    mode, k = w["mode"], w["k"]
    m_zero = not np.any(w["cur"][6:])
    ns, nt = w["s7"].shape[1], w["t7"].shape[1]
    nout = engine.n_out(mode)
    far = mode == "FF"
    cot_np = cot_for(mode, nt)
    rng = np.random.default_rng(8)
    s7 = torch.tensor(np.ascontiguousarray(w["s7"]), device=dev)
    cur = torch.tensor(np.ascontiguousarray(w["cur"]), device=dev)
    t7 = torch.tensor(np.ascontiguousarray(w["t7"]), device=dev)
    cot = torch.tensor(cot_np, device=dev)
    out = torch.empty((nout, nt), dtype=torch.float64, device=dev)
    g_cur = torch.empty((12, ns), dtype=torch.float64, device=dev)
    g_ds = torch.empty(ns, dtype=torch.float64, device=dev)
    g_dt = None if far else torch.empty(nt, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream(dev)
    grid = (w["gmode"], w["ncx"], w["ncy"])

    def step():
        flush.zero_()
        engine.propagate_dev(mode, s7, cur, *grid, t7, k, 1.0, -1.0, "mixed", m_zero=m_zero, out=out,
                             stream=stream)
        n1 = engine.last_launches()
        engine.adjoint_dev(mode, s7, cur, *grid, t7, k, cot, 1.0, -1.0, "mixed", m_zero=m_zero, grad_cur=g_cur,
                           grad_ds=g_ds, grad_dt=g_dt, stream=stream)
        return n1 + engine.last_launches()

    for _ in range(args.warmup):
        launches_per_step = step()
    torch.cuda.synchronize()
    kernels_per_step = 2   # forward + adjoint
    engine.timing_enable(args.steps * kernels_per_step)
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    launch_ms = np.array(engine.timing_collect()).reshape(args.steps, kernels_per_step)
    engine.timing_enable(0)
    assert engine.device_error(stream) == 0, "a kernel reported a wait timeout"
    if world > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = w["pairs"] * args.steps * world / (ms * 1e-3) / 1e9

    # ---- end to end through the host-buffer C-ABI (pinned host memory)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    s7_h, cur_h, t7_h, cot_h = pin(w["s7"]), pin(w["cur"]), pin(w["t7"]), pin(cot_np)
    out_h = torch.empty((nout, nt), dtype=torch.float64).pin_memory()
    gc_h = torch.empty((12, ns), dtype=torch.float64).pin_memory()
    gs_h = torch.empty(ns, dtype=torch.float64).pin_memory()
    gt_h = torch.empty(nt, dtype=torch.float64).pin_memory()
    lib = load()

    def step_e2e():
        flush.zero_()
        engine.propagate(mode, s7_h.numpy(), cur_h.numpy(), *grid, t7_h.numpy(), k, 1.0, -1.0, "mixed",
                         out=out_h.numpy())
        rc = lib.po_adjoint_d(engine.MODE_ID[mode], ns, s7_h.data_ptr(), *grid, cur_h.data_ptr(), nt,
                              t7_h.data_ptr(), float(k), 1.0, -1.0, 0, cot_h.data_ptr(), gc_h.data_ptr(),
                              gs_h.data_ptr(), None if far else gt_h.data_ptr())
        assert rc == 0, lib.po_last_error()

    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = w["pairs"] * args.steps / e2e_s / 1e9 * world
    h2d = 2 * (7 + 12) * ns * 8 + 2 * 7 * nt * 8 + nout * nt * 8
    d2h = nout * nt * 8 + 13 * ns * 8 + (0 if far else nt * 8)

    # ---- the forward as a PyPO user calls it: BindGPU.PyPO_GPUf with the
    # reference's arguments (reflDicts, runPODict, a currents object) through
    # the float drop-in ABI callKernelf_*, which generates both grids inside
    # the call; the result comes back as PyPO field objects
    drop_in = None
    if w.get("src") is not None and w.get("tgt") is not None:
        from pypo_gb300 import BindGPU, PyPOTypes as PT
        shape = tuple(int(v) for v in w["src"]["gridsize"])
        comps = [(w["cur"][6 * g + a] + 1j * w["cur"][6 * g + 3 + a]).reshape(shape) for g in range(2)
                 for a in range(3)]
        sc = PT.currents(*comps)
        sc.setMeta("src", float(k))
        rdict = {"mode": mode, "exp": "fwd", "epsilon": 1.0, "k": float(k), "nThreads": 256, "s_current": sc}
        BindGPU.PyPO_GPUf(w["src"], w["tgt"], dict(rdict))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            BindGPU.PyPO_GPUf(w["src"], w["tgt"], dict(rdict))
        drop_s = (time.perf_counter() - t0) / args.steps
        drop_in = {"value": w["pairs"] / drop_s / 1e9, "unit": "Gpairs/s", "ms_per_call": drop_s * 1e3,
                   "path": "BindGPU.PyPO_GPUf -> callKernelf_" + mode + " (the reference's float ABI, both grids "
                           "generated inside the call, results as PyPO field objects), forward only: the "
                           "reference has no adjoint"}
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- forward accuracy against the plain FP64 GPU sum (sampled targets, all sources)
    idx = np.sort(rng.choice(nt, size=min(1024, nt), replace=False))
    t7s = torch.tensor(np.ascontiguousarray(w["t7"][:, idx]), device=dev)
    ref = engine.propagate_dev(mode, s7, cur, *grid, t7s, k, 1.0, -1.0, "fp64")
    torch.cuda.synchronize()
    acc_gpu64 = field_errors(out[:, idx].cpu().numpy(), ref.cpu().numpy(), mode)

    # ---- the reference's CPU path (the FP64 oracle) on a random target sample:
    # its rate (cpu_baseline) and the GPU results against its outputs
    threads = os.cpu_count() or 1
    crng = np.random.default_rng(123)
    ncpu = cpu_sample_size(w, cot_np, args.cpu_sample_s, threads, crng)
    cidx = np.sort(crng.choice(nt, size=ncpu, replace=False))
    ref_out, ref_g, cpu_tf, cpu_ta = cpu_step(w, cot_np, cidx, threads)
    cpu_rate = ns * ncpu / (cpu_tf + cpu_ta)
    acc_cpu = field_errors(out[:, cidx].cpu().numpy(), ref_out, mode)
    # the mixed adjoint over every source and the sampled targets, against the CPU adjoint
    t7c = torch.tensor(np.ascontiguousarray(w["t7"][:, cidx]), device=dev)
    cotc = torch.tensor(np.ascontiguousarray(cot_np[:, cidx]), device=dev)
    gcc = torch.empty((12, ns), dtype=torch.float64, device=dev)
    gsc = torch.empty(ns, dtype=torch.float64, device=dev)
    gtc = None if far else torch.empty(ncpu, dtype=torch.float64, device=dev)
    engine.adjoint_dev(mode, s7, cur, *grid, t7c, k, cotc, 1.0, -1.0, "mixed", m_zero=m_zero, grad_cur=gcc,
                       grad_ds=gsc, grad_dt=gtc)
    torch.cuda.synchronize()
    rel_np = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    adj_cpu = {"grad_cur_rel_l2": rel_np(gcc.cpu().numpy(), ref_g["cur"]),
               "grad_ds_rel_l2": rel_np(gsc.cpu().numpy(), ref_g["ds"])}
    if not far:
        adj_cpu["grad_dt_rel_l2"] = rel_np(gtc.cpu().numpy(), ref_g["dt"])

    # ---- adjoint accuracy and FP64 step rate on a sub-problem: all targets and
    # every fstep-th source, with fstep chosen so that the FP64 kernels, one
    # thread per source or per target, still get >= 65536 threads (a full GPU)
    fstep = max(1, ns // 65536)
    sub = slice(0, ns, fstep)
    s7f, curf = s7[:, sub].contiguous(), cur[:, sub].contiguous()
    nsf = s7f.shape[1]

    def adj(prec):
        gc = torch.empty((12, nsf), dtype=torch.float64, device=dev)
        gs = torch.empty(nsf, dtype=torch.float64, device=dev)
        gt = None if far else torch.empty(nt, dtype=torch.float64, device=dev)
        engine.adjoint_dev(mode, s7f, curf, -1, 0, 0, t7, k, cot, 1.0, -1.0, prec, m_zero=m_zero, grad_cur=gc,
                           grad_ds=gs, grad_dt=gt)
        return gc, gs, gt

    def rel(a, b):
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))

    am, ad = adj("mixed"), adj("fp64")
    torch.cuda.synchronize()
    adj_acc = {"grad_cur_rel_l2": rel(am[0], ad[0]), "grad_ds_rel_l2": rel(am[1], ad[1])}
    if not far:
        adj_acc["grad_dt_rel_l2"] = rel(am[2], ad[2])
    outf = torch.empty_like(out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    engine.propagate_dev(mode, s7f, curf, -1, 0, 0, t7, k, 1.0, -1.0, "fp64", out=outf)
    adj("fp64")
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_rate = nsf * nt / (e0.elapsed_time(e1) * 1e-3) / 1e9

    # ---- FP32 roofline of each kernel of the step
    probe = torch.empty(152 * 8 * 256, dtype=torch.float32, device=dev)
    blocks, iters = probe.numel() // 256, 100000
    peak = 0.0
    for _ in range(3):
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        assert lib.po_fp32_probe(blocks, iters, probe.data_ptr(), stream.cuda_stream) == 0
        p1.record(stream)
        torch.cuda.synchronize()
        peak = max(peak, blocks * 256 * iters * 16 / (p0.elapsed_time(p1) * 1e-3) / 1e12)
    mk = ("EH" if not far else "FF", not m_zero)
    # pair-packed forward and adjoint (near field: the fused adjoint)
    names = ["forward " + ("po_ff_kernel" if far else "po_pk_kernel"), "adjoint po_adj_pk_kernel"]
    flops = [FWD_FLOPS[mk], ADJ_FLOPS[mk]]
    kernels = []
    for j in range(kernels_per_step):
        lm = float(launch_ms[:, j].mean())
        ach = flops[j] * w["pairs"] / (lm * 1e-3) / 1e12 if flops[j] else None
        kernels.append({"kernel": names[j], "launch_ms": lm, "gpairs_per_s": w["pairs"] / (lm * 1e-3) / 1e9,
                        "flops_per_pair": flops[j], "achieved_tflops": ach,
                        "frac": ach / peak if ach else None})
    dom = max(kernels, key=lambda x: x["launch_ms"])
    traffic = None
    prof = ROOT / "profiles" / f"traffic_{w['name']}.json"
    if prof.exists():   # DRAM bytes per launch from an ncu capture, per kernel
        traffic = json.loads(prof.read_text()).get("kernels", {}).get(dom["kernel"].split()[-1])
    step_flops = sum(f for f in flops[:kernels_per_step] if f)
    step_ms_kernels = float(launch_ms.sum(axis=1).mean())

    line = {
        "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded currents with the configuration's taper and phase noise; random cotangent)",
        "config": config_of(args.workload, args.scale, w["pairs"], ns=ns, nt=nt),
        "device": "gpu", "parallelism": f"replica per GPU x{world}",
        "precision": "FP32 bulk in packed FP32x2; separation, R and phase in split hi/lo form",
        "forward_gpairs_per_s": kernels[0]["gpairs_per_s"],
        "adjoint_gpairs_per_s": w["pairs"] / (sum(kk["launch_ms"] for kk in kernels[1:]) * 1e-3) / 1e9,
        "accuracy": {
            "against_reference_cpu": {
                "forward": acc_cpu, "adjoint": adj_cpu,
                "against": f"the reference's CPU FP64 path (oracle restatement, pinned to the reference's "
                           f"outputs) on {ncpu} random targets x all {ns} sources, the GPU step's own outputs "
                           f"(forward) and the GPU mixed adjoint over the same targets"},
            "against_fp64_gpu": {
                "forward": acc_gpu64, "adjoint": adj_acc,
                "against": f"plain FP64 GPU sum on {idx.size} random targets (all sources); plain FP64 GPU "
                           f"adjoint, all targets x one source in {fstep} ({nsf})"},
            "phase_on": "max |arg(got/ref)| over the E and H components whose magnitude is within 20 dB "
                        "(and 40 dB) of the sample's largest component; rel_l2 over every output row"},
        "fp64_gpu": {"value": fp64_rate, "unit": "Gpairs/s (fwd+adjoint step)", "speedup": value / world / fp64_rate,
                     "sample": f"all {nt} targets x one source in {fstep} ({nsf})"},
        "roofline": {"bound": "fp32", "kernel": dom["kernel"], "achieved": dom["achieved_tflops"], "peak": peak,
                     "unit": "TFLOP/s", "frac": dom["frac"], "traffic": traffic,
                     "flops_per_pair": dom["flops_per_pair"],
                     "step_frac": step_flops * w["pairs"] / (step_ms_kernels * 1e-3) / 1e12 / peak,
                     "kernels": kernels,
                     "peak_source": "measured: po_fp32_probe FFMA chains on this GPU, best of 3"},
        "cpu_baseline": {"value": cpu_rate / 1e9, "unit": "Gpairs/s", "cores": threads, "kind": "port",
                         "sample": f"{ncpu} random targets x {ns} sources, forward {cpu_tf:.1f} s + adjoint "
                                   f"{cpu_ta:.1f} s, FP64 oracle (the reference's algorithm)"},
        "e2e": {"value": e2e, "unit": "Gpairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "drop_in_forward": drop_in,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    if world > 1:
        torch.distributed.destroy_process_group()
    return line


def run_chain(args):
    """A chain workload (the perturbed-dish or the Cassegrain chain); see the module docstring."""
    import torch
    from pypo_gb300 import build as B
    B.build()
    from pypo_gb300 import autograd as A, engine

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    c, stages, refl, disp0 = chain_config(args.workload, args.scale)
    k = c["k"]
    T = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    keys = sorted({sk for _, sk, _, _ in stages} | {tk for _, _, _, tk in stages})
    n = {key: c[key].shape[1] for key in keys}
    stage_pairs = [n[sk] * n[tk] for _, sk, _, tk in stages]
    pairs = sum(stage_pairs)
    nff = n[stages[-1][3]]
    cot_np = np.random.default_rng(7).standard_normal((12, nff))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def forward_backward(cc, dv, precision, ct):
        """Forward chain and backward pass; dv: reflector -> displacement tensor (requires grad)."""
        pts = {key: torch.tensor(np.ascontiguousarray(cc[key]), device=dev) for key in keys}
        cur = torch.tensor(np.ascontiguousarray(cc["feed_cur"]), device=dev)
        for mode, sk, gk, tk in stages:
            cur = A.propagate(mode, pts[sk], cur, *cc[gk], pts[tk], k, ds=dv.get(sk),
                              dt=dv.get(tk) if mode != "FF" else None, precision=precision)
        (cur * ct).sum().backward()
        return cur

    dvars = {r: torch.tensor(disp0[r], device=dev, requires_grad=True) for r in refl}
    cot = T(cot_np)

    def step():
        flush.zero_()
        for v in dvars.values():
            v.grad = None
        forward_backward(c, dvars, "mixed", cot)

    for _ in range(args.warmup):
        step()
    # kernel launches of one step: every device call of the chain reports its own
    launches = [0]
    real_fwd, real_adj = engine.propagate_dev, engine.adjoint_dev

    def counted(fn):
        def wrap(*a, **kw):
            r = fn(*a, **kw)
            launches[0] += engine.last_launches()
            return r
        return wrap
    engine.propagate_dev, engine.adjoint_dev = counted(real_fwd), counted(real_adj)
    step()
    engine.propagate_dev, engine.adjoint_dev = real_fwd, real_adj
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    if world > 1:
        from pypo_gb300.dist import max_over_ranks
        ms = max_over_ranks(ms)
    value = world * pairs * args.steps / (ms * 1e-3) / 1e9
    g_auto = {r: v.grad.cpu().numpy() for r, v in dvars.items()}

    # ---- e2e: host buffers through the C-ABI, chain rule stage by stage; every
    # host buffer (inputs, each stage's output, each stage's gradients) is
    # page-locked and allocated once, as a user of the C-ABI would
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    pinned_empty = lambda *shape: torch.empty(shape, dtype=torch.float64).pin_memory().numpy()
    host = {key: pinned(c[key]) for key in keys}
    for r in refl:                                   # displaced reflector points (normals, areas frozen)
        host[r][:3] += disp0[r][None, :] * host[r][3:6]
    feed_cur = pinned(c["feed_cur"])
    cot_h = pinned(cot_np)
    stage_out = [pinned_empty(engine.n_out(mode), n[tk]) for mode, _, _, tk in stages]
    stage_grad = [{"cur": pinned_empty(12, n[sk]), "ds": pinned_empty(n[sk]), "dt": pinned_empty(n[tk])}
                  for _, sk, _, tk in stages]
    io_bytes = []

    def host_step():
        curs = [feed_cur]
        for j, (mode, sk, gk, tk) in enumerate(stages[:-1]):
            curs.append(engine.propagate(mode, host[sk], curs[-1], *c[gk], host[tk], k, out=stage_out[j]))
        mode, sk, gk, tk = stages[-1]
        engine.propagate(mode, host[sk], curs[-1], *c[gk], host[tk], k, out=stage_out[-1])
        grads = {r: np.zeros(n[r]) for r in refl}
        ct = cot_h
        b_in = b_out = 0
        for i in range(len(stages) - 1, -1, -1):
            mode, sk, gk, tk = stages[i]
            want = (("cur",) if i > 0 else ()) + (("ds",) if sk in refl else ()) + \
                (("dt",) if tk in refl and mode != "FF" else ())
            g = engine.adjoint(mode, host[sk], curs[i], *c[gk], host[tk], k, ct, want=want, out=stage_grad[i])
            if sk in refl:
                grads[sk] += g["ds"]
            if tk in refl and mode != "FF":
                grads[tk] += g["dt"]
            b_in += 8 * (host[sk].size + curs[i].size + host[tk].size + ct.size)
            b_out += 8 * sum(v.size for v in g.values() if v is not None)
            ct = g.get("cur")
        if not io_bytes:
            fwd_in = sum(8 * (host[sk].size + curs[j].size + host[tk].size) for j, (_, sk, _, tk) in enumerate(stages))
            fwd_out = sum(8 * x.size for x in curs[1:]) + 8 * 12 * nff
            io_bytes.extend([fwd_in + b_in, fwd_out + b_out])
        return grads

    g_host = host_step()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        host_step()
    e2e_s = (time.perf_counter() - t0) / max(1, args.steps)
    e2e = pairs / e2e_s / 1e9
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    host_vs_autograd = max(rel(g_host[r], g_auto[r]) for r in refl)

    # ---- FP64 GPU chain: each stage's forward + adjoint on a subsample, combined by
    # pairs; every s-th source and t-th target with >= 65536 of each kept where a
    # stage has that many (the FP64 kernels run one thread per source or target)
    fp64_s = 0.0
    for (mode, skey, gkey, tkey), sp in zip(stages, stage_pairs):
        s_step, t_step = max(1, n[skey] // 65536), max(1, n[tkey] // 65536)
        src_sub = np.ascontiguousarray(c[skey][:, ::s_step])
        tgt_sub = np.ascontiguousarray(c[tkey][:, ::t_step])
        cur_sub = np.random.default_rng(1).standard_normal((12, src_sub.shape[1]))
        s_t, c_t, t_t = T(src_sub), T(cur_sub), T(tgt_sub)
        nts = tgt_sub.shape[1]
        cot_t = T(np.random.default_rng(2).standard_normal((12, nts)))
        gcur = torch.empty((12, src_sub.shape[1]), dtype=torch.float64, device=dev)
        gs = torch.empty(src_sub.shape[1], dtype=torch.float64, device=dev)
        gt = None if mode == "FF" else torch.empty(nts, dtype=torch.float64, device=dev)
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        engine.propagate_dev(mode, s_t, c_t, -1, 0, 0, t_t, k, precision="fp64")
        engine.adjoint_dev(mode, s_t, c_t, -1, 0, 0, t_t, k, cot_t, precision="fp64", grad_cur=gcur, grad_ds=gs,
                           grad_dt=gt)
        q1.record(stream)
        torch.cuda.synchronize()
        rate = src_sub.shape[1] * nts / (q0.elapsed_time(q1) * 1e-3)
        fp64_s += sp / rate
    fp64_rate = pairs / fp64_s / 1e9

    # ---- accuracy: the mixed chain against the FP64 chain at scale 0.2
    cs, _, _, ds0 = chain_config(args.workload, 0.2)
    ct_s = T(np.random.default_rng(3).standard_normal((12, cs[stages[-1][3]].shape[1])))
    outs = {}
    for precision in ("fp64", "mixed"):
        dv = {r: torch.tensor(ds0[r], device=dev, requires_grad=True) for r in refl}
        ff = forward_backward(cs, dv, precision, ct_s)
        outs[precision] = (ff.detach().cpu().numpy(), {r: v.grad.cpu().numpy() for r, v in dv.items()})
    acc = {"ff_rel_l2": rel(outs["mixed"][0], outs["fp64"][0])}
    for r in refl:
        acc[f"grad_{r[:-1]}_rel_l2"] = rel(outs["mixed"][1][r], outs["fp64"][1][r])
    # the perturbed-dish chain's gradient against finite differences, at full size
    grad_fd = None
    if args.workload == "dish_chain" and args.scale == 1.0:
        grad_fd = dish_chain_fd(c, dvars["dish7"].grad.detach().cpu().numpy(), cot_np, k)

    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    ws = chain_stage_workloads(c, stages)
    crng = np.random.default_rng(123)
    frac = cpu_chain_fraction(ws, args.cpu_sample_s * 0.6, threads, crng)
    cpu_pairs, cpu_s, cpu_parts = cpu_chain_step(ws, frac, threads, crng)
    line = {
        "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (Gaussian feed of the configuration; random cotangent on the far field)",
        "config": config_of(args.workload, args.scale, pairs, stage_pairs=stage_pairs),
        "device": "gpu", "parallelism": f"replica per GPU x{world}",
        "accuracy": dict(acc, against="FP64 GPU chain, configuration at scale 0.2"),
        **({"gradient_vs_finite_differences": grad_fd} if grad_fd else {}),
        "fp64_gpu": {"value": fp64_rate, "unit": "Gpairs/s (chain fwd+adjoint)", "speedup": value / world / fp64_rate,
                     "sample": "each stage timed on every s-th source x every t-th target (>= 65536 of each where "
                               "available), combined by pairs"},
        "e2e": {"value": e2e, "unit": "Gpairs/s", "h2d_bytes_per_step": io_bytes[0], "d2h_bytes_per_step": io_bytes[1],
                "path": "po_run_d / po_adjoint_d per stage from page-locked host arrays, chain rule on the host",
                "host_vs_autograd_grad_rel": host_vs_autograd},
        "cpu_baseline": {"value": cpu_pairs / cpu_s / 1e9, "unit": "Gpairs/s", "cores": threads,
                         "kind": "port", "sample": "per stage " + "; ".join(cpu_parts) +
                         f" (a fraction {frac:.2e} of every stage's targets), forward + adjoint, FP64 oracle"},
        "gpu_launches": launches[0] * args.steps, "clocks": clocks,
    }
    return line

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dish_eh",
                    choices=["dish_eh", "dish_ff", "feed_dish_jm", "cassegrain", "dish_chain"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink both grids (profiling runs only; the bench line is the full size)")
    ap.add_argument("--cpu-seconds", type=float, default=90.0,
                    help="reference arm: host time of the whole run (warm-up and timed steps), which sizes "
                         "each step's target sample")
    ap.add_argument("--no-others", action="store_true",
                    help="default run: skip the shorter runs of the far-field and Cassegrain configurations "
                         "that the line carries under other_configs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    args.cpu_sample_s = 10.0
    if args.impl == "reference":
        run_reference(args)
        return
    line = run_chain(args) if args.workload in CHAINS else run_ours(args)
    if line is None:
        return
    rank, world, _ = dist_env()
    if args.workload == "dish_eh" and args.scale == 1.0 and world == 1 and not args.no_others:
        # the far-field (1.6e11 pairs) and Cassegrain-chain (2.1e11 pairs)
        # configurations, each measured the same way in a shorter run
        others = {}
        for name in ("dish_ff", "cassegrain"):
            sub = argparse.Namespace(**vars(args))
            sub.workload, sub.steps, sub.warmup, sub.cpu_sample_s = name, min(args.steps, 3), 3, 4.0
            o = run_chain(sub) if name in CHAINS else run_ours(sub)
            if o is not None:
                o.pop("metric", None)
                others[name] = o
        line["other_configs"] = others
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
