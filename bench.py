#!/usr/bin/env python3
"""Benchmark of the physical-optics integrator on one GB300 per rank.

Workload (default `dish_eh`): paraboloid D 1000 mm, f 500 mm, uv 501x501
(251,001 source points, lambda 1 mm) radiating to a 301x301 focal-plane grid
(90,601 targets), mode EH: 2.27e10 source-target pairs per step. Inputs are
seeded synthetic currents with the configuration's taper and phase noise.

A step is one mixed-precision forward propagation of the whole workload.
  value  pairs / s with inputs resident on the device (po_run_dev)
  e2e    the same through the host-buffer C-ABI (po_run_d): H2D of the
         step's inputs from pinned memory, the propagation, D2H of the fields
Also reported: accuracy of the step's output against the plain FP64 GPU sum
(sampled targets), the FP64 GPU sum's own pair rate, the FP32 roofline of the
main kernel (CUDA events around every launch on its stream), the clocks seen
during the timed region, and the FP64 CPU oracle on a bounded sample.

`--impl reference` times the reference's CPU path (its compiled library when
it loads here, else the oracle's C restatement of it) on the same workload.

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
#: algorithmic FP32 flops per pair (FMA = 2), split-precision overhead not counted
FLOPS_PER_PAIR = {("EH", True): 234, ("EH", False): 140, ("FF", True): 61, ("FF", False): 37}


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


def cpu_oracle_rate(w, seconds, threads, impl_ref=False):
    """Pairs/s of the FP64 CPU path on a target subsample sized to ~`seconds`."""
    from oracle import oracle as O
    rng = np.random.default_rng(123)
    nt = w["t7"].shape[1]
    ns = w["s7"].shape[1]

    def run(n):
        idx = np.sort(rng.choice(nt, size=n, replace=False))
        t0 = time.perf_counter()
        O.run(w["mode"], w["s7"], w["cur"], w["gmode"], w["ncx"], w["ncy"], w["t7"], w["k"],
              1.0, -1.0, nthreads=threads, tidx=idx)
        return time.perf_counter() - t0

    n0 = max(threads, 16)
    dt = run(n0)
    n = int(min(nt, max(n0, n0 * seconds / max(dt, 1e-3))))
    dt = run(n)
    return ns * n / dt, n, dt


def reference_lib_rate(w, seconds, threads):
    """Pairs/s of the reference's own compiled CPU library on leading target rows."""
    from oracle import oracle as O
    ref = O.Reference()
    tgt = dict(w["tgt"])
    ncy = int(tgt["gridsize"][1])
    ncx = int(tgt["gridsize"][0])
    lx = np.asarray(tgt["lims_x"], dtype=float)
    dx = (lx[1] - lx[0]) / (ncx - 1)
    ns = w["s7"].shape[1]

    def run(rows):
        sub = dict(tgt, gridsize=np.array([rows, ncy]), lims_x=np.array([lx[0], lx[0] + (rows - 1) * dx]))
        t0 = time.perf_counter()
        ref.propagate(w["mode"], w["src"], sub, w["cur"], w["k"], 1.0, -1.0, nthreads=threads)
        return time.perf_counter() - t0

    r0 = 2
    dt = run(r0)
    rows = int(min(ncx, max(r0, r0 * seconds / max(dt, 1e-3))))
    dt = run(rows)
    return ns * rows * ncy / dt, rows * ncy, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from pypo_gb300 import configs
    w = configs.WORKLOADS[args.workload]()
    threads = os.cpu_count() or 1
    per_step = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    kind = "port"
    try:
        from oracle import oracle as O
        if O.REF_PATH.exists():
            O.Reference()
            kind = "reference"
    except OSError:
        kind = "port"
    rates, sample = [], ""
    for i in range(args.warmup + args.steps):
        if kind == "reference":
            rate, n, dt = reference_lib_rate(w, per_step, threads)
            sample = f"{n} targets (leading grid rows) x {w['s7'].shape[1]} sources per step"
        else:
            rate, n, dt = cpu_oracle_rate(w, per_step, threads)
            sample = f"{n} random targets x {w['s7'].shape[1]} sources per step"
        if i >= args.warmup:
            rates.append(rate)
    value = float(np.mean(rates)) / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": w["pairs"] / (value * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": w["name"], "desc": w["desc"], "pairs_per_step": w["pairs"],
                                            "device": "cpu", "threads": threads},
            "cpu_baseline": {"value": value, "unit": "Gpairs/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    w = configs.WORKLOADS[args.workload]()
    mode, k = w["mode"], w["k"]
    m_zero = not np.any(w["cur"][6:])
    ns, nt = w["s7"].shape[1], w["t7"].shape[1]
    s7 = torch.tensor(w["s7"], device=dev)
    cur = torch.tensor(w["cur"], device=dev)
    t7 = torch.tensor(w["t7"], device=dev)
    out = torch.empty((engine.n_out(mode), nt), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream(dev)

    def step():
        flush.zero_()
        engine.propagate_dev(mode, s7, cur, w["gmode"], w["ncx"], w["ncy"], t7, k, 1.0, -1.0, "mixed",
                             m_zero=m_zero, out=out, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches_per_step = engine.last_launches()
    engine.timing_enable(args.steps)
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
    main_ms = engine.timing_collect()
    engine.timing_enable(0)
    assert engine.device_error(stream) == 0, "a kernel reported a wait timeout"
    if world > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = w["pairs"] * args.steps * world / (ms * 1e-3) / 1e9

    # ---- end to end through the host-buffer C-ABI (pinned host memory)
    s7_h = torch.from_numpy(np.ascontiguousarray(w["s7"])).pin_memory()
    cur_h = torch.from_numpy(np.ascontiguousarray(w["cur"])).pin_memory()
    t7_h = torch.from_numpy(np.ascontiguousarray(w["t7"])).pin_memory()
    out_h = torch.empty((engine.n_out(mode), nt), dtype=torch.float64).pin_memory()

    def step_e2e():
        flush.zero_()
        engine.propagate(mode, s7_h.numpy(), cur_h.numpy(), w["gmode"], w["ncx"], w["ncy"], t7_h.numpy(), k,
                         1.0, -1.0, "mixed", out=out_h.numpy())

    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = w["pairs"] * args.steps / e2e_s / 1e9 * world
    h2d = (7 + 12) * ns * 8 + 7 * nt * 8
    d2h = engine.n_out(mode) * nt * 8
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- accuracy of the step's output against the plain FP64 GPU sum
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(nt, size=min(1024, nt), replace=False))
    t7s = torch.tensor(np.ascontiguousarray(w["t7"][:, idx]), device=dev)
    ref = engine.propagate_dev(mode, s7, cur, w["gmode"], w["ncx"], w["ncy"], t7s, k, 1.0, -1.0, "fp64")
    got = out[:, idx]
    torch.cuda.synchronize()
    ref_n, got_n = ref.cpu().numpy(), got.cpu().numpy()
    rel_l2 = float(np.linalg.norm(got_n - ref_n) / np.linalg.norm(ref_n))
    rc = ref_n[0:3] + 1j * ref_n[3:6]
    gc = got_n[0:3] + 1j * got_n[3:6]
    sel = np.abs(rc) >= np.abs(rc).max() * 0.1
    max_phase = float(np.abs(np.angle(gc[sel] / rc[sel])).max())

    # ---- the FP64 GPU sum's own pair rate (all targets, every 16th source)
    sub = slice(0, ns, 16)
    s7f = s7[:, sub].contiguous()
    curf = cur[:, sub].contiguous()
    nsf = s7f.shape[1]
    outf = torch.empty_like(out)
    engine.propagate_dev(mode, s7f, curf, -1, 0, 0, t7, k, 1.0, -1.0, "fp64", out=outf)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    engine.propagate_dev(mode, s7f, curf, -1, 0, 0, t7, k, 1.0, -1.0, "fp64", out=outf)
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_rate = nsf * nt / (e0.elapsed_time(e1) * 1e-3) / 1e9

    # ---- FP32 roofline of the main kernel
    lib = load()
    probe = torch.empty(152 * 8 * 256, dtype=torch.float32, device=dev)
    blocks, iters = probe.numel() // 256, 100000
    best = 0.0
    for _ in range(3):
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        rc_ = lib.po_fp32_probe(blocks, iters, probe.data_ptr(), stream.cuda_stream)
        p1.record(stream)
        torch.cuda.synchronize()
        assert rc_ == 0
        best = max(best, blocks * 256 * iters * 16 / (p0.elapsed_time(p1) * 1e-3) / 1e12)
    fpp = FLOPS_PER_PAIR[(mode, not m_zero)]
    launch_ms = float(np.mean(main_ms)) if main_ms else float("nan")
    achieved = fpp * w["pairs"] / (launch_ms * 1e-3) / 1e12
    traffic = None
    prof = ROOT / "profiles" / f"traffic_{w['name']}.json"
    if prof.exists():
        traffic = json.loads(prof.read_text()).get("bytes_per_launch")

    # ---- FP64 CPU oracle on a bounded sample
    threads = os.cpu_count() or 1
    cpu_rate, cpu_n, cpu_dt = cpu_oracle_rate(w, 10.0, threads)

    line = {
        "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded currents with the configuration's taper and phase noise)",
        "config": {"workload": w["name"], "desc": w["desc"], "ns": ns, "nt": nt, "pairs_per_step": w["pairs"],
                   "step": "forward propagation (adjoint not in this step)",
                   "precision": "FP32 bulk; separation, R and phase in split hi/lo form",
                   "l2": "flushed between steps (256 MB write inside the timed loop)",
                   "parallelism": f"replica per GPU x{world}"},
        "accuracy": {"rel_l2": rel_l2, "max_phase_rad": max_phase,
                     "against": f"plain FP64 GPU sum on {idx.size} random targets (all sources)",
                     "phase_on": "E components within 20 dB of the sampled peak"},
        "fp64_gpu": {"value": fp64_rate, "unit": "Gpairs/s", "speedup": value / world / fp64_rate,
                     "sample": f"all {nt} targets x every 16th source ({nsf})"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": best, "unit": "TFLOP/s",
                     "frac": achieved / best, "traffic": traffic,
                     "flops_per_pair": fpp, "kernel": "po_main_kernel (near field, M=0)" if mode == "EH" else
                     "po_main_kernel", "launch_ms": launch_ms,
                     "peak_source": "measured: po_fp32_probe FFMA chains on this GPU, best of 3"},
        "cpu_baseline": {"value": cpu_rate / 1e9, "unit": "Gpairs/s", "cores": threads, "kind": "port",
                         "sample": f"{cpu_n} random targets x {ns} sources ({cpu_dt:.1f} s), FP64 oracle"},
        "e2e": {"value": e2e, "unit": "Gpairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dish_eh", choices=["dish_eh", "dish_ff"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
