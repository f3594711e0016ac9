"""Benchmark of the transient Newton hot path on GB300.

Workload (default): the CMOS ring oscillator of 10,001 MOSFET level-1
inverter stages (20,002 transistors, 10,003 unknowns), VDD 1.8 V, 5 fF loads,
a 1 ns PWL kick, .TRAN 0 20n with 5 ps maximum step, FP64 throughout.

A bench step is one window of WINDOW accepted transient time steps of that
circuit, advanced through the device-resident Newton/OneStep loop
(xg_tran_advance).  value = accepted transient steps per second over the
timed windows (L2 flushed between windows with a 256 MiB write), summed over
ranks for --gpus N (independent replicas: the circuit is one coupled system).

e2e = the same metric through the full C-ABI call a user makes with host
buffers: context creation, netlist upload, operating point, analysis, the
transient windows and the copy of the probe waveforms back to the host.

--impl reference times the CPU FP64 restatement of the reference's
algorithms (oracle/, single thread: the reference path is serial) on the same
workload, metric and windows.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "transient steps/s (device evals/s alongside), plain GPU path, FP64"
UNIT = "steps/s"
WINDOW = 200          # accepted time steps per bench step
CPU_SAMPLE_STEPS = 1500


def _peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _clock_sampler(path):
    try:
        return subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=open(path, "w"), stderr=subprocess.DEVNULL)
    except Exception:
        return None


def _clock_summary(path, device_index):
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    try:
        for line in open(path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(device_index):
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
    except FileNotFoundError:
        pass
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons)}


def _workload(stages):
    from xyce_gb300 import netlist as N
    nl = N.ring_oscillator(stages)
    probes = [nl.names["n1"], nl.names[f"n{stages // 2}"]]
    return nl, probes


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """CPU restatement of the reference path, single thread, same windows."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build(with_reference=False)
    import numpy as np
    nl, probes = _workload(args.stages)
    o = oracle.Oracle(nl)
    # one run of (warmup + steps) windows; the wall clock at every accepted
    # step gives each window's time
    tran = nl.tran
    total = args.warmup + args.steps
    tran.max_steps = total * WINDOW
    wall = np.zeros(total * WINDOW)
    _, _, st = o.transient(tran, probes=probes, cap=8, wall_log=wall)
    done = st["accepted"]
    first = args.warmup * WINDOW
    secs = wall[done - 1] - wall[first - 1]
    steps = done - first
    value = steps / secs
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"ring_oscillator_{args.stages}_stages", "window_steps": WINDOW,
                       "mosfets": 2 * args.stages},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{args.steps} windows of {WINDOW} accepted steps after "
                                       f"{args.warmup} warm-up windows, CPU FP64 restatement of "
                                       "the reference algorithms (oracle/), one thread"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(stages, n_steps):
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build(with_reference=False)
    nl, probes = _workload(stages)
    o = oracle.Oracle(nl)
    nl.tran.max_steps = n_steps
    t0 = time.perf_counter()
    _, _, st = o.transient(nl.tran, probes=probes, cap=8)
    dt = time.perf_counter() - t0
    return {"value": st["accepted"] / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {st['accepted']} accepted steps of the same circuit from its "
                      f"operating point ({dt:.1f} s), CPU FP64 restatement (oracle/), one thread"}


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    import xyce_gb300 as xg
    if not os.path.exists(xg.LIB_PATH):
        xg.build()
    hbm_peak, peak_kind = _peaks()
    nl, probes = _workload(args.stages)

    # ---- device-resident windows -----------------------------------------
    circ = xg.Circuit(nl, device=dev)
    circ.tran_start(probes=probes, cap=16)
    stream = torch.cuda.ExternalStream(xg.lib().xg_get_stream(circ.h))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    for _ in range(args.warmup):
        circ.tran_advance(WINDOW)
    st0 = circ.tran_results()[3]
    info = circ.lu_info()
    clk_path = os.path.join(HERE, "gpurun_out", f"clocks_rank{rank}.csv") \
        if os.path.isdir(os.path.join(HERE, "gpurun_out")) else f"/tmp/xg_clocks_{os.getpid()}.csv"
    sampler = _clock_sampler(clk_path)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms_total = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        circ.tran_advance(WINDOW)
        e1.record(stream)
        e1.synchronize()
        ms_total += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    if sampler:
        sampler.terminate()
        sampler.wait()
    st1 = circ.tran_results()[3]
    steps_done = st1["accepted"] - st0["accepted"]
    ticks = st1["ticks"] - st0["ticks"]
    evals = st1["device_evals"] - st0["device_evals"]
    local_vals = torch.tensor([ms_total, float(steps_done), float(evals)], dtype=torch.float64,
                              device=f"cuda:{dev}")
    if world > 1:
        t = local_vals.clone()
        torch.distributed.all_reduce(t[:1], op=torch.distributed.ReduceOp.MAX)
        s = local_vals.clone()
        torch.distributed.all_reduce(s, op=torch.distributed.ReduceOp.SUM)
        ms_max, steps_all, evals_all = float(t[0]), float(s[1]), float(s[2])
    else:
        ms_max, steps_all, evals_all = ms_total, float(steps_done), float(evals)
    value = steps_all / (ms_max / 1e3)
    kernels_per_tick = 11 + info["factor_levels"] + info["lsolve_levels"] + info["usolve_levels"]
    gpu_launches = int(ticks * kernels_per_tick)
    circ.tran_end()

    # ---- roofline of the device-evaluation kernel (MOSFET eval + stamp) ----
    roof = None
    if rank == 0:
        n = circ.n
        z = lambda k: torch.zeros(max(1, k), dtype=torch.float64, device=f"cuda:{dev}")
        x = torch.full((n,), 0.9, dtype=torch.float64, device=f"cuda:{dev}")
        stac, stan, stoc, ston = z(circ.nsta), z(circ.nsta), z(circ.nsto), z(circ.nsto)
        for _ in range(5):
            circ.update_state(x, stac, stoc, stan, ston, newton_iter=1)
        reps = 200
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            circ.update_state(x, stac, stoc, stan, ston, newton_iter=1)
        e1.record(stream)
        e1.synchronize()
        us = e0.elapsed_time(e1) * 1e3 / reps
        nm = 2 * args.stages
        # per instance: reads 4 node indices, model index, circuit index (24 B),
        # beta + vbi (16 B), 4 node voltages (32 B), 5 history stores (40 B);
        # writes 6 stores + 8 states (112 B) and 47 stamp slots (376 B): 600 B
        bytes_per_inst = 24 + 16 + 32 + 40 + 112 + 376
        achieved = bytes_per_inst * nm / (us * 1e-6) / 1e9
        traffic = None
        prof = os.path.join(HERE, "profiles", "k_mos1_ring10001.traffic.json")
        if os.path.exists(prof):
            try:
                traffic = json.load(open(prof)).get("dram_bytes_per_launch")
            except Exception:
                traffic = None
        roof = {"kernel": "k_mos1 (MOSFET-1 evaluation + stamp, separate dF/dQ slots)",
                "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": bytes_per_inst * nm, "launch_us": us}
    circ.close()

    # ---- end to end through the C-ABI with host buffers --------------------
    e2e = None
    if rank == 0:
        tr = nl.tran
        tr.max_steps = (args.warmup + args.steps) * WINDOW
        a = nl.arrays()
        h2d = sum(v.nbytes for k, v in a.items() if hasattr(v, "nbytes"))
        h2d += sum(x.nbytes for k in ("res", "cap", "vsrc", "isrc", "diode", "mos1") for x in a[k])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c2 = xg.Circuit(nl, device=dev)
        counts, tt, vv, st = c2.transient(tr, probes=probes, cap=tr.max_steps + 8)
        dt = time.perf_counter() - t0
        c2.close()
        d2h = int(counts[0]) * (8 + 8 * len(probes))
        nsteps = args.warmup + args.steps
        e2e = {"value": st["accepted"] / dt, "unit": UNIT,
               "h2d_bytes_per_step": h2d / nsteps, "d2h_bytes_per_step": d2h / nsteps,
               "seconds": dt, "accepted": st["accepted"]}
        tr.max_steps = 0

    if rank == 0:
        cpu = cpu_baseline(args.stages, args.cpu_steps) if args.cpu_steps > 0 else None
        clocks = _clock_summary(clk_path, dev)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"ring_oscillator_{args.stages}_stages",
                           "mosfets": 2 * args.stages, "unknowns": n,
                           "window_steps": WINDOW, "tran": "0 20n, hmax 5p",
                           "l2": "flushed between windows (256 MiB write)",
                           "parallelism": f"replicas x{world}"},
                "device_evals_per_s": evals_all / (ms_max / 1e3),
                "newton_iters_per_step": (st1["newton_iters"] - st0["newton_iters"]) / max(1, steps_done),
                "ticks": ticks, "gpu_launches": gpu_launches,
                "lu": info, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--stages", type=int, default=10001)
    ap.add_argument("--cpu-steps", type=int, default=CPU_SAMPLE_STEPS)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
