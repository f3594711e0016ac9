"""Benchmark of the transient Newton hot path on GB300.

Workloads (--workload):
  mc    (default) batched Monte-Carlo form: 4,096 MOSFET level-1 ring
        oscillators in one netlist, odd stage counts uniform in [11, 301]
        (~1.28 M transistors, ~0.64 M unknowns), per-instance VTO ~ N(+-0.5, 0.03),
        KP ~ N(nominal, 5 %), load C ~ U[3, 7] fF; .TRAN 0 10n; every ring keeps
        its own step control; FP64 device evaluation, residual and LU.
  ring  plain GPU path: one ring oscillator of 10,001 MOSFET level-1 inverter
        stages (20,002 transistors), .TRAN 0 20n with 5 ps maximum step.

A bench step is one window in which every circuit accepts WINDOW more
transient steps, advanced by the device-resident Newton/OneStep loop
(xg_tran_advance).  value = accepted transient steps per second summed over
all circuits of the timed windows (inputs > L2: the device state of the mc
workload is ~2 GB, and L2 is flushed with a 256 MiB write before every
window), summed over ranks for --gpus N (independent replicas).

e2e = the same metric through the full C-ABI call a user makes with host
buffers (xg_transient): context creation, upload of the netlist's flat host
arrays (the C-ABI's input, built before the timed region), operating point,
analysis, the transient windows and the copy of the probe waveforms back.

The FP32-LU + FP64 iterative-refinement form is timed on the same workload
in the same run (key "forms"), and so is, for mc, the plain unbatched path: a
sample of the rings run one at a time, each in its own context.

--impl reference times the CPU FP64 restatement of the reference's
algorithms (oracle/) on the same metric: for mc, a sample of the same rings
run one per process on every host core; for ring, the whole circuit on one
thread (the reference path is serial).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "transient steps/s (device evals/s alongside), FP64"
UNIT = "steps/s"
WORKLOADS = {
    # mc: the CPU arm times each sampled ring's accepted steps 151..650, the
    # region the GPU arm times (3 warm-up windows of 50 steps, then 10 timed)
    "mc": dict(window=50, cpu_steps=500, cpu_warm=150, cpu_rings=64),
    "ring": dict(window=200, cpu_steps=1500, cpu_rings=0),
    "grid": dict(window=10, cpu_steps=6, cpu_rings=0),
    "dag": dict(window=10, cpu_steps=20, cpu_rings=0),
}


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


def _workload(name, rings=4096):
    from xyce_gb300 import netlist as N
    if name == "mc":
        nl = N.monte_carlo_rings(rings)
        probes = [nl.names[f"c{i}.n1"] for i in (0, 1, 2, 3)]
        desc = dict(workload=f"monte_carlo_rings_{rings}", circuits=rings, mosfets=len(nl.mos1),
                    stages="odd U[11,301]", tran="0 10n, hmax 5p")
    elif name == "grid":
        nl = N.power_grid(500)
        probes = [nl.names["center"]]
        desc = dict(workload="power_grid_500x500", circuits=1, unknowns_hint="250k nodes, 2,000 PWL sinks",
                    tran="0 2n, step 1p")
    elif name == "dag":
        nl = N.bsim4_logic_dag(50000)
        probes = [nl.names["g10"], nl.names["g1000"]]
        desc = dict(workload="bsim4_logic_dag_50000", circuits=1, bsim4=len(nl.bsim4), tran="0 5n, hmax 5p")
    else:
        nl = N.ring_oscillator(10001)
        probes = [nl.names["n1"], nl.names["n5000"]]
        desc = dict(workload="ring_oscillator_10001_stages", circuits=1, mosfets=len(nl.mos1),
                    tran="0 20n, hmax 5p")
    return nl, probes, desc


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---- CPU: the oracle (CPU FP64 restatement of the reference algorithms) ----
_BATCH = None


def _cpu_init():
    global _BATCH
    sys.path.insert(0, HERE)
    from xyce_gb300 import netlist as N
    _BATCH = N.monte_carlo_rings(4096)


def _cpu_ring_task(args):
    """One Monte-Carlo ring run alone by the oracle: its accepted steps
    n_warm+1 .. n_warm+n_steps, timed from the per-step wall-clock log
    (the operating point and the first n_warm steps are not timed)."""
    idx, n_warm, n_steps = args
    import numpy as np
    import oracle
    from xyce_gb300 import netlist as N
    nl = N.extract_circuit(_BATCH, idx)
    nl.tran.max_steps = n_warm + n_steps
    wall = np.zeros(n_warm + n_steps + 1)
    _, _, st = oracle.Oracle(nl).transient(nl.tran, probes=[0], cap=8, wall_log=wall)
    k = int(st["accepted"])
    if k <= n_warm:
        return 0, 0.0
    return k - n_warm, float(wall[k - 1] - wall[n_warm - 1])


def cpu_mc(n_rings, n_warm, n_steps, cores):
    """Aggregate steps/s of the oracle on a sample of the batch's rings, one
    ring per process on `cores` processes (spawned: no state shared with a
    CUDA context): the per-core rate over the timed steps of every sampled
    ring (sum of steps / sum of their seconds) times the cores, the rings
    being independent."""
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build(with_reference=False)
    tasks = [(int(i), n_warm, n_steps) for i in range(0, 4096, max(1, 4096 // n_rings))][:n_rings]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_cpu_init) as pool:
        pool.map(abs, range(cores))  # workers up and the batch built before the clock starts
        t0 = time.perf_counter()
        res = pool.map(_cpu_ring_task, tasks, chunksize=1)
        wall = time.perf_counter() - t0
    steps = sum(r[0] for r in res)
    secs = sum(r[1] for r in res)
    return cores * steps / secs, steps, secs, wall


def cpu_single(workload, n_steps):
    """Steps/s of the oracle on one circuit: its first n_steps accepted steps,
    timed from the first accepted step to the last (the operating point
    excluded).  Rings keep the LU's natural order (it fills little there);
    grids and logic DAGs use the minimum-degree order, as KLU orders them."""
    import numpy as np
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build(with_reference=False)
    nl, probes, _ = _workload(workload)
    nl.tran.max_steps = n_steps
    o = oracle.Oracle(nl)
    if workload in ("grid", "dag"):
        o.use_minimum_degree()
    wall = np.zeros(n_steps + 1)
    _, _, st = o.transient(nl.tran, probes=probes, cap=8, wall_log=wall)
    k = int(st["accepted"])
    dt = float(wall[k - 1] - wall[0])
    return (k - 1) / dt, k - 1, dt


def cpu_baseline(args):
    # Rings keep the LU's natural order: it fills little there, while a
    # minimum-degree order with threshold pivoting fills a long ring's
    # operating-point factors (5.7 s against 4 ms for 3,001 stages).
    w = WORKLOADS[args.workload]
    if args.workload == "mc":
        cores = os.cpu_count() or 1
        v, steps, secs, wall = cpu_mc(w["cpu_rings"], w["cpu_warm"], w["cpu_steps"], cores)
        a, b = w["cpu_warm"] + 1, w["cpu_warm"] + w["cpu_steps"]
        return {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"{w['cpu_rings']} rings of the same batch, accepted steps {a}..{b} of each (the "
                          f"steps the GPU arm times; {steps} timed steps, {secs:.1f} core-seconds, "
                          f"{wall:.1f} s wall with the untimed operating points and first {w['cpu_warm']} "
                          f"steps), CPU FP64 restatement (oracle/, LU in the ring's natural order), one ring "
                          f"per process on {cores} processes; rate = cores x timed steps / core-seconds"}
    v, steps, dt = cpu_single(args.workload, w["cpu_steps"])
    order = "the natural order" if args.workload == "ring" else "minimum-degree order"
    return {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} accepted steps of the same circuit after its first one ({dt:.1f} s), CPU FP64 "
                      f"restatement (oracle/, LU in {order}), one thread"}


def run_reference(args):
    """The reference algorithms on the CPU (the oracle port), same metric."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    nl, _, desc = _workload(args.workload, args.rings)
    cb = cpu_baseline(args)
    # a step of the GPU arm is one window: `window` accepted steps of every circuit
    step_units = WORKLOADS[args.workload]["window"] * nl.n_circuits
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * step_units / cb["value"],
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": desc,
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- GPU ----------------------------------------------------------------
SAMPLE_RINGS = 8          # rings of the mc batch whose waveforms are checked against the oracle
PROFILE_TICKS = 40        # ticks timed stage by stage for the rooflines
MOS1_ALG_BYTES = 712      # algorithmic bytes per MOSFET-1 evaluation + stamp, per-unit convention
MOS1_BYTES_CODE = 440     # bytes the transient-mode kernel reads (112) and writes (328) per instance
LU_BYTES_PER_NNZ = 12     # algorithmic bytes of a refactorization per nnz(L+U): value + index


def _sample(nl, workload):
    """(circuit, probe) pairs whose waveforms the oracle checks."""
    if workload == "mc":
        picks = [int(i * nl.n_circuits / SAMPLE_RINGS) for i in range(SAMPLE_RINGS)]
        return [(ci, nl.names[f"c{ci}.n1"]) for ci in picks]
    if workload == "ring":
        return [(0, nl.names["n1"]), (0, nl.names["n5000"])]
    return []  # grid, dag: the oracle's replay of a whole window takes minutes (parity: the GPU tests)


def _timed_windows(xg, nl, probes, dev, args, window, prec, flush, stream_of, cap=16, tune=None, form=None):
    import torch
    circ = xg.Circuit(nl, device=dev)
    circ.lu_set_precision(prec, 2)
    circ.lu_set_tuning(xg.TUNE_TIMED if tune is None else tune)
    circ.tran_set_form(xg.FORM_AUTO if form is None else form)
    if args.tail is not None:
        circ.tran_set_tail(args.tail)
    circ.tran_start(probes=probes, cap=cap)
    stream = stream_of(circ)
    for _ in range(args.warmup):
        circ.tran_advance(window)
    st0 = circ.tran_results()[3]
    torch.cuda.synchronize()
    ms = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        circ.tran_advance(window)
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    st1 = circ.tran_results()[3]
    return circ, ms, st0, st1


def _one_at_a_time(xg, nl, dev, window, stream_of, batched, sample=8, timed=4):
    """The plain (unbatched) GPU path on the same rings: a sample of `sample`
    rings spread over the batch, each alone in its own context, `timed`
    windows of `window` steps after 3 warm-up windows; steps/s = all accepted
    steps / all device time, i.e. the rate of running the batch one ring at a
    time."""
    import torch
    from xyce_gb300 import netlist as N
    steps, ms = 0, 0.0
    picks = [int(i * nl.n_circuits / sample) for i in range(sample)]
    for ci in picks:
        sub = N.extract_circuit(nl, ci)
        c = xg.Circuit(sub, device=dev)
        c.tran_start(probes=[0], cap=16)
        stream = stream_of(c)
        for _ in range(3):
            c.tran_advance(window)
        a0 = c.tran_results()[3]["accepted"]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(timed):
            c.tran_advance(window)
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        steps += c.tran_results()[3]["accepted"] - a0
        c.tran_end()
        c.close()
    rate = steps / (ms / 1e3)
    return {"one_ring_at_a_time": rate, "one_ring_at_a_time_sample": f"{sample} rings x {timed * window} steps",
            "batched_over_one_ring_at_a_time": batched / rate}


OTHER_CONFIGS = (
    # name, netlist builder, window (accepted steps per advance), timed windows
    ("c1_diode_ladder_1000", lambda N: N.diode_ladder(1000, seed=1), 200, 3),
    ("c2_ring_10001", lambda N: N.ring_oscillator(10001), 200, 3),
    ("c3_power_grid_200x200", lambda N: N.power_grid(200), 10, 3),
    ("c3_power_grid_500x500", lambda N: N.power_grid(500), 5, 2),
    ("c5_bsim4_logic_dag_50000", lambda N: N.bsim4_logic_dag(50000), 10, 3),
)


def _other_configs(xg, dev, flush, stream_of):
    """Steps/s of the plain FP64 path on the other single-circuit configs,
    timed like the headline (CUDA events on the context's stream around each
    advance, L2 flushed between advances, after one warm-up advance past the
    operating point): the full-size diode ladder, the 10,001-stage ring, the
    200x200 and 500x500 power grids and the 50k-transistor BSIM4 logic DAG."""
    import torch
    from xyce_gb300 import netlist as N
    out = {}
    for name, build, window, timed in OTHER_CONFIGS:
        try:
            nl = build(N)
            t0 = time.perf_counter()
            c = xg.Circuit(nl, device=dev)
            c.tran_start(probes=[0], cap=16)
            c.tran_advance(window)
            setup_s = time.perf_counter() - t0
            stream = stream_of(c)
            a0 = c.tran_results()[3]
            ms = 0.0
            for _ in range(timed):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                c.tran_advance(window)
                e1.record(stream)
                e1.synchronize()
                ms += e0.elapsed_time(e1)
            a1 = c.tran_results()[3]
            steps = a1["accepted"] - a0["accepted"]
            out[name] = {"steps_per_s": steps / (ms / 1e3), "steps": steps, "unknowns": c.n,
                         "newton_iters_per_step": (a1["newton_iters"] - a0["newton_iters"]) / max(1, steps),
                         "setup_and_first_window_s": setup_s}
            c.tran_end()
            c.close()
        except Exception as e:  # noqa: BLE001 - reported, not required
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def _learned_form(xg):
    """The learned-predictor form on the BSIM4 logic family: train on the
    plain runs of two 800-transistor DAGs (the network's own forward and
    backward kernels on the GPU), then run an unseen third DAG with the
    polynomial and with the learned predictor (TIMEINT reltol 1e-4, abstol
    1e-7); Newton iterations per step and accepted steps per second of
    each (wall time of the whole transient, operating point included)."""
    from xyce_gb300 import netlist as N
    from xyce_gb300 import predictor as P
    import numpy as np

    def fam(seed):
        nl = N.bsim4_logic_dag(800, 12, seed=seed, tstop=3e-9)
        nl.tran.reltol, nl.tran.abstol = 1e-4, 1e-7
        return nl

    Xs, Ys = [], []
    t0 = time.perf_counter()
    for seed in (21, 22):
        counts, t, v, p, probes, st = P.record(fam(seed), cap=4000)
        X, Y = P.dataset(counts, t, v, p, [len(probes)])
        Xs.append(X)
        Ys.append(Y)
    c = xg.Circuit(N.bsim4_inverter_chain(2))
    theta, norm, hist = P.train(c, np.concatenate(Xs), np.concatenate(Ys), iters=600, lr=3e-3, batch=200000)
    c.close()
    train_s = time.perf_counter() - t0
    test = fam(23)
    out = {"family": "bsim4_logic_dag_800, trained on seeds 21 and 22, run on seed 23",
           "train_loss_first_last": [float(hist[0]), float(hist[-1])], "record_and_train_s": train_s}
    for name, args in (("polynomial", ()), ("learned", (theta, norm))):
        a = time.perf_counter()
        _, _, _, st, ps = P.run(test, *args)
        dt = time.perf_counter() - a
        out[name] = {"newton_iters_per_step": st["newton_iters"] / max(1, st["accepted"]),
                     "steps_per_s_wall": st["accepted"] / dt, "accepted": st["accepted"]}
        if args:
            out[name]["learned_steps"] = ps["learned_steps"]
            out[name]["fallback_steps"] = ps["poly_steps"]
    return out


def _rooflines(circ, nl, window, hbm_peak, peak_kind, info, args):
    """Rooflines of the two dominant kernels of the tick, timed by the tick
    profiler (each stage of PROFILE_TICKS ticks of a new window launched on
    its own, CUDA events on the context's stream, state > L2 between ticks):
    k_mos1 in its transient form (combined Jacobian slots, the form the tick
    runs) and the grouped LU refactorization."""
    s0 = circ.tran_results()[3]
    stage_ms, ev = circ.tran_profile(PROFILE_TICKS, n_steps=window)
    s1 = circ.tran_results()[3]
    total = sum(stage_ms.values())
    inst = ev["mos1"] / PROFILE_TICKS
    us = stage_ms["mos1"] * 1e3 / PROFILE_TICKS
    alg = MOS1_ALG_BYTES * inst
    achieved = alg / (us * 1e-6) / 1e9
    traffic = None
    prof = os.path.join(HERE, "profiles", "k_mos1_mc4096.traffic.json")
    if args.workload == "mc" and args.rings == 4096 and os.path.exists(prof):
        try:
            t = json.load(open(prof))
            # the capture's launch evaluated t["instances"]; scale to this launch's active instances
            traffic = t["dram_bytes_per_launch"] * inst / t["instances"]
        except Exception:
            traffic = None
    mos = {"kernel": "k_mos1, transient form (MOSFET-1 evaluation + stamp into combined Jacobian slots, "
                     "masked by circuit activity), as launched by the tick",
           "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
           "peak_kind": peak_kind, "traffic": traffic,
           "algorithmic_bytes_per_launch": alg, "bytes_per_instance": MOS1_ALG_BYTES,
           "bytes_moved_by_code_per_instance": MOS1_BYTES_CODE, "instances_per_launch": inst, "launch_us": us,
           "share_of_tick": stage_ms["mos1"] / total,
           "note": "FP64-pipe bound on GB300: ncu shows the FP64 pipe ~80 % busy in this kernel"}
    # the factor launch refactors the circuits whose Newton iteration solves this tick
    circ_ticks = max(1, ev["circuits"])
    solving = min(1.0, (s1["newton_iters"] - s0["newton_iters"]) / circ_ticks)
    lu_us = stage_ms["lu_factor"] * 1e3 / PROFILE_TICKS
    lu_alg = LU_BYTES_PER_NNZ * info["nnz_lu"] * solving
    lu_ach = lu_alg / (lu_us * 1e-6) / 1e9
    lu = {"kernel": "k_factor_groups_s (grouped left-looking refactorization on the frozen pattern)",
          "bound": "hbm", "achieved": lu_ach, "peak": hbm_peak, "unit": "GB/s", "frac": lu_ach / hbm_peak,
          "peak_kind": peak_kind, "traffic": None, "algorithmic_bytes_per_launch": lu_alg,
          "nnz_lu": info["nnz_lu"], "fraction_of_circuits_refactoring": solving, "launch_us": lu_us,
          "share_of_tick": stage_ms["lu_factor"] / total,
          "note": "latency-bound: a dependent chain of factor levels per circuit"}
    stages = {k: v / PROFILE_TICKS * 1e3 for k, v in stage_ms.items()}
    return mos, lu, stages


def _error_vs_fp64(nl, sample, seqs, workload):
    """Largest |dv| of the sampled circuits' recorded waveforms against the
    oracle (the CPU FP64 restatement) replaying the same accepted steps, and
    the oracle's own round-off floor (the same replay with every time point
    moved by one ulp); the exact window is where that floor stays below
    1e-9 max|v|."""
    import numpy as np
    import oracle
    from xyce_gb300 import netlist as N
    alt = "ulp"
    circuits = sorted({ci for ci, _ in sample})
    tasks, meta = [], []
    for ci in circuits:
        sub = N.extract_circuit(nl, ci) if nl.n_circuits > 1 else nl
        prs = [pr for c, pr in sample if c == ci]
        t, o, _ = seqs[(ci, prs[0])]
        v = np.stack([seqs[(ci, pr)][2] for pr in prs], axis=1)
        lp = [pr - nl.offsets[ci] for pr in prs]
        tasks += [(sub, lp, t, o, None), (sub, lp, t, o, alt)]
        meta.append((ci, v))
    res = oracle.run_many(tasks)
    worst, worst_exact, floor_max, pts = 0.0, 0.0, 0.0, 0
    for k, (ci, v) in enumerate(meta):
        ta, va, sa = res[2 * k]
        tb, vb, sb = res[2 * k + 1]
        if sa["status"] != 0 or sb["status"] != 0 or len(va) != len(v) or len(vb) != len(v):
            return {"error": f"oracle replay of circuit {ci} failed (status {sa['status']}, {sb['status']})"}
        err = np.max(np.abs(va - v), axis=1)
        floor = np.max(np.abs(vb - va), axis=1)
        vmax = float(np.max(np.abs(va)))
        above = np.nonzero(floor > 1e-9 * vmax)[0]
        exact = int(above[0]) if len(above) else len(floor)
        worst = max(worst, float(err.max()))
        worst_exact = max(worst_exact, float(err[:exact].max()) if exact else 0.0)
        floor_max = max(floor_max, float(floor.max()))
        pts += len(v)
    return {"max_abs_v": worst, "max_abs_v_exact_window": worst_exact, "roundoff_floor_v": floor_max,
            "circuits": len(meta), "points": pts,
            "method": "oracle (CPU FP64) replaying the GPU's accepted times and integration orders; "
                      "floor = the oracle's own replay with every time moved by one ulp; exact window = points "
                      "before that floor exceeds 1e-9 max|v|"}


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
    w = WORKLOADS[args.workload]
    window = w["window"]
    nl, probes, desc = _workload(args.workload, args.rings)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    stream_of = lambda c: torch.cuda.ExternalStream(xg.lib().xg_get_stream(c.h))

    if args.ncu_case:
        # the profiling case: operating point, first analysis and one window
        circ = xg.Circuit(nl, device=dev)
        circ.tran_set_form(xg.FORM_RESIDENT if args.ncu_form == "resident" else xg.FORM_TICK_GRAPH)
        circ.tran_start(probes=probes, cap=16)
        circ.tran_advance(window)
        torch.cuda.synchronize()
        print(json.dumps({"ncu_case": desc["workload"], "form": args.ncu_form, "instances": len(nl.mos1)}),
              flush=True)
        circ.close()
        return
    sample = _sample(nl, args.workload)
    rec_probes = sorted({p for _, p in sample} | set(probes))
    cap = (args.warmup + args.steps) * window + PROFILE_TICKS + 16
    clk_path = (f"{args.clocks_csv}.rank{rank}" if world > 1 else args.clocks_csv) if args.clocks_csv \
        else os.path.join(tempfile.gettempdir(), f"xg_clocks_{os.getpid()}.csv")
    sampler = _clock_sampler(clk_path)
    if world > 1:
        torch.distributed.barrier()
    main_form = {"auto": xg.FORM_AUTO, "tick_graph": xg.FORM_TICK_GRAPH, "resident": xg.FORM_RESIDENT}[args.form]
    circ, ms_total, st0, st1 = _timed_windows(xg, nl, rec_probes, dev, args, window, xg.PREC_FP64, flush,
                                              stream_of, cap=cap, form=main_form)
    if sampler:
        sampler.terminate()
        sampler.wait()
    steps_done = st1["accepted"] - st0["accepted"]
    ticks = st1["ticks"] - st0["ticks"]
    evals = st1["device_evals"] - st0["device_evals"]
    info = circ.lu_info()
    info["tuning"] = circ.lu_tuning()
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
    # kernels launched in the timed windows, counted by the driver: the
    # kernel nodes of each replayed tick graph, or, in the circuit-resident
    # form, the resident kernel and the completion count of each launch
    kernels_per_tick = int(st1.get("kernels_per_tick", 0))
    gpu_launches = int(st1["kernel_launches"] - st0["kernel_launches"])
    form = {xg.FORM_TICK_GRAPH: "tick_graph", xg.FORM_RESIDENT: "circuit_resident"}.get(st1["form"], "?")
    # the sampled circuits' accepted-step sequences (for the error against FP64)
    counts, times, values, _ = circ.tran_results()
    orders = circ.tran_orders()
    seqs = {}
    for ci, pr in sample:
        m = int(counts[ci])
        col = [p for p in rec_probes if nl.offsets[ci] <= p < nl.offsets[ci + 1]].index(pr)
        seqs[(ci, pr)] = (times[ci, :m].copy(), orders[ci, :m].copy(), values[ci, :m, col].copy())
    n_unknowns = circ.n
    roof = lu_roof = stages = None
    resident_roof = None
    if form == "circuit_resident":
        # the whole tick in one kernel: its algorithmic bytes are the device
        # evaluations' (the per-instance figure) over the timed windows
        alg = MOS1_ALG_BYTES * evals_all
        ach = alg / (ms_max / 1e3) / 1e9
        resident_roof = {"kernel": "k_resident (every stage of every tick of a circuit in one CTA)", "bound": "hbm",
                         "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                         "peak_kind": peak_kind, "algorithmic_bytes": alg,
                         "note": "device-evaluation bytes only (MOSFET-1 evaluation + stamp per instance per "
                                 "Newton iteration) over the timed windows; assembly, LU and control bytes not counted"}
    resident_stages = None
    if rank == 0:
        # the tick profiler launches the tick-graph kernels one by one, stage by stage
        roof, lu_roof, stages = _rooflines(circ, nl, window, hbm_peak, peak_kind, info, args)
        try:
            # where the circuit-resident tick's CTAs spend their cycles (one window, 64-thread CTAs)
            cyc, cticks = circ.tran_profile_resident(window, threads=64)
            tot = sum(cyc.values())
            resident_stages = {"cta_kcycles_per_circuit_iter": tot / max(1, cticks) / 1e3,
                               "share": {k: v / tot for k, v in cyc.items()}, "circuit_iters": cticks}
        except xg.XgError as e:
            resident_stages = {"unavailable": str(e)}
    circ.tran_end()
    circ.close()

    # ---- the FP32-LU + FP64-refinement form, same workload ------------------
    forms = None
    if rank == 0 and args.forms:
        # the comparison forms are reported, not required: a failure of one
        # is recorded under its name instead of losing the others
        forms = {"fp64": value}

        def rate(prec, **kw):
            c, ms_, s0_, s1_ = _timed_windows(xg, nl, probes, dev, args, window, prec, flush, stream_of, **kw)
            tun = c.lu_tuning()
            c.tran_end()
            c.close()
            steps = s1_["accepted"] - s0_["accepted"]
            return steps / (ms_ / 1e3), (s1_["newton_iters"] - s0_["newton_iters"]) / max(1, steps), tun

        def attempt(name, fn):
            try:
                fn()
            except Exception as e:  # noqa: BLE001
                forms[name + "_error"] = f"{type(e).__name__}: {e}"

        def fp32():
            r, it, t32 = rate(xg.PREC_FP32_IR)
            forms.update({"fp32_lu_fp64_ir": r, "fp32_lu_fp64_ir_newton_iters_per_step": it,
                          # one factorization and one solve as the tuner timed them on this pattern
                          # (all circuits refactoring; the FP32 solve includes its refinement steps)
                          "fp32_factor_us": t32["factor_us"], "fp32_solve_us": t32["solve_us"],
                          "fp64_factor_us": info["tuning"]["factor_us"], "fp64_solve_us": info["tuning"]["solve_us"]})

        attempt("fp32_lu_fp64_ir", fp32)
        # the tick graph alone (15 kernels per tick over the whole batch)
        attempt("fp64_tick_graph",
                lambda: forms.__setitem__("fp64_tick_graph", rate(xg.PREC_FP64, form=xg.FORM_TICK_GRAPH)[0]))
        if st1["option"] == 5 and form == "tick_graph" and any(st1["option_us_per_iter"][:5]):
            # the timed trials chose the tick graph: the resident form alone, for comparison
            attempt("fp64_resident",
                    lambda: forms.__setitem__("fp64_resident", rate(xg.PREC_FP64, form=xg.FORM_RESIDENT)[0]))
        # the LU sweeps with the analysis' closed-form launch shapes instead of the timed ones
        attempt("fp64_tick_graph_lu_model_shapes",
                lambda: forms.__setitem__("fp64_tick_graph_lu_model_shapes",
                                          rate(xg.PREC_FP64, tune=xg.TUNE_MODEL, form=xg.FORM_TICK_GRAPH)[0]))
        if args.workload == "mc":
            attempt("one_ring_at_a_time", lambda: forms.update(_one_at_a_time(xg, nl, dev, window, stream_of, value)))
            attempt("learned_predictor", lambda: forms.__setitem__("learned_predictor", _learned_form(xg)))

    # ---- the other configs, plain FP64 path ---------------------------------
    others = None
    if rank == 0 and args.others and args.workload == "mc":
        others = _other_configs(xg, dev, flush, stream_of)

    # ---- end to end through the C-ABI with host buffers --------------------
    e2e = None
    if rank == 0:
        tr = nl.tran
        per_circuit = (args.warmup + args.steps) * window
        tr.max_steps = per_circuit
        a = nl.arrays()
        h2d = sum(v.nbytes for k, v in a.items() if hasattr(v, "nbytes"))
        h2d += sum(x.nbytes for k in ("res", "cap", "vsrc", "isrc", "diode", "mos1", "bsim4") for x in a[k])
        ecap = per_circuit + 8
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c3 = xg.Circuit(nl, device=dev, arrays=a)
        counts3, tt, vv, st = c3.transient(tr, probes=probes, cap=ecap)
        dt = time.perf_counter() - t0
        c3.close()
        # xg_tran_results copies the time and probe buffers of every circuit
        d2h = nl.n_circuits * ecap * 8 * 2 + nl.n_circuits * 4
        nsteps = args.warmup + args.steps
        e2e = {"value": st["accepted"] / dt, "unit": UNIT,
               "h2d_bytes_per_step": h2d / nsteps, "d2h_bytes_per_step": d2h / nsteps,
               "seconds": dt, "accepted": st["accepted"]}
        tr.max_steps = 0

    if rank == 0:
        cpu = err = None
        if args.cpu:
            cpu = cpu_baseline(args)
            if sample:
                err = _error_vs_fp64(nl, sample, seqs, args.workload)
        clocks = _clock_summary(clk_path, dev)
        config = dict(desc)
        config.update({"unknowns": n_unknowns, "window_steps_per_circuit": window,
                       "l2": "flushed between windows (256 MiB write); device state > L2",
                       "parallelism": f"replicas x{world}"})
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "device_evals_per_s": evals_all / (ms_max / 1e3),
                "newton_iters_per_step": (st1["newton_iters"] - st0["newton_iters"]) / max(1, steps_done),
                "form": form, "ticks": ticks, "kernels_per_tick": kernels_per_tick, "gpu_launches": gpu_launches,
                "form_trials_us_per_newton_iter": dict(zip(("resident_32", "resident_64", "resident_128",
                                                            "resident_256", "resident_512", "tick_graph"),
                                                           st1["option_us_per_iter"])),
                "lu": info, "roofline": roof, "roofline_lu": lu_roof, "roofline_resident": resident_roof,
                "tick_stages_us": stages, "resident_stages": resident_stages,
                "max_err_vs_fp64": err, "forms": forms, "other_configs": others, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mc", choices=sorted(WORKLOADS))
    ap.add_argument("--rings", type=int, default=4096,
                    help="rings of the mc workload (a smaller batch is the profiling case)")
    ap.add_argument("--no-cpu", dest="cpu", action="store_false", help="skip the CPU baseline")
    ap.add_argument("--ncu-case", action="store_true",
                    help="only the operating point and one window (the case the ncu captures profile)")
    ap.add_argument("--tail", type=float, default=None,
                    help="active fraction below which the resident kernel finishes a tick-graph advance "
                         "(default: the library's)")
    ap.add_argument("--form", default="auto", choices=["auto", "tick_graph", "resident"],
                    help="advancing form of the timed run (auto: timed choice on the run itself)")
    ap.add_argument("--ncu-form", default="tick_graph", choices=["tick_graph", "resident"],
                    help="advancing form of the --ncu-case run")
    ap.add_argument("--no-forms", dest="forms", action="store_false", help="skip the FP32-IR form")
    ap.add_argument("--no-others", dest="others", action="store_false",
                    help="skip the other configs (diode ladder, 10,001-stage ring, grid, BSIM4 DAG)")
    ap.add_argument("--clocks-csv", default=None,
                    help="keep the nvidia-smi clock samples of the timed region in this file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
