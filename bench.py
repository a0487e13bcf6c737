"""Benchmark: cell-updates/s of the FARGO_THORIN hydro loop on one GB300.

Workload: the 1024 x 3072 pebble + embryo disk (log r in [0.4, 2.5], gas with
Sigma = 5e-4 r^-0.5 perturbed by 1e-4 u, pebbles at 0.01 Sigma with Stokes
number 0.1, a 3e-5 M* embryo at r = 1 that feels the disk, accretes pebbles
and heats the gas, Bell & Lin opacity, SOR radiative diffusion at a relative
residual of 1e-8), FP64, synthetic data built by the library's own set-up.

A step is one DT of AlgoGas (all its CFL substeps, each one full hydro
substep with SOR); cell-updates = nrad * nsec * substeps.  ``value`` is timed
on the device with CUDA events on the library's stream with the state
resident in HBM; ``e2e`` restores the state from before those steps and
replays the same DTs (same substeps and SOR sweeps, checked) through the C
ABI with the state uploaded from pinned host buffers and downloaded back
every step.

--impl reference times the CPU restatement of the reference algorithm (the
oracle, OpenMP over all host cores) on the same disk and the same DTs: the
GPU arm's warm-up DTs from t = 0, then its --steps timed DTs (about 4 s per
DT on 16 Grace cores).  ``cpu_baseline`` in the GPU line runs the oracle from
the GPU arm's own snapshot, i.e. on the first timed DTs, for about 20 s, and
checks their substep and SOR sweep counts against the GPU's.
With torchrun (N > 1) every rank advances its own replica (the disk does not
shard); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NR, NS = 1024, 3072
SOR_EPS = 1e-8
METRIC = "cell-updates/s per full step (1024x3072 pebble+embryo disk, SOR 1e-8)"
UNIT = "cell-updates/s"
# Algorithmic bytes per cell of one full SOR sweep: T read + write, the five
# matrix coefficients and the right-hand side (8 FP64 values).
SOR_BYTES_PER_CELL_SWEEP = 64.0
# Algorithmic bytes per cell of one hydro substep: the gas state (Sigma, v_r,
# v_theta, e read and written, 64 B) and the pebble state (Sigma_p, v_r,p,
# v_theta,p read and written, the size read, 56 B).
STATE_BYTES_PER_CELL_SUBSTEP = 120.0
WORKLOAD = f"disk1 {NR}x{NS} gas+pebbles+3e-5 embryo, BL94, SOR eps {SOR_EPS}"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


STATE_FIELDS = [0, 1, 2, 3, 4, 5, 6, 7]      # dens, vrad, vtheta, energy, pebble dens/vrad/vtheta/size
SNAPSHOT_FIELDS = STATE_FIELDS + [8, 9, 11]   # + temperature, sound speed, Stokes number


def make_disk(nr=NR, ns=NS):
    from fargo_thorin_gb300 import workloads
    from fargo_thorin_gb300.disk import GpuDisk
    p = workloads.params_for("disk1", nr, ns, sor_eps=SOR_EPS)
    d = GpuDisk(p)
    d.init_default()
    st = workloads.perturbed_state(p, {"dens": d.get(0), "temper": d.get(8)})
    d.set(0, st["dens"]); d.set(1, st["vrad"]); d.set(3, st["energy"])
    d.set(4, st["pebdens"]); d.set(7, st["pebsize"])
    d.refresh(2)
    sys_ = workloads.make_planets(p, [workloads.PLANET1])
    return p, d, sys_


def reduce_over_ranks(values, ops, device):
    """All-reduce each value over the ranks of the initialised process group
    ("max" or "sum"); with one rank (or no group) the values come back as
    they are.  Used for the max-over-ranks step time and summed updates."""
    import torch
    import torch.distributed as dist
    multi = dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1
    out = []
    for v, op in zip(values, ops):
        t = torch.tensor([float(v)], dtype=torch.float64, device=device)
        if multi:
            dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
        out.append(float(t.item()))
    return out


WARMNET = os.environ.get("THORIN_WARMNET", os.path.join(ROOT, "fargo_thorin_gb300", "warmnet_disk1_1024x3072.npy"))
WARMNET_FACTOR = int(os.environ.get("THORIN_WARMNET_FACTOR", "1"))   # disk cells per network cell per axis


def warm_start_phase(d, snapd, snap_sys, steps, stream, barrier, t_plain, plain_per_solve):
    """Replay the timed DTs with the trained network attached in PREDICT
    mode: SOR sweeps per solve against the plain run, the throughput, and the
    temperature difference after the DTs (both meet the same threshold)."""
    import torch
    from fargo_thorin_gb300 import warmstart as WS
    if not os.path.exists(WARMNET):
        return {"unavailable": "no trained network file"}

    def replay(params):
        """the timed DTs again from the snapshot with a network attached"""
        net = WS.WarmNet(NR, NS, params=params, factor=WARMNET_FACTOR)
        d.restore(snapd)
        sys_ = snap_sys.copy()
        WS.attach(d, net, WS.PREDICT)
        st0, pred0 = d.stats(), WS.stats(d).predictions
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        subs = 0
        for _ in range(steps):
            d.algogas(sys_)
            subs += d.stats().substeps
        e1.record(stream)
        barrier()
        st1 = d.stats()
        pred = WS.stats(d).predictions - pred0
        WS.attach(d, None, WS.OFF)
        net.close()
        return (e0.elapsed_time(e1), subs, pred,
                (st1.sor_sweeps - st0.sor_sweeps) / max(st1.sor_calls - st0.sor_calls, 1), d.get(8))

    def replay_extrapolated(order=2):
        """the timed DTs again, each solve started from the extrapolated update"""
        d.restore(snapd)
        sys_ = snap_sys.copy()
        WS.set_order(d, order)
        WS.attach(d, None, WS.EXTRAPOLATE)
        st0 = d.stats()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        subs = 0
        for _ in range(steps):
            d.algogas(sys_)
            subs += d.stats().substeps
        e1.record(stream)
        barrier()
        st1 = d.stats()
        WS.attach(d, None, WS.OFF)
        ms = e0.elapsed_time(e1)
        per = (st1.sor_sweeps - st0.sor_sweeps) / max(st1.sor_calls - st0.sor_calls, 1)
        t = d.get(8)
        return {"order": order, "sweeps_per_solve": per, "sweeps_ratio_plain_over_extrapolated": plain_per_solve / per,
                "value": NR * NS * subs / (ms / 1e3), "ms_per_step": ms / steps, "substeps": subs,
                "t_rel_l2_vs_plain": float(np.linalg.norm(t - t_plain) / np.linalg.norm(t_plain)),
                "start": "one Jacobi step from T_old + s dt (2 r_1 - r_2), r_k = (T_conv - T_start) / dt of the k-th "
                         "last solve, s minimising the L2 residual along it"}

    extrapolated = replay_extrapolated()
    # control: the same coupling with an untrained network (zero output
    # layer), i.e. the previous temperature plus one Jacobi step
    _, _, _, jacobi_per_solve, _ = replay(WS.init_params(0))
    ms, subs, pred, per_solve, t = replay(WS.WarmNet.load_params(WARMNET))
    return {"plain_sweeps_per_solve": plain_per_solve, "extrapolated": extrapolated,
            "learned_sweeps_per_solve": per_solve,
            "jacobi_start_sweeps_per_solve": jacobi_per_solve,
            "sweeps_ratio_plain_over_learned": plain_per_solve / per_solve if per_solve else None,
            "learned_value": NR * NS * subs / (ms / 1e3), "learned_ms_per_step": ms / steps, "substeps": subs,
            "network_applications": pred, "network": os.path.relpath(WARMNET, ROOT), "network_factor": WARMNET_FACTOR,
            "t_rel_l2_vs_plain": float(np.linalg.norm(t - t_plain) / np.linalg.norm(t_plain)),
            "threshold": "eps * L1 residual of the previous-temperature start, as the plain solve"}


def ensemble_phase(n=64, seed=0, ndt=2, settle=3):
    """The batched ensemble: n drawn gas + pebble + embryo disks of uneven
    sizes (Nrad in {128, 192, 256, 384, 512}, Nsec = 3 Nrad; alpha, Sigma0,
    h and the embryo mass drawn per disk).  After each disk's first DT (the
    omega calibration) and `settle` DTs as device-resident DT graphs, the
    autotuner picks the schedule (graph mode or a host thread pool, then the
    SOR launch shape per disk size) on one DT from a snapshot of every disk.
    The same ndt DTs from that snapshot then run with the chosen schedule
    and with the disks one after the other on the host path: aggregate
    cell-updates/s and the speed-up on identical work (the substeps and SOR
    sweeps of both runs are checked equal)."""
    from fargo_thorin_gb300.ensemble import Ensemble
    ens = Ensemble.drawn(n, seed=seed)           # each disk has done its first DT
    for _ in range(settle):
        ens.step_graph()
    snaps = ens.snapshot()
    tune = ens.tune_schedule(snaps)
    ens.restore(snaps)
    best = ens.run_schedule(tune["schedule"], ndt)
    ens.restore(snaps)
    seq = ens.run_schedule({"mode": "sequential"}, ndt)
    sched = tune["schedule"]
    sizes = sorted(d.nr for d in ens.disks)
    out = {"disks": len(ens.disks), "nrad": sizes, "cells": ens.cells,
           "schedule": {"mode": sched["mode"], "workers": sched.get("workers"),
                        "sor_launch_shapes": {str(k): list(v) for k, v in sched.get("shapes", {}).items()}},
           "value": best["cell_updates"] / best["seconds"], "unit": UNIT, "ms_per_dt": 1e3 * best["seconds"] / ndt,
           "sequential_ms_per_dt": 1e3 * seq["seconds"] / ndt,
           "speedup_vs_sequential": seq["seconds"] / best["seconds"],
           "same_work": bool(best["cell_updates"] == seq["cell_updates"] and best["sweeps"] == seq["sweeps"]),
           "settle_dts": settle, "tuner_trials": tune["trials"],
           "graph": "one CUDA graph per disk and DT (substep loop, planet side and SOR schedule on the device), "
                    "all disks launched on their own streams before any is waited for",
           "timing": "wall clock with a device synchronisation on both sides; every run replays the same DTs "
                     "from one snapshot of every disk"}
    ens.close()
    return out


def combined_phase(n_each=8, ndt=1, settle=1, seed=11):
    """The combined workload: 2 n_each gas + pebble + embryo disks, n_each of
    1024x3072 and n_each of 2048x6144 rings x sectors, with drawn alpha,
    Sigma0, aspect ratio and embryo mass, FP64 hydro, SOR tolerance 1e-8.
    Every disk starts from the omega schedule calibrated on the 1024x3072
    bench disk, takes its first DT and `settle` more as device-resident DT
    graphs (all disks together); from one snapshot of every disk the same
    ndt DTs then run (a) batched: every disk a
    device-resident DT graph, all launched together, each with the learned
    SOR warm start attached, and (b) plain: the disks one after the other on
    the host path without the network, and (c) as (a) with the extrapolated
    SOR start in place of the network.  Cell-updates/s, the speed-ups of (a)
    and (c) over (b) and the SOR sweeps per solve of each."""
    from fargo_thorin_gb300 import warmstart as WS
    from fargo_thorin_gb300.ensemble import Ensemble
    t_setup = time.perf_counter()
    # the omega schedule of a calibrated 1024x3072 disk (the bench workload's
    # first DT) seeds every disk
    _, d0, s0 = make_disk()
    d0.algogas(s0)
    sor0 = d0.sor_state()[:3]
    d0.close()
    ens = Ensemble.drawn_sizes([1024] * n_each + [2048] * n_each, seed=seed, sor_state=sor0)
    for _ in range(settle):
        ens.step_graph()
    snaps = ens.snapshot()
    t_setup = time.perf_counter() - t_setup
    params = WS.WarmNet.load_params(WARMNET) if os.path.exists(WARMNET) else None
    nets = []
    if params is not None:
        for dd in ens.disks:
            net = WS.WarmNet(dd.nr, dd.ns, params=params)
            WS.attach(dd, net, WS.PREDICT)
            nets.append(net)
    ens.restore(snaps)
    calls0 = sum(dd.stats().sor_calls for dd in ens.disks)
    a = ens.run_schedule({"mode": "graph"}, ndt)
    a_calls = sum(dd.stats().sor_calls for dd in ens.disks) - calls0
    for dd, net in zip(ens.disks, nets):
        WS.attach(dd, None, WS.OFF)
        net.close()
    # (c) batched with the extrapolated start instead of the network
    ens.restore(snaps)
    for dd in ens.disks:
        WS.attach(dd, None, WS.EXTRAPOLATE)
    calls0 = sum(dd.stats().sor_calls for dd in ens.disks)
    c = ens.run_schedule({"mode": "graph"}, ndt)
    c_calls = sum(dd.stats().sor_calls for dd in ens.disks) - calls0
    for dd in ens.disks:
        WS.attach(dd, None, WS.OFF)
    ens.restore(snaps)
    calls0 = sum(dd.stats().sor_calls for dd in ens.disks)
    b = ens.run_schedule({"mode": "sequential"}, ndt)
    b_calls = sum(dd.stats().sor_calls for dd in ens.disks) - calls0
    out = {"disks": len(ens.disks), "grids": f"{n_each} x 1024x3072 + {n_each} x 2048x6144", "cells": ens.cells,
           "dts": ndt, "value": a["cell_updates"] / a["seconds"], "unit": UNIT,
           "ms_per_dt": 1e3 * a["seconds"] / ndt, "sequential_plain_value": b["cell_updates"] / b["seconds"],
           "sequential_plain_ms_per_dt": 1e3 * b["seconds"] / ndt,
           "speedup_vs_sequential_plain": (a["cell_updates"] / a["seconds"]) / (b["cell_updates"] / b["seconds"]),
           "sweeps_per_solve_batched_learned": a["sweeps"] / max(a_calls, 1),
           "sweeps_per_solve_sequential_plain": b["sweeps"] / max(b_calls, 1),
           "batched_extrapolated": {"value": c["cell_updates"] / c["seconds"], "ms_per_dt": 1e3 * c["seconds"] / ndt,
                                    "speedup_vs_sequential_plain": (c["cell_updates"] / c["seconds"]) /
                                                                   (b["cell_updates"] / b["seconds"]),
                                    "sweeps_per_solve": c["sweeps"] / max(c_calls, 1)},
           "warm_start": os.path.relpath(WARMNET, ROOT) if params is not None else None,
           "setup_s": t_setup, "settle_dts": settle,
           "timing": "wall clock with a device synchronisation on both sides; both runs replay the same DTs from "
                     "one snapshot of every disk"}
    ens.close()
    return out


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from fargo_thorin_gb300 import _lib
    _lib.load()
    p, d, sys_ = make_disk()
    for _ in range(args.warmup):
        d.algogas(sys_)
    stream = torch.cuda.ExternalStream(d.stream())
    # snapshot of the whole disk state, so that the end-to-end phase below
    # repeats exactly the DTs of the device-timed phase
    snapd = d.snapshot(SNAPSHOT_FIELDS)
    snap = snapd["fields"]
    snap_sys = sys_.copy()
    d.set_timing(True)
    launches0 = d.stats().kernel_launches
    clocks = ClockSampler(local)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # device-timed steps, state resident in HBM
    barrier()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    subs, sweeps0, calls0 = 0, d.stats().sor_sweeps, d.stats().sor_calls
    per_dt = []                               # (substeps, SOR sweeps) of each timed DT
    for _ in range(args.steps):
        w0 = d.stats().sor_sweeps
        d.algogas(sys_)
        st_ = d.stats()
        subs += st_.substeps
        per_dt.append((st_.substeps, st_.sor_sweeps - w0))
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    st = d.stats()
    sweeps = st.sor_sweeps - sweeps0
    solves = st.sor_calls - calls0
    t_plain = d.get(8)
    launches = st.kernel_launches - launches0
    sor_avg_ms = st.sor_time_ms / max(st.sor_passes, 1)
    ms_max, subs_all = reduce_over_ranks([ms, subs], ["max", "sum"], "cuda")
    total_updates = NR * NS * subs_all
    value = total_updates / (ms_max / 1e3)

    # the same DTs as device-resident DT graphs (one graph launch per DT)
    graph = None
    if d.graph_supported(snap_sys):
        d.restore(snapd)
        gsys = snap_sys.copy()
        gsw0 = d.stats().sor_sweeps
        barrier()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        gsubs = 0
        for _ in range(args.steps):
            d.algogas_graph(gsys)
            gsubs += d.stats().substeps
        g1.record(stream)
        barrier()
        gms = g0.elapsed_time(g1)
        gsweeps = d.stats().sor_sweeps - gsw0
        graph = {"value": NR * NS * gsubs / (gms / 1e3), "ms_per_step": gms / args.steps, "substeps": gsubs,
                 "sor_sweeps": gsweeps, "same_work_as_value": bool(gsubs == subs and gsweeps == sweeps),
                 "t_rel_l2_vs_value": float(np.linalg.norm(d.get(8) - t_plain) / np.linalg.norm(t_plain)),
                 "mode": "one CUDA graph launch per DT: substep loop, planet side and SOR schedule on the device"}

    # end to end through the C ABI with host buffers (pinned), from the same
    # starting state: the same DTs, substeps and SOR sweeps as above
    d.restore(snapd)
    sys_ = snap_sys.copy()
    sweeps_e0 = d.stats().sor_sweeps
    n = (NR + 1) * NS
    host = {f: torch.empty(n, dtype=torch.float64, pin_memory=True) for f in STATE_FIELDS}
    for f in STATE_FIELDS:
        host[f].numpy()[:] = snap[f]
    L, h = d.L, d.h
    ptr = {f: C.cast(host[f].data_ptr(), C.POINTER(C.c_double)) for f in STATE_FIELDS}
    barrier()
    t0 = time.perf_counter()
    esubs = 0
    for _ in range(args.steps):
        for f in STATE_FIELDS:
            _lib.check(L.thorin_gpu_upload(h, f, ptr[f]), "upload")
        d.algogas(sys_)
        esubs += d.stats().substeps
        for f in STATE_FIELDS:
            _lib.check(L.thorin_gpu_download(h, f, ptr[f]), "download")
    barrier()
    e_s = time.perf_counter() - t0
    esweeps = d.stats().sor_sweeps - sweeps_e0
    e_max, esubs_all = reduce_over_ranks([e_s, esubs], ["max", "sum"], "cuda")
    e2e_value = NR * NS * esubs_all / e_max

    # the same DTs again with the learned SOR warm start (device-timed)
    learned = warm_start_phase(d, snapd, snap_sys, args.steps, stream, barrier, t_plain,
                               sweeps / max(solves, 1))
    ens = None
    if rank == 0 and not args.no_ensemble:
        try:
            ens = ensemble_phase()
        except Exception as exc:          # reported in the line, the headline stands
            ens = {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}

    if rank == 0:
        peak, peak_kind = peaks()
        cells_pass = (NR - 2) * NS / 2
        bytes_pass = SOR_BYTES_PER_CELL_SWEEP * cells_pass
        achieved = bytes_pass / (sor_avg_ms / 1e3) / 1e9
        prof = {}
        tf = os.path.join(ROOT, "profiles", "k_sor_pass_disk1_1024x3072.json")
        if os.path.exists(tf):
            try:
                with open(tf) as f:
                    prof = json.load(f)
            except Exception:
                prof = {}
        traffic = prof.get("bytes_per_launch")
        # The pass is bound by the FP64 pipe: its FP64 instructions per launch
        # (ncu count) over the live launch time, against this GPU's FMA rate.
        fp64 = None
        gf = C.c_double()
        if _lib.load().thorin_selftest_fp64_peak(C.byref(gf)) == 0 and prof.get("fp64_inst_per_launch"):
            inst = float(prof["fp64_inst_per_launch"])
            ach = inst / (sor_avg_ms / 1e3) / 1e9
            fp64 = {"bound": "fp64 pipe", "kernel": "k_sor_pass", "achieved": ach, "peak": gf.value / 2.0,
                    "unit": "G FP64 inst/s", "frac": ach / (gf.value / 2.0), "inst_per_launch": inst,
                    "peak_source": "FMA loop on this GPU at run time (thorin_selftest_fp64_peak), one FMA per "
                                   "instruction"}
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            cpu = cpu_baseline(p, snapd, snap_sys, per_dt)
        # the whole DT against both roofs: algorithmic bytes (state traffic of
        # every substep plus 64 B per cell per SOR sweep) and FP64
        # instructions (per-kernel ncu counts per cell, scaled to the DT)
        step_s = ms_max / args.steps / 1e3
        step_bytes = NR * NS * (STATE_BYTES_PER_CELL_SUBSTEP * subs + SOR_BYTES_PER_CELL_SWEEP * sweeps) / args.steps
        step_roof = {"bound": "hbm", "achieved": step_bytes / step_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": step_bytes / step_s / 1e9 / peak, "algorithmic_bytes_per_step": step_bytes,
                     "peak_kind": peak_kind}
        step_fp64 = None
        ff = os.path.join(ROOT, "profiles", "fp64_inst_per_cell_disk1.json")
        if fp64 and os.path.exists(ff):
            with open(ff) as f:
                fc = json.load(f)
            inst = NR * NS * (fc["hydro_per_cell_substep"] * subs + fc["sor_per_cell_sweep"] * sweeps) / args.steps
            step_fp64 = {"bound": "fp64 pipe", "achieved": inst / step_s / 1e9, "peak": fp64["peak"],
                         "unit": "G FP64 inst/s", "frac": inst / step_s / 1e9 / fp64["peak"],
                         "fp64_inst_per_step": inst, "counts": os.path.relpath(ff, ROOT)}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "nrad": NR, "nsec": NS, "substeps": subs, "sor_sweeps_per_substep": sweeps / max(subs, 1),
                       "timed_dts": f"DTs {args.warmup + 1}-{args.warmup + args.steps} from t = 0",
                       "per_dt_substeps_sweeps": per_dt,
                       "step": "one DT of AlgoGas (all CFL substeps)", "l2": "inputs larger than L2 (1.7 GB state)",
                       "parallelism": "replicas" if ws > 1 else "single disk"},
            "clocks": clk,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n * 8,
                    "d2h_bytes_per_step": 8 * n * 8, "substeps": esubs, "sor_sweeps": esweeps,
                    "same_work_as_value": bool(esubs == subs and esweeps == sweeps)},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": "k_sor_pass", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": bytes_pass, "avg_launch_ms": sor_avg_ms},
            "fp64_roofline": fp64,
            "graph_dt": graph,
            "step_roofline": step_roof,
            "step_fp64_roofline": step_fp64,
            "sor_warm_start": learned,
            "ensemble": ens,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    d.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return O


def oracle_disk(O, omp=True):
    """The bench workload on the oracle, set up like make_disk()."""
    from fargo_thorin_gb300 import workloads
    p = workloads.params_for("disk1", NR, NS, sor_eps=SOR_EPS)
    o = O.OracleDisk(p, omp=omp)
    o.init_default()
    st = workloads.perturbed_state(p, {"dens": o.get(0), "temper": o.get(8)})
    o.set(0, st["dens"]); o.set(1, st["vrad"]); o.set(3, st["energy"])
    o.set(4, st["pebdens"]); o.set(7, st["pebsize"])
    o.refresh(2)
    return p, o, workloads.make_planets(p, [workloads.PLANET1])


def cpu_baseline(p, snapd, snap_sys, per_dt, budget_s=20.0):
    """The oracle (OpenMP, all host cores) from the GPU arm's own snapshot
    taken after the warm-up: the same first timed DTs, as many as fit in
    about budget_s seconds (at least one).  Their substep and SOR sweep
    counts are compared with the GPU's."""
    O = _oracle()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    _, o, _ = oracle_disk(O)              # initial profiles and damping targets as on the GPU
    for f, v in snapd["fields"].items():
        o.set(f, v)
    o.refresh(0)                          # EOS of the snapshot's state
    o.set_sor_state(*snapd["sor"][:3])
    o.set_time(snapd["time"])
    o.set_dt_stellar(snapd["dt_stellar"])
    s = snap_sys.copy()
    t0 = time.perf_counter()
    mine = []
    while len(mine) < len(per_dt) and (not mine or time.perf_counter() - t0 < budget_s):
        w0 = o.stats().sor_sweeps
        o.algogas(s)
        st = o.stats()
        mine.append((st.substeps, st.sor_sweeps - w0))
    el = time.perf_counter() - t0
    subs = sum(m[0] for m in mine)
    sweeps = sum(m[1] for m in mine)
    return {"value": NR * NS * subs / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the first {len(mine)} timed DTs ({subs} substeps, {sweeps} SOR sweeps) of the {NR}x{NS} "
                      f"disk from the GPU arm's snapshot, {el:.1f} s",
            "sor_sweeps_per_substep": sweeps / max(subs, 1), "per_dt_substeps_sweeps": mine,
            "same_dts_as_gpu": bool(mine == [tuple(x) for x in per_dt[:len(mine)]])}


def run_reference(args):
    """The oracle on all host cores: the GPU arm's warm-up DTs from t = 0,
    then its --steps timed DTs, each DT one step."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    O = _oracle()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    p, o, s = oracle_disk(O)
    for _ in range(args.warmup):
        o.algogas(s)
    t0 = time.perf_counter()
    subs, dts, w0 = 0, [], o.stats().sor_sweeps
    for _ in range(args.steps):
        wd = o.stats().sor_sweeps
        o.algogas(s)
        st = o.stats()
        subs += st.substeps
        dts.append((st.substeps, st.sor_sweeps - wd))
    el = time.perf_counter() - t0
    sweeps = o.stats().sor_sweeps - w0
    value = NR * NS * subs / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nrad": NR, "nsec": NS, "substeps": subs,
                   "sor_sweeps_per_substep": sweeps / max(subs, 1),
                   "timed_dts": f"DTs {args.warmup + 1}-{args.warmup + args.steps} from t = 0",
                   "per_dt_substeps_sweeps": dts, "step": "one DT of AlgoGas (all CFL substeps)",
                   "implementation": "CPU restatement of the reference algorithm (oracle, bit-identical to the "
                                     "reference binary), OpenMP"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} DTs ({subs} substeps, {sweeps} SOR sweeps) after {args.warmup} "
                                   f"warm-up DTs, {el:.1f} s"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile(args, nr=NR, ns=NS):
    """One warm-up DT, then ``--steps`` DTs bracketed by cuProfilerStart/Stop,
    for ``ncu --profile-from-start off``.  Prints one line; no bench value."""
    import ctypes
    from fargo_thorin_gb300 import _lib
    _lib.load()
    p, d, sys_ = make_disk(nr, ns)
    d.algogas(sys_)
    cu = ctypes.CDLL("libcuda.so.1")
    cu.cuProfilerStart()
    for _ in range(args.steps):
        d.algogas(sys_)
    cu.cuProfilerStop()
    st = d.stats()
    print(json.dumps({"profiled_dts": args.steps, "nrad": nr, "nsec": ns, "substeps_last_dt": st.substeps,
                      "sor_last_niter": st.sor_last_niter}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 64-disk ensemble measurement")
    ap.add_argument("--combined", action="store_true",
                    help="only the combined 16-disk workload (1024x3072 and 2048x6144 grids, batched with the learned "
                         "and with the extrapolated SOR start against plain sequential; about 15 minutes); prints its "
                         "JSON line")
    ap.add_argument("--profile", action="store_true",
                    help="run --steps DTs inside cuProfilerStart/Stop for ncu; prints no bench line")
    ap.add_argument("--grid", type=int, nargs=2, metavar=("NRAD", "NSEC"), default=(NR, NS),
                    help="grid of the --profile run")
    args = ap.parse_args()
    if args.profile:
        run_profile(args, *args.grid)
        return
    if args.combined:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"metric": "combined workload", **combined_phase()}), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
