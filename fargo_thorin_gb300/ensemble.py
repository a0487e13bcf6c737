"""Ensembles of independent disks on one GPU (C ABI of include/thorin_ensemble.h).

Every disk is a full `GpuDisk` with its own streams; one ensemble step
advances each disk by one DT on a pool of host worker threads, so the
kernels of several disks share the GPU.  `tune` picks the worker count and
order by timing real DTs.

The drawn ensemble is the batched many-disk workload: gas + pebble disks
with Nrad in {128, 192, 256, 384, 512} and Nsec = 3 Nrad, alpha
log-uniform in [1e-4, 1e-2], Sigma0 scaled log-uniform in [0.3, 3], aspect
ratio uniform in [0.03, 0.07] and an embryo of 0 to 20 Earth masses at r = 1.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .disk import GpuDisk

SIZES = (128, 192, 256, 384, 512)
EARTH = 3.0e-6
GIVEN, LARGEST = 0, 1


def _sync():
    import torch
    torch.cuda.synchronize()


def draw(rng: np.random.Generator) -> dict:
    return {"nrad": int(rng.choice(SIZES)), "alpha": float(10.0 ** rng.uniform(-4.0, -2.0)),
            "sigma_scale": float(10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0))),
            "aspect": float(rng.uniform(0.03, 0.07)), "mplanet": float(rng.uniform(0.0, 20.0) * EARTH)}


def make_disk(spec: dict, seed: int = 0, nsec: int | None = None, sor_eps: float = 1e-8, sor_maxiters: int = 0):
    """A pebble + embryo disk of the drawn parameters in the measured initial
    state (perturbed Sigma, v_r = 0, Sigma_p = 0.01 Sigma, Stokes 0.1).
    sor_maxiters > 0 caps the SOR iterations (the reference's cap is 100000)."""
    from . import workloads
    nr = spec["nrad"]
    ns = nsec if nsec is not None else 3 * nr
    p = workloads.params_for("disk1", nr, ns, sor_eps=sor_eps, AlphaViscosity=spec["alpha"],
                             AspectRatio=spec["aspect"], Sigma0=5.0e-4 * spec["sigma_scale"])
    if sor_maxiters > 0:
        p.sor_maxiters = sor_maxiters
    d = GpuDisk(p)
    d.init_default()
    st = workloads.perturbed_state(p, {"dens": d.get(0), "temper": d.get(8)}, seed=seed)
    d.set(0, st["dens"]); d.set(1, st["vrad"]); d.set(3, st["energy"])
    d.set(4, st["pebdens"]); d.set(7, st["pebsize"])
    d.refresh(2)
    row = list(workloads.PLANET1)
    row[0] = spec["mplanet"]
    return p, d, workloads.make_planets(p, [tuple(row)])


class Ensemble:
    """A set of disks advanced together."""

    def __init__(self, specs: list, seed: int = 0, sor_maxiters: int = 0):
        self.L = _lib.load()
        self.specs = list(specs)
        built = [make_disk(s, seed=seed + k, sor_maxiters=sor_maxiters) for k, s in enumerate(self.specs)]
        self.params = [b[0] for b in built]
        self.disks = [b[1] for b in built]
        self.systems = [b[2] for b in built]
        self._arrays()

    @classmethod
    def drawn_sizes(cls, sizes: list, seed: int = 0, sor_maxiters: int = 20000, tries: int = 4,
                    sor_state=None) -> "Ensemble":
        """Disks of the given ring counts (Nsec = 3 Nrad) with drawn alpha,
        Sigma0, aspect ratio and embryo mass, each advanced by its first DT;
        a draw whose first DT fails is replaced by another of the same size.
        With sor_state = (omega, domega, niterlast) the disks start from that
        omega schedule instead of the reference's calibration of the first
        solve (IterateRelaxationParameter, whose cold SOR solves take
        thousands of sweeps on the largest grids), and their first DTs run
        together as device-resident DT graphs."""
        rng = np.random.default_rng(seed)
        specs, kept = [], []
        for k, nr in enumerate(sizes):
            for attempt in range(tries):
                spec = draw(rng)
                spec["nrad"] = int(nr)
                p, d, s = make_disk(spec, seed=seed + 100 * k + attempt, sor_maxiters=sor_maxiters)
                if sor_state is not None:
                    d.set_sor_state(*sor_state)
                    specs.append(spec)
                    kept.append((p, d, s))
                    break
                rc = d.L.thorin_gpu_algogas(d.h, C.byref(s))
                if rc == 0 and np.isfinite(d.get(8)).all():
                    specs.append(spec)
                    kept.append((p, d, s))
                    break
                d.close()
            else:
                raise RuntimeError(f"ensemble: no viable draw of a disk with {nr} rings")
        ens = cls.__new__(cls)
        ens.L = _lib.load()
        ens.specs = specs
        ens.params = [b[0] for b in kept]
        ens.disks = [b[1] for b in kept]
        ens.systems = [b[2] for b in kept]
        ens._arrays()
        if sor_state is not None:
            st = ens.step_graph()
            if any(x not in (0, 4) for x in st):
                raise RuntimeError(f"ensemble: first DTs failed: {st}")
        return ens

    @classmethod
    def drawn(cls, n: int, seed: int = 0, sor_maxiters: int = 2000, tries: int = 8) -> "Ensemble":
        """n drawn disks, each advanced by its first DT (with the SOR omega
        calibration).  Some draws are not viable on the coarser grids: the
        reference's own solver fails on them (no omega converges, or the
        temperature turns NaN).  Those are replaced by fresh draws.  The cap
        on SOR iterations makes such a failure quick."""
        rng = np.random.default_rng(seed)
        specs, kept = [], []
        k = 0
        while len(kept) < n:
            if k >= n * tries:
                raise RuntimeError("ensemble: too many drawn disks failed their first DT")
            spec = draw(rng)
            p, d, s = make_disk(spec, seed=seed + k, sor_maxiters=sor_maxiters)
            k += 1
            rc = d.L.thorin_gpu_algogas(d.h, C.byref(s))
            if rc == 0 and np.isfinite(d.get(8)).all():
                specs.append(spec)
                kept.append((p, d, s))
            else:
                d.close()
        ens = cls.__new__(cls)
        ens.L = _lib.load()
        ens.specs = specs
        ens.params = [b[0] for b in kept]
        ens.disks = [b[1] for b in kept]
        ens.systems = [b[2] for b in kept]
        ens._arrays()
        return ens

    def _arrays(self):
        n = len(self.disks)
        self._dp = (C.c_void_p * n)(*[d.h.value for d in self.disks])
        self._sp = (C.c_void_p * n)(*[C.cast(C.pointer(s), C.c_void_p).value for s in self.systems])

    @property
    def cells(self) -> int:
        return sum(d.nr * d.ns for d in self.disks)

    def step(self, workers: int = 1, order: int = LARGEST) -> list:
        """One DT of every disk; returns the per-disk status codes."""
        n = len(self.disks)
        st = (C.c_int * n)()
        rc = self.L.thorin_ensemble_algogas(self._dp, self._sp, n, workers, order, st)
        _lib.check(rc, "thorin_ensemble_algogas", ok=(0, 4))       # 4: a solve reached the iteration cap
        return list(st)

    def step_graph(self) -> list:
        """One DT of every disk, each as one device-resident DT graph, all
        launched before any is waited for; returns the status codes."""
        n = len(self.disks)
        st = (C.c_int * n)()
        rc = self.L.thorin_ensemble_algogas_graph(self._dp, self._sp, n, st)
        _lib.check(rc, "thorin_ensemble_algogas_graph", ok=(0, 4))
        return list(st)

    def tune(self, max_workers: int = 16, ndt: int = 1) -> dict:
        """Time every schedule (worker counts 1, 2, 4, ... in both orders) on
        real DTs and return the fastest.  Each schedule runs on the next DTs,
        so tune once the disks are past their initial transient; the
        one-worker time it reports is not a like-for-like baseline while the
        cost per DT is still falling."""
        bw, bo = C.c_int(), C.c_int()
        bms, sms = C.c_double(), C.c_double()
        _lib.check(self.L.thorin_ensemble_tune(self._dp, self._sp, len(self.disks), max_workers, ndt, C.byref(bw),
                                               C.byref(bo), C.byref(bms), C.byref(sms)), "thorin_ensemble_tune")
        return {"workers": bw.value, "order": "largest first" if bo.value == LARGEST else "given",
                "order_code": bo.value, "ms_per_dt": bms.value, "sequential_ms_per_dt": sms.value}

    # -- snapshots and the schedule autotuner of the device-resident DTs --

    SNAP_FIELDS = (0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 11)   # state, temperature, sound speed, Stokes number

    def snapshot(self) -> list:
        """Every disk's state (GpuDisk.snapshot) and planets (host copies)."""
        return [(d.snapshot(self.SNAP_FIELDS), s.copy()) for d, s in zip(self.disks, self.systems)]

    def restore(self, snaps: list):
        for d, s, (snap, sy) in zip(self.disks, self.systems, snaps):
            d.restore(snap)
            C.memmove(C.byref(s), C.byref(sy), C.sizeof(s))

    def run_schedule(self, sched: dict, ndt: int = 1) -> dict:
        """ndt DTs of the ensemble with a schedule: {"mode": "graph"} (every
        disk one DT graph, all launched before any is waited for) or
        {"mode": "pool", "workers": w} (host path on w threads, largest
        first) or {"mode": "sequential"}; with sched["shapes"] = {nrad:
        (sweeps per loop body, SOR threads per SM)} set first.  Wall time
        with a device synchronisation on both sides."""
        import time
        for d in self.disks:
            shape = sched.get("shapes", {}).get(d.nr, (8, 1536))
            if d.launch_shape() != tuple(shape):
                d.set_launch_shape(*shape)
        sw0 = sum(d.stats().sor_sweeps for d in self.disks)
        _sync()
        t0 = time.perf_counter()
        upd = 0
        for _ in range(ndt):
            if sched["mode"] == "graph":
                self.step_graph()
            elif sched["mode"] == "pool":
                self.step(sched["workers"], LARGEST)
            else:
                self.step(1, GIVEN)
            upd += sum(d.nr * d.ns * d.stats().substeps for d in self.disks)
        _sync()
        sec = time.perf_counter() - t0
        return {"seconds": sec, "cell_updates": upd, "sweeps": sum(d.stats().sor_sweeps for d in self.disks) - sw0}

    def tune_schedule(self, snaps: list, shapes=((8, 1536), (16, 1536), (8, 1024), (16, 2048)),
                      pool_workers=(8, 16, 32)) -> dict:
        """Autotuner: every candidate runs the same DT from the snapshot.
        First the mode (graph, or a host thread pool of each worker count);
        then, in graph mode, the SOR launch shape of each disk size in turn
        (sweeps per run of the sweep loop, resident threads per SM of a
        colour pass), keeping a size's best before the next size is tried.
        Returns the schedule and the time of every candidate."""
        trials = []

        def time_of(sched):
            self.restore(snaps)
            r = self.run_schedule(sched)
            trials.append({"schedule": {k: v for k, v in sched.items() if k != "shapes"},
                           "shapes": {str(k): list(v) for k, v in sched.get("shapes", {}).items()},
                           "ms": 1e3 * r["seconds"]})
            return r["seconds"]

        best = {"mode": "graph", "shapes": {}}
        best_t = time_of(best)
        for w in pool_workers:
            cand = {"mode": "pool", "workers": w, "shapes": {}}
            t = time_of(cand)
            if t < best_t:
                best, best_t = cand, t
        if best["mode"] == "graph":
            for nr in sorted({d.nr for d in self.disks}, reverse=True):
                for shape in shapes[1:]:
                    cand = {"mode": "graph", "shapes": dict(best["shapes"])}
                    cand["shapes"][nr] = shape
                    t = time_of(cand)
                    if t < best_t:
                        best, best_t = cand, t
        return {"schedule": best, "ms_per_dt": 1e3 * best_t, "trials": trials}

    def substeps(self) -> int:
        return sum(d.stats().substeps for d in self.disks)

    def close(self):
        for d in self.disks:
            d.close()
        self.disks = []
