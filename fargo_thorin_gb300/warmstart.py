"""Learned warm start of the SOR solve: host handle of the network and its
training driver (C ABI of include/thorin_warmnet.h).

The reference starts every SuccessiveOverrelaxation solve
(src_main/EnergySources.c:406-511) from the previous temperature.  With a
network attached in PREDICT mode the library starts it from the previous
temperature plus one Jacobi step plus the network's prediction, and iterates
to the same threshold (eps times the residual of the previous-temperature
start), so the converged temperature satisfies the same criterion as the
plain solve.  In TRAIN mode the solve stays plain and each converged update
becomes one training step of the network on the GPU.

Training data are the plain solver's own solves on disks with drawn
parameters: alpha log-uniform in [1e-4, 1e-2], aspect ratio uniform in
[0.03, 0.07] and an embryo of 0 to 20 Earth masses at r = 1.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib

NPARAMS = 57825
INPUTS = 16
OFF, PREDICT, TRAIN, EXTRAPOLATE = 0, 1, 2, 3
EARTH = 3.0e-6                         # Earth mass in solar masses
# (cin, cout) per layer: e0 e1 e2 e3 d2 d1 d0 out
LAYERS = [(7, 32)] + [(32, 32)] * 6 + [(32, 1)]


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights (std sqrt(2 / (9 cin))), zero biases; the output
    layer starts at zero so an untrained network predicts the Jacobi step."""
    rng = np.random.default_rng(seed)
    out = []
    for k, (cin, cout) in enumerate(LAYERS):
        std = 0.0 if k == len(LAYERS) - 1 else math.sqrt(2.0 / (9 * cin))
        out.append(rng.standard_normal(cout * 9 * cin) * std)
        out.append(np.zeros(cout))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == NPARAMS
    return p


class WarmNet:
    """The network on the GPU for a disk of nrad x nsec cells.  With
    factor 2 it runs on the half-resolution grid (each network cell averages
    2 x 2 disk cells' inputs, and its prediction applies to all four).  nr,
    ns are the network's grid, used by the raw forward and gradient calls."""

    def __init__(self, nrad: int, nsec: int, max_batch: int = 1, params: np.ndarray | None = None, factor: int = 1):
        if factor not in (1, 2) or nrad % (8 * factor) or nsec % (8 * factor):
            raise ValueError("factor 1 or 2, and nrad, nsec multiples of 8 * factor")
        self.L = _lib.load()
        self.factor = factor
        self.disk_nr, self.disk_ns = nrad, nsec
        self.nr, self.ns, self.maxb = nrad // factor, nsec // factor, max_batch
        self.h = C.c_void_p()
        _lib.check(self.L.thorin_warmnet_create(self.nr, self.ns, max_batch, C.byref(self.h)), "thorin_warmnet_create")
        self.set_params(init_params() if params is None else params)

    def close(self):
        if self.h:
            self.L.thorin_warmnet_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: np.ndarray):
        a = np.ascontiguousarray(p, dtype=np.float32)
        if a.size != NPARAMS:
            raise ValueError(f"expected {NPARAMS} parameters, got {a.size}")
        _lib.check(self.L.thorin_warmnet_set_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), NPARAMS),
                   "warmnet_set_params")

    def get_params(self) -> np.ndarray:
        a = np.empty(NPARAMS, np.float32)
        _lib.check(self.L.thorin_warmnet_get_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), NPARAMS),
                   "warmnet_get_params")
        return a

    def _x(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.uint16)
        if x.ndim != 4 or x.shape[1:] != (self.nr, self.ns, INPUTS) or not 1 <= x.shape[0] <= self.maxb:
            raise ValueError(f"x must be uint16 [batch<={self.maxb}][{self.nr}][{self.ns}][{INPUTS}]")
        return x

    def forward(self, x_bits: np.ndarray) -> np.ndarray:
        """x_bits: bf16 bit patterns [batch][nrad][nsec][16] -> y [batch][nrad][nsec]."""
        x = self._x(x_bits)
        y = np.empty(x.shape[:3], np.float32)
        _lib.check(self.L.thorin_warmnet_forward(self.h, x.shape[0], x.ctypes.data_as(C.POINTER(C.c_uint16)),
                                                 y.ctypes.data_as(C.POINTER(C.c_float))), "warmnet_forward")
        return y

    def gradient(self, x_bits: np.ndarray, target: np.ndarray):
        """Loss mean over rings 1..nrad-2 of (y - target)^2 and its gradient."""
        x = self._x(x_bits)
        t = np.ascontiguousarray(target, dtype=np.float32).reshape(x.shape[:3])
        loss = C.c_float()
        g = np.empty(NPARAMS, np.float32)
        _lib.check(self.L.thorin_warmnet_gradient(self.h, x.shape[0], x.ctypes.data_as(C.POINTER(C.c_uint16)),
                                                  t.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss),
                                                  g.ctypes.data_as(C.POINTER(C.c_float))), "warmnet_gradient")
        return float(loss.value), g

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, max_norm: float = 1.0):
        _lib.check(self.L.thorin_warmnet_adam(self.h, lr, beta1, beta2, eps, max_norm), "warmnet_adam")

    def save(self, path: str):
        np.save(path, self.get_params())

    @staticmethod
    def load_params(path: str) -> np.ndarray:
        p = np.load(path)
        if p.dtype != np.float32 or p.size != NPARAMS:
            raise ValueError(f"{path}: not a warm-start parameter file")
        return p


def attach(disk, net: WarmNet | None, mode: int, lr: float = 0.0):
    """Attach net to disk (PREDICT or TRAIN), start every solve from the
    previous solve's update (EXTRAPOLATE, net None) or detach (OFF)."""
    h = net.h if net is not None else C.c_void_p()
    _lib.check(disk.L.thorin_gpu_warmstart(disk.h, h, mode, lr), "thorin_gpu_warmstart")


def set_order(disk, order: int):
    """Order of the EXTRAPOLATE start (1 .. 4): the update rate of the last
    `order` solves extrapolated to the next one."""
    _lib.check(disk.L.thorin_gpu_warmstart_order(disk.h, order), "thorin_gpu_warmstart_order")


class WsStats(C.Structure):
    _fields_ = [("predictions", C.c_longlong), ("train_steps", C.c_longlong), ("last_loss", C.c_double),
                ("last_res_loss", C.c_double), ("last_sup_loss", C.c_double), ("step_sum", C.c_double)]


def stats(disk) -> WsStats:
    s = WsStats()
    _lib.check(disk.L.thorin_gpu_warmstart_stats(disk.h, C.byref(s)), "thorin_gpu_warmstart_stats")
    return s


def draw_disk(rng: np.random.Generator) -> dict:
    """One training disk: alpha log-U[1e-4, 1e-2], h U[0.03, 0.07], embryo
    mass U[0, 20] Earth masses."""
    return {"alpha": float(10.0 ** rng.uniform(-4.0, -2.0)), "aspect": float(rng.uniform(0.03, 0.07)),
            "mplanet": float(rng.uniform(0.0, 20.0) * EARTH)}


def make_training_disk(nrad: int, nsec: int, draw: dict, seed: int, dt_div: float = 1.0, sor_eps: float = 1e-8):
    """A pebble + embryo disk of the drawn parameters in its measured initial
    state (perturbed Sigma, v_r = 0, Sigma_p = 0.01 Sigma, Stokes 0.1)."""
    from . import workloads
    from .disk import GpuDisk
    p = workloads.params_for("disk1", nrad, nsec, sor_eps=sor_eps, AlphaViscosity=draw["alpha"],
                             AspectRatio=draw["aspect"])
    p.dt = p.dt / dt_div
    d = GpuDisk(p)
    d.init_default()
    st = workloads.perturbed_state(p, {"dens": d.get(0), "temper": d.get(8)}, seed=seed)
    d.set(0, st["dens"]); d.set(1, st["vrad"]); d.set(3, st["energy"])
    d.set(4, st["pebdens"]); d.set(7, st["pebsize"])
    d.refresh(2)
    row = list(workloads.PLANET1)
    row[0] = draw["mplanet"]
    return p, d, workloads.make_planets(p, [tuple(row)])


def train(net: WarmNet, ndisks: int, steps_per_disk: int, lr: float = 1e-3, seed: int = 0, dt_div: float = 1.0,
          lr_final: float | None = None, log=None) -> list:
    """Train net on the plain solver's solves: ndisks drawn disks, each run
    for steps_per_disk DTs with the network attached in TRAIN mode (one Adam
    step per SOR solve).  The learning rate decays geometrically from lr to
    lr_final over the disks.  Returns the loss after each disk."""
    rng = np.random.default_rng(seed)
    losses = []
    for k in range(ndisks):
        rate = lr if lr_final is None or ndisks == 1 else lr * (lr_final / lr) ** (k / (ndisks - 1))
        draw = draw_disk(rng)
        p, d, sys_ = make_training_disk(net.disk_nr, net.disk_ns, draw, seed=1000 * seed + k, dt_div=dt_div)
        attach(d, net, TRAIN, rate)
        for _ in range(steps_per_disk):
            d.algogas(sys_)
        s = stats(d)
        losses.append(s.last_loss)
        if log:
            log(f"disk {k}: alpha {draw['alpha']:.2e} h {draw['aspect']:.3f} m {draw['mplanet']:.1e} "
                f"lr {rate:.1e} steps {s.train_steps} loss {s.last_loss:.3e} (residual {s.last_res_loss:.3e}, "
                f"supervised {s.last_sup_loss:.3e})", flush=True)
        attach(d, None, OFF)
        d.close()
    return losses


def compare_sweeps(net: WarmNet, draw: dict, ndt: int, seed: int = 12345, dt_div: float = 1.0, warm: int = 1) -> dict:
    """SOR sweeps per solve of the same disk run plain and with the network
    (PREDICT), after `warm` DTs that include the omega calibration.  Also
    returns the relative L2 difference of the temperatures after the first
    compared DT and after the last (both solves meet the same residual
    threshold)."""
    out = {}
    temps, lasts = {}, {}
    for mode in (OFF, PREDICT):
        p, d, sys_ = make_training_disk(net.disk_nr, net.disk_ns, draw, seed=seed, dt_div=dt_div)
        for _ in range(warm):
            d.algogas(sys_)
        attach(d, net if mode == PREDICT else None, mode)
        s0 = d.stats()
        sweeps0, calls0 = s0.sor_sweeps, s0.sor_calls
        for k in range(ndt):
            d.algogas(sys_)
            if k == 0:
                temps[mode] = d.get(8)
        lasts[mode] = d.get(8)
        s1 = d.stats()
        out["plain" if mode == OFF else "learned"] = (s1.sor_sweeps - sweeps0) / max(s1.sor_calls - calls0, 1)
        out["solves"] = s1.sor_calls - calls0
        if mode == PREDICT:
            out["predictions"] = stats(d).predictions
        attach(d, None, OFF)
        d.close()
    a, b = temps[OFF], temps[PREDICT]
    out["t_rel_l2"] = float(np.linalg.norm(a - b) / np.linalg.norm(a))
    a, b = lasts[OFF], lasts[PREDICT]
    out["t_rel_l2_last"] = float(np.linalg.norm(a - b) / np.linalg.norm(a))
    return out


if __name__ == "__main__":
    import argparse
    import time
    ap = argparse.ArgumentParser(description="train the SOR warm-start network on the plain solver's solves")
    ap.add_argument("--nrad", type=int, default=1024)
    ap.add_argument("--nsec", type=int, default=3072)
    ap.add_argument("--disks", type=int, default=24)
    ap.add_argument("--steps", type=int, default=6, help="DTs per training disk")
    ap.add_argument("--factor", type=int, default=1, help="disk cells per network cell along each axis (1 or 2)")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--init", default=None, help="start from this parameter file")
    ap.add_argument("--out", default=None, help="write the trained parameters here (.npy)")
    ap.add_argument("--eval-dts", type=int, default=2)
    ap.add_argument("--forward", type=int, default=0,
                    help="only time this many forward passes on random inputs (no training, no evaluation)")
    a = ap.parse_args()
    t0 = time.time()
    net = WarmNet(a.nrad, a.nsec, params=WarmNet.load_params(a.init) if a.init else None, factor=a.factor)
    if a.forward > 0:
        rng = np.random.default_rng(0)
        x = np.zeros((1, net.nr, net.ns, INPUTS), np.float32)
        x[..., :7] = rng.uniform(-1.0, 1.0, (1, net.nr, net.ns, 7))
        bits = (np.ascontiguousarray(x).view(np.uint32) >> 16).astype(np.uint16)
        net.forward(bits)
        t1 = time.time()
        for _ in range(a.forward):
            net.forward(bits)
        print(f"{a.forward} forward passes of {net.nr}x{net.ns} in {time.time() - t1:.3f} s "
              f"(host copies included)", flush=True)
        raise SystemExit(0)
    if a.disks > 0:
        train(net, a.disks, a.steps, lr=a.lr, seed=a.seed, lr_final=a.lr_final, log=print)
        print(f"trained in {time.time() - t0:.1f} s", flush=True)
        if a.out:
            net.save(a.out)
    if a.eval_dts > 0:
        from . import workloads
        draw = {"alpha": 1.0e-3, "aspect": 0.05, "mplanet": workloads.PLANET1[0]}
        print("disk1 workload:", compare_sweeps(net, draw, a.eval_dts), flush=True)
