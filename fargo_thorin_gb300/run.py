"""Run a FARGO_THORIN simulation with the hydro loop on the GPU.

    python -m fargo_thorin_gb300.run [-a] [-0] [-s N] [-f F] [-o DIR] in.par

The host driver of src_main/main.c:30-230 around the GPU library: it reads
the in.par and the planet configuration, sets the disk up (InitEuler, the
InitializeFromFile path, or a restart ``-s N``), then runs DTs
``begin..NTOT`` (the reference's loop runs NTOT+1 of them) and writes the
reference's output files in the reference's formats:

* every NINTERM DTs (SendOutput, Output.c:215-258; WriteDiskPolar writes
  nrad*nsec raw doubles): gasdens<N>.dat, gasvrad<N>.dat, gasvtheta<N>.dat,
  gastemper<N>.dat (energy equation) and, when asked for in the in.par,
  gasenergy, gasdivv, gasqplus, gasopacity; with pebbles gaspebbledens,
  gaspebblevrad, gaspebblevtheta; omegaframe.dat (DumpOmegaFrame);
* once: run.commandline, used_rad.dat (FillPolar1DArrays,
  SourceEuler.c:119-130), dims.dat (WriteDim, Output.c:205-213),
  gaspebblestokes0.dat and gaspebblesize0.dat (InitPebblesViaFlux,
  Pebbles.c:187-188);
* at the first DT that ends with negative values: gas{dens,vrad,vtheta,
  temper}999.dat (DetectCrash dumps; the reference writes them at the
  crashing substep itself);
* every DT: tqwk<k>.dat (UpdateLog, Force.c:27-70) when WriteTorqueFiles;
* ``-a``: the integrals of MonitorIntegral (main.c:215-219) on stdout.

The planets are integrated by the library's host N-body step, which stands
in for REBOUND; their state at each output goes to nbody.state<N>.dat
(PhysicalTime, then one line per planet: mass gas solid x y z vx vy vz),
which ``-s N`` reads back where the reference reads its REBOUND binary
nbody.simulation<N>.dat (ReboundInterface.c:211-259).  Options outside the
GPU path (Qbalance, torque maps, custom radii.dat) are refused.
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

from . import params as P
from . import workloads

FIELD = {"dens": 0, "vrad": 1, "vtheta": 2, "energy": 3, "pebbledens": 4, "pebblevrad": 5, "pebblevtheta": 6,
         "pebblesize": 7, "temper": 8, "soundspeed": 9, "pebblestokes": 11, "qplus": 12, "divv": 13, "opacity": 14,
         "label": 16}


def _yes(s) -> bool:
    return str(s)[:1] in ("Y", "y")


class Run:
    """One simulation: in.par variables, the GPU disk, the planets, the files."""

    def __init__(self, inpar_path: str, outdir: str | None = None, scaling: float = 1.0,
                 sor_eps: float | None = None, disk_factory=None):
        """``disk_factory(params)`` builds the disk; the default is the GPU
        disk (GpuDisk), and the run fails if the CUDA library is missing."""
        with open(inpar_path) as f:
            self.v = P.read_inpar(f.read())
        kw = {"scaling_factor": scaling}
        if sor_eps is not None:
            kw["sor_eps"] = sor_eps
        self.p = P.derive(self.v, **kw)
        P.check_supported(self.p)
        self.scaling = scaling
        out = outdir if outdir is not None else self.v["OUTPUTDIR"]
        self.out = out if out.endswith("/") else out + "/"
        os.makedirs(self.out, exist_ok=True)
        if os.path.exists(self.out + "radii.dat"):
            raise NotImplementedError("a custom radii.dat grid is not supported by the GPU path")
        self.ntot, self.ninterm = int(self.v["NTOT"]), int(self.v["NINTERM"])
        self.nr, self.ns = self.p.nrad, self.p.nsec
        if disk_factory is None:
            from .disk import GpuDisk as disk_factory
        self.disk = disk_factory(self.p)
        self.write_density = not str(self.v["WRITEDENSITY"])[:1] in ("N", "n")
        self.write_velocity = not str(self.v["WRITEVELOCITY"])[:1] in ("N", "n")
        self.write = {"energy": _yes(self.v["WRITEENERGY"]),
                      "temper": bool(self.p.energy_eq) or _yes(self.v["WRITETEMPERATURE"]),
                      "divv": _yes(self.v["WRITEDIVV"]), "qplus": _yes(self.v["WRITEQPLUS"]),
                      "opacity": _yes(self.v["WRITEOPACITY"])}
        if _yes(self.v["WRITEQBALANCE"]):
            raise NotImplementedError("WriteQbalance is not supported by the GPU path")
        self.write_torque = _yes(self.v["WRITETORQUEFILES"])
        self.sys = None

    # -- files -----------------------------------------------------------
    def _path(self, name):
        return self.out + name

    def write_polar(self, name: str, fid: int, number: int):
        """WriteDiskPolar: rows 0..nrad-1 as raw doubles."""
        a = self.disk.get(fid)[: self.nr * self.ns]
        a.astype("<f8").tofile(self._path(f"gas{name}{number}.dat"))

    def read_polar(self, name: str, number: int):
        """ReadfromFile (Init.c:23-57): nrad*nsec doubles, or None if absent."""
        path = self._path(f"gas{name}{number}.dat")
        if not os.path.exists(path):
            print(f"WARNING ! Can't read {path}. Restarting with t=0 settings.", file=sys.stderr)
            return None
        a = np.fromfile(path, dtype="<f8", count=self.nr * self.ns)
        if a.size != self.nr * self.ns:
            raise ValueError(f"{path} holds fewer than nrad*nsec values")
        return a

    def radii(self):
        """Radii of FillPolar1DArrays (SourceEuler.c:76-99) without radii.dat."""
        n, rmin, rmax = self.nr, self.p.rmin, self.p.rmax
        if self.p.log_grid:
            return [rmin * math.exp(i / n * math.log(rmax / rmin)) for i in range(n + 1)]
        dr = (rmax - rmin) / n
        return [rmin + dr * i for i in range(n + 1)]

    def write_setup_files(self):
        with open(self._path("used_rad.dat"), "w") as f:
            for r in self.radii():
                f.write("%.18g\n" % r)
        with open(self._path("dims.dat"), "w") as f:
            f.write("%d\t%d\t\t%d\t%d\t%f\t%d\t%d\t%d\n" % (0, 0, 0, 0, self.p.rmax, self.ntot // self.ninterm,
                                                             self.nr, self.ns))

    def send_output(self, index: int):
        """SendOutput (Output.c:215-258) plus the N-body state and OmegaFrame."""
        d = self.write_density and index or 0
        self.write_polar("dens", FIELD["dens"], d)
        vi = self.write_velocity and index or 0
        self.write_polar("vrad", FIELD["vrad"], vi)
        self.write_polar("vtheta", FIELD["vtheta"], vi)
        if self.p.label_advection:
            self.write_polar("label", FIELD["label"], index)
        for name in ("energy", "temper", "divv", "qplus", "opacity"):
            if self.write[name]:
                self.write_polar(name, FIELD[name], index)
        if self.p.pebbles:
            for name in ("pebbledens", "pebblevrad", "pebblevtheta"):
                self.write_polar(name, FIELD[name], index)
        with open(self._path(f"nbody.state{index}.dat"), "w") as f:
            f.write("%.18g\n" % self.disk.stats().physical_time)
            for k in range(self.sys.nb):
                s = self.sys
                f.write("\t".join("%.18g" % v for v in (s.mass[k], s.gas[k], s.solid[k], s.x[k], s.y[k], s.z[k],
                                                         s.vx[k], s.vy[k], s.vz[k])) + "\n")
        with open(self._path("omegaframe.dat"), "a") as f:
            f.write("%d\t%#.18g\n" % (index, self.disk.stats().omega_frame))

    def write_torques(self):
        """One tqwk<k>.dat line per planet (UpdateLog, Force.c:65-67)."""
        for k, t in enumerate(self.disk.torques()):
            with open(self._path(f"tqwk{k}.dat"), "a") as f:
                f.write("\t".join("%#.18g" % v for v in t.row()) + "\n")

    # -- set-up ----------------------------------------------------------
    def setup(self, restart: int | None = None):
        """Initialization (Init.c:59-148) and the planets (SetupReboundSimulation
        / RestartReboundSimulation)."""
        d, p = self.disk, self.p
        if restart is None:
            with open(self.v["PLANETCONFIG"]) as f:
                rows = P.read_planet_config(f.read())
            self.sys = workloads.make_planets(p, rows)
            for name in ("tqwk%d.dat" % k for k in range(self.sys.nb)):
                open(self._path(name), "w").close()
        else:
            self._restart_planets(restart)            # also sets PhysicalTime
        if p.opacity_law == 4:                        # InitOpacities (Opacity2.c:247-297)
            indir = self.v["INPUTDIR"]
            path = os.path.join(indir if indir.endswith("/") else indir + "/", "data_gasopacity_malygin.txt")
            if not os.path.exists(path):
                raise FileNotFoundError(f"Opacity file '{path}' not found. Stopping.")
            d.set_opacity_table(*P.read_opacity_table(path))
        if p.corotating:                              # OmegaFrame = GetPsysInfo (sys, FREQUENCY), main.c:161
            P.corotating_frame(p, self.sys)
            d.set_frame(p.omega_frame)
        d.init_default()                              # InitEuler (+ pebble equilibrium)
        init_file = _yes(self.v["INITIALIZEFROMFILE"])
        if init_file or restart is not None:
            rho_full = d.get(FIELD["dens"])
            if init_file:
                for key, fid in (("DENSINFILE", "dens"), ("VRADINFILE", "vrad"), ("VTHETAINFILE", "vtheta")):
                    self._upload_rows(fid, self._read_ascii(self.v[key]))
                rho_full = d.get(FIELD["dens"])
                if p.energy_eq:
                    t = self._read_ascii(self.v["TEMPERINFILE"])
                    self._upload_rows("energy", t * rho_full[: t.size] / (p.adiabind - 1.0))
            d.refresh(1)                              # RefillSigma / RefillEnergy, then the EOS
            if restart is not None:
                for name in ("dens", "vrad", "vtheta"):
                    a = self.read_polar(name, restart)
                    if a is not None:
                        self._upload_rows(name, a)
                if p.energy_eq:
                    t = self.read_polar("temper", restart)
                    if t is not None:
                        rho = d.get(FIELD["dens"])[: t.size]
                        self._upload_rows("energy", t * rho / (p.adiabind - 1.0))
                if p.label_advection:
                    lab = self.read_polar("label", restart)
                    if lab is not None:
                        self._upload_rows("label", lab)
                d.refresh(0)
                if p.corotating:                      # GetOmegaFrame (Output.c:280-310)
                    d.set_frame(self._omega_frame_at(restart))
        if self.scaling != 1.0:                       # main.c:160
            self._upload_rows("dens", d.get(FIELD["dens"])[: self.nr * self.ns] * self.scaling)
            d.refresh(0)
        self.write_setup_files()
        if p.pebbles:
            if restart is not None:                   # RestartPebbleDisk (Pebbles.c:66-75)
                for name, num in (("pebbledens", restart), ("pebblesize", 0), ("pebblevrad", restart),
                                  ("pebblevtheta", restart)):
                    a = self.read_polar(name, num)
                    if a is not None:
                        self._upload_rows(name, a)
                d.refresh(2)
            else:
                if init_file:
                    d.init_pebbles()                  # EquilPebbleDisk on the loaded gas
                self.write_polar("pebblestokes", FIELD["pebblestokes"], 0)
                self.write_polar("pebblesize", FIELD["pebblesize"], 0)

    def _upload_rows(self, name: str, rows: np.ndarray):
        fid = FIELD[name]
        full = self.disk.get(fid)
        full[: rows.size] = rows
        self.disk.upload(fid, full)

    def _read_ascii(self, path: str) -> np.ndarray:
        """ReadfromAsciiFile (Init.c:151-199): exactly nrad*nsec numbers."""
        a = np.loadtxt(path, dtype=np.float64).ravel()
        n = self.nr * self.ns
        if a.size < n:
            raise ValueError(f"Number of values in the initialization file {path} is smaller than the size of "
                             "hydrodynamic arrays")
        if a.size > n:
            raise ValueError(f"Number of values in the initialization file {path} is larger than the size of "
                             "hydrodynamic arrays")
        return a

    def _omega_frame_at(self, n: int) -> float:
        with open(self._path("omegaframe.dat")) as f:
            for line in f:
                tok = line.split()
                if tok and int(tok[0]) == n:
                    return float(tok[1])
        raise ValueError(f"Can't read entry {n} in 'omegaframe.dat' file. Aborting restart.")

    def _restart_planets(self, n: int):
        with open(self._path(f"nbody.state{n}.dat")) as f:
            lines = [ln.split() for ln in f if ln.strip()]
        t = float(lines[0][0])
        rows = [[float(x) for x in ln] for ln in lines[1:]]
        s = P.ThorinPlanets()
        s.nb = len(rows)
        for k, r in enumerate(rows):
            s.mass[k], s.gas[k], s.solid[k], s.x[k], s.y[k], s.z[k], s.vx[k], s.vy[k], s.vz[k] = r
            s.acc[k] = self.p.accretion_rate
            s.feel_disk[k] = self.p.feel_disk
        self.sys = s
        self.disk.set_time(t)

    # -- main loop -------------------------------------------------------
    def run(self, restart: int | None = None, only_init: bool = False, monitor: bool = False, log=print,
            argv=None):
        with open(self._path("run.commandline"), "w") as f:      # DumpSources, LowTasks.c:123-139
            f.write("".join(a + " " for a in (argv if argv is not None else sys.argv)))
        self.setup(restart)
        begin = restart * self.ninterm if restart is not None else 0
        crashed = False
        for i in range(begin, self.ntot + 1):
            if i % self.ninterm == 0:
                step = i // self.ninterm
                log(f"\n*** OUTPUT {step} ***")
                self.send_output(step)
                if only_init:
                    return
            self.disk.algogas(self.sys)
            if self.disk.stats().crashed and not crashed:     # DetectCrash dumps (SourceEuler.c:274-283)
                crashed = True
                log("\nCrash! at time %.12g" % self.disk.stats().physical_time)
                for name in ("dens", "vrad", "vtheta", "temper"):
                    self.write_polar(name, FIELD[name], 999)
            if self.write_torque:
                self.write_torques()
            if monitor:
                m, mom, e, _, _ = self.disk.integrals()
                log("Gas Momentum   : %.18g" % mom)
                log("Gas total Mass : %.18g" % m)
                log("Gas total Energy: %.18g" % e)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("-a", action="store_true", help="monitor the integrals (MonitorIntegral)")
    ap.add_argument("-0", dest="only_init", action="store_true", help="write the initial outputs and stop")
    ap.add_argument("-s", type=int, default=None, metavar="N", help="restart from output N")
    ap.add_argument("-f", type=float, default=1.0, metavar="F", help="scale the surface density by F")
    ap.add_argument("-o", default=None, metavar="DIR", help="override the output directory")
    ap.add_argument("inpar")
    a = ap.parse_args(argv)
    if a.f <= 0:
        ap.error("Incorrect scaling factor")
    if a.s is not None and a.s < 0:
        ap.error("Incorrect restart number")
    r = Run(a.inpar, a.o, a.f)
    r.run(restart=a.s, only_init=a.only_init, monitor=a.a, argv=sys.argv)


if __name__ == "__main__":
    main()
