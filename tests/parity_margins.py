"""Parity margins of the GPU path against the reference's golden runs.

Not a pytest module (the parity tests in test_gpu_parity.py assert the
tolerances); this prints, for each golden case, the worst relative L2 error
of every saved field over the run, the worst relative error of the mass and
momentum integrals, and the number of SOR iteration counts and substep counts
that differ from the reference's.  Needs a GPU and the built library:

    python tests/parity_margins.py [case ...]

Default cases: the two short runs and the two long runs (200 DTs of the gas
disk at 128x384, 40 DTs of the pebble + embryo disk at 64x192).
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import harness as H  # noqa: E402
from fargo_thorin_gb300 import workloads  # noqa: E402
from fargo_thorin_gb300.disk import GpuDisk  # noqa: E402

DEFAULT = ["disk0_24x72", "disk1_32x96", "disk0_128x384_200", "disk1_64x192_40"]


def margins(name: str) -> dict:
    g = H.load(name)
    p = H.case_params(g)
    d = GpuDisk(p)
    d.init_default()
    H.opacity_table(d, g)
    nr, ns = p.nrad, p.nsec
    n = nr * ns
    H.start_state(d, p, {"dens": g["init_dens"].ravel(), "temper": g["init_temper"].ravel()})
    sys_ = workloads.make_planets(p, [tuple(g["planet"])])
    tq = g["tqwk"]
    ntot, ninterm = int(g["ntot"]), int(g["ninterm"])
    fields = H.GAS + (H.PEB if p.pebbles else []) + (["label"] if p.label_advection else [])
    worst, mass, mom, bad = {}, 0.0, 0.0, 0
    for step in range(1, ntot + 1):
        sys_.x[0], sys_.y[0] = tq[step - 1][3], tq[step - 1][4]     # the reference's planet trajectory
        d.algogas(sys_)
        st = d.stats()
        if len(g["sor_niter"]):
            bad += int(st.sor_last_niter != g["sor_niter"][step - 1])
        bad += int(st.substeps != g["substeps"][step - 1])
        m, mo, _, _, _ = d.integrals()
        mass = max(mass, abs(m / g["mass"][step - 1] - 1))
        mom = max(mom, abs(mo / g["momentum"][step - 1] - 1))
        if step % ninterm == 0:
            k = step // ninterm
            for f in fields:
                a = d.get(H.FIELD_IDS[f])[:n].reshape(nr, ns)
                if f"out{k}_{f}" in g:
                    e = H.rel_l2(a, g[f"out{k}_{f}"])
                else:
                    e = H.rel_l2(a[g["sample_rows"]], g[f"out{k}_{f}_rows"])
                worst[f] = max(worst.get(f, 0.0), e)
    d.close()
    return {"integer_mismatches": bad, "mass": mass, "momentum": mom, "fields": worst}


def main(argv):
    for name in argv or DEFAULT:
        r = margins(name)
        fields = " ".join(f"{k} {v:.2e}" for k, v in r["fields"].items())
        print(f"{name}: integer mismatches {r['integer_mismatches']}, mass {r['mass']:.2e}, "
              f"momentum {r['momentum']:.2e}, {fields}", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
