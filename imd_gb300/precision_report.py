"""FP64 against FP32-force / FP64-accumulate on the binary Sutton-Chen alloy.

    python -m imd_gb300.precision_report [--cells 100] [--steps 10000]
        [--out precision.json]

Workload: species A (Cu: eps 1.2382e-2 eV, c 39.432, a 3.61 A, 63.546 amu)
and B (Ni: eps 1.5707e-2 eV, c 39.432, a 3.52 A, 58.69 amu), cross terms
with the geometric-mean eps and the arithmetic-mean a, cutoff 7.2 A with a
0.3 A cubic taper, 2000-point eam2 tables; fcc a0 = 3.57 A, cells^3 cubic
cells (4,000,000 atoms at 100), species 50/50 uniformly at random (seed 3),
Maxwell momenta at 600 K (seed 3), NVE with dt = 1 fs, skin 0.4 A.

The same start runs `steps` NVE steps once in each precision on the GPU.
Reported:
- the relative RMS force error and relative energy error of the mixed path
  against FP64 on the same positions, at the start and at the FP64 run's
  final positions;
- per path, the drift of the total energy per atom (last minus first step,
  the largest excursion, and a least-squares slope per 1000 steps);
- per path, the device time per step (nve_run with CUDA events).
Prints one JSON object and writes it to --out when given.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

from imd_gb300 import api, workloads as wl  # noqa: E402

SKIN = 0.4


def _system(tabs, st, precision, x=None):
    s = api.GpuSystem(2, api.EAM2, precision)
    s.read_tables(tabs)
    s.set_box(st.box, (1, 1, 1), SKIN)
    s.set_atoms(st.number, st.types, st.mass, st.x if x is None else x, st.p)
    return s


def force_error(tabs, st, x):
    """Mixed against FP64 forces and energy at positions x."""
    out = {}
    for prec, name in ((api.FP64, "fp64"), (api.MIXED, "mixed")):
        s = _system(tabs, st, prec, x)
        s.calc_forces(0)
        out[name] = (s.get_atoms()["f"], s.scalars().tot_pot_energy)
        s.close()
    f64, e64 = out["fp64"]
    fm, em = out["mixed"]
    return {"force_rel_rms": float(np.sqrt(np.mean((fm - f64) ** 2) / np.mean(f64 ** 2))),
            "force_max_abs_ev_per_a": float(np.abs(fm - f64).max()),
            "energy_rel": float(abs(em - e64) / abs(e64))}


def drift(etot, n):
    e = (etot - etot[0]) / n
    k = np.arange(len(e))
    slope = float(np.polyfit(k, e, 1)[0]) * 1000.0 if len(e) > 1 else 0.0
    return {"last_minus_first_ev_per_atom": float(e[-1]),
            "max_abs_excursion_ev_per_atom": float(np.abs(e).max()),
            "slope_ev_per_atom_per_1000_steps": slope}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=100)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    tmp = tempfile.mkdtemp(prefix="imdprec")
    tabs = wl.sutton_chen_tables(os.path.join(tmp, "cuni"), [wl.CU, wl.NI])
    st = wl.eam_fcc_system(a.cells, a0=3.57, T=600.0, seed=3, species=(wl.CU, wl.NI),
                           fractions=[0.5], type_seed=3)
    n = st.n
    dt = wl.FS
    rec = {"atoms": n, "steps": a.steps, "workload": "binary Sutton-Chen Cu/Ni, fcc a0 3.57 A, "
           "%d^3 cells, 50/50 (seed 3), 600 K (seed 3), dt 1 fs, skin 0.4 A" % a.cells}
    rec["start"] = force_error(tabs, st, st.x)
    final_x = None
    for prec, name in ((api.FP64, "fp64"), (api.MIXED, "mixed")):
        s = _system(tabs, st, prec)
        s.nve_run(3, dt, record=False)   # warm-up of the graphs, then the run from the start
        s.put_state(st.x, st.p)
        s.make_nblist()
        s.set_profiling(True)
        t0 = time.perf_counter()
        ep, ek = s.nve_run(a.steps, dt)
        wall = time.perf_counter() - t0
        t = s.timing()
        etot = np.asarray(ep) + np.asarray(ek)
        rec[name] = {"atom_steps_per_s": n * a.steps / (t.ms_total * 1e-3),
                     "ms_per_step": t.ms_total / a.steps, "wall_s": wall,
                     "rebuilds": t.rebuilds, "drift": drift(etot, n),
                     "epot_first": float(ep[0]), "epot_last": float(ep[-1])}
        if name == "fp64":
            xx = np.empty((n, 3))
            s.get_state(xx)
            final_x = xx
        s.close()
        print(name, json.dumps(rec[name]), flush=True)
    rec["end"] = force_error(tabs, st, final_x)
    rec["speedup_mixed_vs_fp64"] = rec["mixed"]["atom_steps_per_s"] / rec["fp64"]["atom_steps_per_s"]
    print(json.dumps(rec))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rec, f, indent=1)


if __name__ == "__main__":
    main()
