#!/usr/bin/env python
"""Benchmark of the GB300 force / neighbour-list / NVE path.

Workload (one step = one main_loop NVE step): single-species Sutton-Chen Cu
EAM2 in IMD eam2 table format (2000-point tables on r^2 from 1.5 A to 7.2 A,
cubic taper over the last 0.3 A; F table 2000 points on [0, 400]), fcc
a0 = 3.615 A, 40x40x40 cells = 256,000 atoms, mass 63.546 amu, periodic,
Maxwell momenta at 300 K (seed 2), dt = 1 fs, skin 0.4 A, FP64.  Synthetic
data, generated here deterministically.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed atom-steps/s with the state
resident in HBM (CUDA events around every step, an L2-sized scratch write
between steps outside the timed windows); `e2e` is the same metric through
the C-ABI with host buffers: every step uploads positions and momenta from
pinned host memory, runs calc_forces / move_atoms_nve / check_nblist (the
calls IMD's main_loop makes) and reads the new positions and momenta and the
step's energies back.

The same line carries the FP32-force / FP64-accumulate run of the same
workload (`mixed`, with its force error against FP64 at the same positions)
and the batched defect relaxations (`batched_cg`): relaxations/s of IMD's CG
on 512 held-out cells, plain and from the learned start (--no-mixed,
--no-batch, --batch-cells N).

--impl reference times the reference's CPU algorithm for this path on the
host cores: the C restatement in oracle/ (the reference itself is compiled
only where its sources are, which the GPU host does not have), one process
per core, a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("EAM atom-steps/s (FP32 vs FP64); defect CG relaxations/s learned vs plain")
NCELL = 40
A0 = 3.615
DT_FS = 1.0
SKIN = 0.4
WORKLOAD = "sutton-chen Cu EAM2 NVE, fcc 40^3 = 256000 atoms, 300 K, dt 1 fs, skin 0.4 A"
FORCE_BYTES_PER_ATOM = 56.0       # force kernel: read x (24) + 2F' (8), write F (24)
PAIR_BYTES_PER_ATOM = 88.0        # both pair passes: x (24) in, rho (8) out; x, 2F' in, F out
# mixed force kernel (k_force_mixed_staged), per full-list entry, loads on
# the L1/shared-memory data path: the list word (4), the partner's FP32
# (hi, lo) position split (32), the fused pair/density row (32, from shared
# memory), the partner's F' (4)
MIXED_L1_BYTES_PER_ENTRY = 72.0
NCU_L1TEX_MIXED_FORCE = 0.628     # l1tex throughput, % of peak (committed ncu profile)
NCU_FP64_PIPE_FORCE = 0.786       # FP64 pipe busy of k_force_cache (committed ncu profile)
NCU_FP64_PIPE_DENSITY = 0.848     # FP64 pipe busy of k_density_cache (committed ncu profile)
STEP_BYTES_PER_ATOM = 232.0       # whole NVE EAM step, canonical count
FLOPS_PER_PAIR = 66.0             # canonical FP64 flops per half-list pair within rc


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, nm in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def workload_files(tmp: str):
    from imd_gb300 import workloads as wl
    return wl.sutton_chen_tables(os.path.join(tmp, "cu"), [wl.CU])


def make_state():
    from imd_gb300 import workloads as wl
    return wl.eam_fcc_system(NCELL, a0=A0, T=300.0, seed=2)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def committed_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


def cpu_sample(tabs, steps: int, cores: int = 1, warm: int = 1):
    """The oracle (C restatement of the reference path) on the same workload:
    `warm` untimed NVE steps (the first list build among them), then `steps`
    timed ones, in `cores` independent processes."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.starmap(_cpu_worker, [(tabs, steps, warm)] * cores)
    n = res[0][0]
    rate = sum(n * steps / t for n, t in res)
    return rate, n


def _cpu_worker(tabs, steps, warm=1):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from imd_gb300 import workloads as wl
    from oracle import OracleSystem
    s = make_state()
    o = OracleSystem(s.box, s.x, s.types, s.mass, s.number, 1, tabs, True, SKIN,
                     timestep=DT_FS * wl.FS, p=s.p)
    o.nve(max(1, warm))   # the first build and the warm-up outside the timed sample
    t = time.perf_counter()
    o.nve(steps)
    return s.n, time.perf_counter() - t


def run_reference(args, rank, world):
    if rank != 0:
        return
    tmp = tempfile.mkdtemp(prefix="imdbench")
    tabs = workload_files(tmp)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    cores = os.cpu_count() or 1
    # the same K timed and W untimed steps as the GPU arm, in every process
    # (a full 256000-atom step takes about 0.6 s on one core)
    steps = max(1, args.steps)
    warm = max(1, args.warmup)
    rate, n = cpu_sample(tabs, steps, cores, warm)
    how = ("%d independent single-core processes, each %d untimed then %d timed NVE steps of "
           "the full 256000-atom system (oracle/imd_oracle.c, the reference's algorithm "
           "restated in C); atom-steps/s summed over processes.  IMD's serial build is one "
           "core; its OpenMP build runs slower on more threads, so independent replicas are "
           "the host's throughput baseline" % (cores, warm, steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "atom-steps/s",
        "n_gpus": world, "steps": steps, "warmup": warm, "ms_per_step": 1e3 * n / (rate / cores),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample": how},
        "cpu_baseline": {"value": rate, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                         "sample": how},
        "e2e": {"value": rate, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _cg_cpu_worker(tabs, box, x, mass):
    """IMD's CG (the C restatement, spline tables) on one cell to max |F| <= 1e-4."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from oracle import OracleSystem
    oracle.set_interpolation(oracle.SPLINE)
    n = len(x)
    o = OracleSystem(box, x, np.zeros(n, np.int32), mass, np.arange(n, dtype=np.int32), 1,
                     tabs, True, 0.4)
    t = time.perf_counter()
    # bounded: a start that IMD's CG cannot leave (a pair inside the tables'
    # first point) would otherwise run for its 100000 steps
    steps, fm = o.cg_relax(1e-4, 3000)
    return n, int(o.nfc), time.perf_counter() - t, steps >= 0 and fm <= 1e-4


def cg_cpu_sample(tabs, cells, count: int):
    """The reference's CG algorithm on the host cores: the `count` smallest
    cells of the batch, one process per cell (spawned), relaxed in parallel.
    Returns (relaxations/s of the sample, atom-force-calls/s per core, cores)."""
    import multiprocessing as mp
    order = np.argsort([c.n for c in cells], kind="stable")[:count]
    jobs = [(tabs, cells[i].box, cells[i].x, cells[i].mass) for i in order]
    cores = min(count, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.starmap(_cg_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    per_core = float(np.mean([n * nfc / t for n, nfc, t, _ in res]))
    return len(res) / wall, per_core, cores, res


def batch_force_rate(tabs, cells, reps: int = 5) -> dict:
    """One force call of every atom of the batch at once (every cell
    unfinished, the list current): device time per atom, the rate the
    relaxation's rounds are compared with."""
    from imd_gb300 import learned
    b = learned.make_batch(tabs, cells)
    b.calc_forces(0)
    b.calc_forces(0)
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        b.calc_forces(0)  # synchronous: results read back
        t.append(time.perf_counter() - t0)
    b.close()
    n = sum(c.n for c in cells)
    best = min(t)
    return {"atoms": n, "ms": 1e3 * best, "ns_per_atom": 1e9 * best / n,
            "how": "calc_forces of the whole batch, best of %d, wall clock around the "
                   "synchronous call" % reps}


def run_batch(args, tabs, rank=0, world=1, dist=None):
    """Defect CG relaxations/s, plain and from the learned start: the held-out
    cells of the learned-start workload (seed 6), each relaxed by IMD's CG
    to max |F| <= 1e-4 eV/A in one batch; the learned start uses the weights
    trained by imd_gb300/train_start.py (imd_gb300/data/start_mlp.npz).
    With N ranks the cells are sharded by atom count (no exchange while they
    relax); the time is the slowest rank's and rank 0 reports."""
    from imd_gb300 import learned, shard
    from imd_gb300 import workloads as wl
    cells = wl.defect_batch(args.batch_cells, seed=6)
    natoms = np.array([c.n for c in cells])
    mine = shard.shard_cells(natoms, world)[rank]
    wpath = os.path.join(ROOT, "imd_gb300", "data", "start_mlp.npz")
    w = np.load(wpath)["w"]
    out = {"workload": "%d Sutton-Chen Cu defect cells, %d atoms (%d-%d), 1-4 vacancies or "
                       "<100> dumbbells, +-2%% strain, 0.05 A noise, seed 6; IMD CG to max |F| "
                       "<= 1e-4 eV/A, FP64, spline tables" % (len(cells), natoms.sum(),
                                                              natoms.min(), natoms.max()),
           "unit": "relaxations/s", "sharding": "%d ranks, cells split by atom count" % world,
           "list_rebuilds": "whole batch: a round rebuilds every cell's list once any cell "
                            "moved past skin/2 (the library default; per-system rebuilds off)"}
    cells4 = wl.defect_batch(args.batch_cells, seed=4)
    natoms4 = np.array([c.n for c in cells4])
    mine4 = shard.shard_cells(natoms4, world)[rank]
    res = {}
    runs = [("plain", cells, mine, None), ("learned", cells, mine, w)]
    if not args.no_seed4:
        runs.append(("seed4", cells4, mine4, None))
    for name, cs, mi, weights in runs:
        if dist:
            dist.barrier()
        r = learned.relax(tabs, [cs[i] for i in mi], weights=weights, trace=True)
        sec = shard.max_over_ranks(r.seconds, dist)
        g = shard.gather_cell_results({"epot": r.epot, "status": r.status, "nfc": r.nfc},
                                      mi, len(cs), dist)
        res[name] = (sec, g, r)
    if rank != 0:
        return None
    for name in ("plain", "learned"):
        sec, g, r = res[name]
        out[name] = {"value": len(cells) / sec, "seconds": sec,
                     "converged": int((g["status"] == 0).sum()),
                     "converged_per_s": float((g["status"] == 0).sum() / sec),
                     "force_calls_per_relaxation": float(g["nfc"].mean()),
                     "rounds_rank0": r.rounds, "rebuilds_rank0": r.rebuilds,
                     "status_counts": np.bincount(g["status"], minlength=5).tolist(),
                     "tail_rank0": r.tail_histogram(len(mine), int(natoms[mine].sum()))}
        if name == "learned":
            out[name]["start_used_rank0"] = int(r.used.sum())
    out["full_batch_force_call"] = batch_force_rate(tabs, [cells[i] for i in mine])
    if "seed4" in res:
        sec, g, r = res["seed4"]
        out["plain_seed4"] = {
            "workload": "the batching workload's own cells: seed 4, %d cells, %d atoms, "
                        "spline tables" % (len(cells4), natoms4.sum()),
            "value": len(cells4) / sec, "seconds": sec,
            "converged": int((g["status"] == 0).sum()),
            "force_calls_per_relaxation": float(g["nfc"].mean()), "rounds_rank0": r.rounds,
            "status_counts": np.bincount(g["status"], minlength=5).tolist()}
    gp, gl = res["plain"][1], res["learned"][1]
    both = (gp["status"] == 0) & (gl["status"] == 0)
    de = np.abs(gl["epot"] - gp["epot"])[both] / natoms[both]
    out["speedup_learned_vs_plain"] = out["learned"]["value"] / out["plain"]["value"]
    if not args.no_cpu:
        try:
            rate, per_core, cores, res = cg_cpu_sample(tabs, cells, 16)
            # the whole workload on the same cores at the sample's per-core
            # rate, with the force calls the device's plain run needed
            work = float((gp["nfc"].astype(np.float64) * natoms).sum())
            out["cpu_baseline"] = {
                "value": rate, "unit": "relaxations/s", "cores": cores, "kind": "port",
                "sample": "the %d smallest of the %d cells (%d-%d atoms), IMD's CG restated in "
                          "C (oracle/imd_oracle.c), spline tables, one process per cell"
                          % (len(res), len(cells), min(r[0] for r in res), max(r[0] for r in res)),
                "atom_force_calls_per_s_per_core": per_core,
                "converged": int(sum(1 for r in res if r[3])),
                "estimated_full_workload": {
                    "value": cores * per_core * len(cells) / work, "unit": "relaxations/s",
                    "how": "cores x per-core atom-force-calls/s / (atoms x force calls) summed "
                           "over the %d cells, force calls from the device's plain run"
                           % len(cells)}}
        except Exception as e:  # the device measurement stays valid
            out["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    out["final_energy_diff_ev_per_atom"] = {"max": float(de.max()), "median": float(np.median(de)),
                                            "within_1e-6": int((de <= 1e-6).sum()),
                                            "compared": int(both.sum())}
    return out


def run_ours(args, rank, world, local):
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    api.set_device(local)
    tmp = tempfile.mkdtemp(prefix="imdbench%d" % rank)
    tabs = workload_files(tmp)
    st = make_state()
    dt = DT_FS * wl.FS
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo")
        dist = dist_mod

    def barrier():
        if dist:
            dist.barrier()

    def build(precision):
        s = api.GpuSystem(1, api.EAM2, precision)
        s.read_tables(tabs)
        s.set_box(st.box, (1, 1, 1), SKIN)
        s.set_atoms(st.number, st.types, st.mass, st.x, st.p)
        return s

    peaks, peak_kind = measured_peaks()
    res = {}
    for prec, name in ((api.FP64, "fp64"), (api.MIXED, "mixed")):
        if name == "mixed" and args.no_mixed:
            continue
        s = build(prec)
        blocks = s.autotune()   # density / force block shapes, outside the timed steps
        blocks = (blocks[0], blocks[1], s.tile())  # and the lanes per atom
        s.nve_run(max(args.warmup, 3), dt, record=False)
        s.set_profiling(True)
        s.set_l2_flush(256 << 20)
        barrier()
        with ClockSampler(local) as clk:
            ep, ek = s.nve_run(args.steps, dt)
        barrier()
        t = s.timing()
        sc = s.scalars()
        # graph replay, unflushed and unprofiled: wall time of the call
        s.set_profiling(False)
        s.set_l2_flush(0)
        s.nve_run(25, dt, record=False)
        tg = time.perf_counter()
        s.nve_run(args.steps, dt, record=False)
        graph_rate = st.n * args.steps / (time.perf_counter() - tg)
        res[name] = dict(ms=t.ms_total, ms_force=t.ms_force, ms_density=t.ms_density,
                         ms_integrate=t.ms_integrate, ms_rebuild=t.ms_rebuild,
                         rebuilds=t.rebuilds, launches=t.kernel_launches,
                         clocks=clk.summary(), etot=(ep + ek), nb=sc.nb_entries, sys=s,
                         graph_rate=graph_rate, blocks=blocks)
    r = res["fp64"]
    ms_max = r["ms"]
    if dist:
        import torch
        v = torch.tensor([ms_max], dtype=torch.float64)
        dist.all_reduce(v, op=dist.ReduceOp.MAX)
        ms_max = float(v[0])
    n = st.n
    value = n * args.steps * world / (ms_max * 1e-3)

    # ---- end to end through the C-ABI with host buffers ----
    s = r["sys"]
    e2e_steps = 0 if args.no_e2e else min(args.steps, 20)
    try:
        import torch
        xh = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        ph = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        fh = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        eh = torch.empty((n,), dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        xh, ph, fh, eh = (np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3)), np.empty(n))
    s.get_state(xh, ph, fh, eh)
    # one step through the C-ABI with host buffers (imdgpu_nve_step_host):
    # the state (positions, momenta) up from pinned memory, calc_forces,
    # move_atoms_nve with check_nblist's test, the new state down and the
    # step's energies (tot_pot_energy, tot_kin_energy) read; one call and one
    # synchronisation a step
    e_host = []
    for _ in range(3 if e2e_steps else 0):   # warm-up of the host path
        sc = s.nve_step_host(xh, ph, dt, xh, ph)
        e_host.append(sc.tot_pot_energy + sc.tot_kin_energy)
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        sc = s.nve_step_host(xh, ph, dt, xh, ph)
        e_host.append(sc.tot_pot_energy + sc.tot_kin_energy)
    t_e2e = time.perf_counter() - t0
    barrier()
    e2e = n * e2e_steps * world / t_e2e if e2e_steps else None

    # ---- precision: mixed-path forces against FP64 at the same (thermal) positions ----
    prec = None
    if not args.no_mixed:
        s.calc_forces(0)
        a64 = s.get_atoms()
        e64 = s.scalars().tot_pot_energy
        s.set_precision(api.MIXED)
        s.calc_forces(0)
        amx = s.get_atoms()
        emx = s.scalars().tot_pot_energy
        s.set_precision(api.FP64)
        prec = {"force_rel_rms_error": float(np.sqrt(np.mean((amx["f"] - a64["f"]) ** 2)
                                                     / np.mean(a64["f"] ** 2))),
                "energy_rel_error": float(abs(emx - e64) / abs(e64)),
                "positions": "the 256000-atom system after the FP64 run (300 K)"}

    # ---- roofline of the dominant kernels: the two EAM pair passes ----
    # The density and force passes are bound by the FP64 pipe (ncu: 83%
    # busy, DRAM a few per cent), so the roofline is FP64 TFLOP/s against
    # this device's measured FP64 FMA rate, the HBM figures beside it.  With
    # the pair cache the density pass evaluates the table terms the force
    # pass reads back, so the two are one unit: achieved = the canonical 66
    # flops per half-list pair within rc / the two passes' CUDA-event time.
    force_ms = r["ms_force"] / args.steps
    dens_ms = r["ms_density"] / args.steps
    pair_ms = force_ms + dens_ms
    pairs_rc = 67.0 * n  # half-list pairs within rc per atom for fcc Cu (6 shells, 134/2)
    pair_flops = FLOPS_PER_PAIR * pairs_rc
    # the FP64 roofline denominator: imdgpu_probe_fp64_peak (kernel
    # k_fp64_probe: 8 independent FMA chains per thread, 8 blocks of 256
    # threads per SM, 4096 iterations, one warm-up launch), repeated, the
    # best run kept, with the SM clock sampled during the repeats
    with ClockSampler(local) as pclk:
        probes = [api.probe_fp64_peak() for _ in range(7)]
    fp64_peak = max(probes)
    peak_how = {"kernel": "k_fp64_probe: 8 independent FP64 FMA chains per thread, "
                          "8 x 256-thread blocks per SM, 4096 iterations, after a warm-up launch",
                "repeats": len(probes), "tflops_each": probes,
                "kept": "the best", "clocks": pclk.summary()}
    pair_tflops = pair_flops / (pair_ms * 1e-3) / 1e12
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_alg = PAIR_BYTES_PER_ATOM * n / (pair_ms * 1e-3) / 1e9
    td, tf = committed_traffic("k_density_cache"), committed_traffic("k_force_cache")
    traffic = (td + tf) if (td is not None and tf is not None) else None
    step_ms = r["ms"] / args.steps
    fp64_achieved = FLOPS_PER_PAIR * pairs_rc / (step_ms * 1e-3) / 1e12

    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "fp64", "atoms": n,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "256 MiB scratch write between timed steps (outside the windows)",
                   "list_entries": r["nb"], "rebuilds_in_timed_steps": r["rebuilds"],
                   "autotuned_blocks": {"density": r["blocks"][0], "force": r["blocks"][1],
                                        "lanes_per_atom": r["blocks"][2]}},
        "clocks": r["clocks"],
        "e2e": {"value": e2e, "unit": "atom-steps/s", "h2d_bytes_per_step": 48 * n,
                "d2h_bytes_per_step": 48 * n + 16, "steps": e2e_steps,
                "per_step": "imdgpu_nve_step_host: x, p up from pinned host memory; "
                            "calc_forces, move_atoms_nve with check_nblist's test; x, p and "
                            "the energies down; one synchronisation"},
        "gpu_launches": int(r["launches"]),
        "roofline": {"bound": "fp64",
                     "kernel": "k_density_cache + k_force_cache (the EAM2 pair passes, balanced "
                               "half list, per-entry pair cache)",
                     "achieved": pair_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": pair_tflops / fp64_peak, "traffic": traffic,
                     "peak_kind": "measured on this device: FP64 FMA chains "
                                  "(imdgpu_probe_fp64_peak); MEASURED_PEAKS.json has no FP64 rate",
                     "peak_how": peak_how,
                     "flops_per_launch": pair_flops,
                     "flops_per_pair": FLOPS_PER_PAIR,
                     "ms_density": dens_ms, "ms_force": force_ms,
                     "ncu_fp64_pipe_busy": {"k_density_cache": NCU_FP64_PIPE_DENSITY,
                                            "k_force_cache": NCU_FP64_PIPE_FORCE},
                     "hbm": {"achieved": hbm_alg, "peak": hbm_peak, "unit": "GB/s",
                             "frac": hbm_alg / hbm_peak, "peak_kind": peak_kind,
                             "bytes_per_atom": PAIR_BYTES_PER_ATOM,
                             "traffic_gbs": (traffic / (pair_ms * 1e-3) / 1e9) if traffic else None},
                     "step_fp64": {"achieved_tflops": fp64_achieved,
                                   "frac": fp64_achieved / fp64_peak,
                                   "flops_per_step": FLOPS_PER_PAIR * pairs_rc}},
        "kernels_ms_per_step": {"density": r["ms_density"] / args.steps,
                                "force": force_ms, "integrate": r["ms_integrate"] / args.steps,
                                "rebuild": r["ms_rebuild"] / args.steps},
        "energy_drift_per_atom": float((r["etot"][-1] - r["etot"][0]) / n),
        "graph_replay_wall": {"value": r["graph_rate"], "unit": "atom-steps/s",
                              "note": "nve_run wall clock, CUDA-graph chunks, warm L2"},
    }
    if "mixed" in res:
        m = res["mixed"]
        mv = n * args.steps * world / (m["ms"] * 1e-3)
        # roofline of the mixed force pass (k_force_mixed_staged): ncu puts it on
        # L1/TEX (the partner gathers), with the FP64 pipe idle and DRAM at a
        # few per cent.  achieved = bytes loaded through L1/TEX per launch
        # (MIXED_L1_BYTES_PER_ENTRY x full-list entries) / the launch's CUDA
        # event time; peak = the nominal L1 load width, 128 B per SM per
        # cycle at the sampled SM clock.  Random 32-byte gathers cost more L1
        # wavefronts than bytes, so the byte fraction is lower than the
        # throughput ncu reports (ncu_l1tex_throughput), which is the figure
        # that binds.
        mforce_ms = m["ms_force"] / args.steps
        sm_mhz = (m["clocks"].get("sm_mhz") or 2070.0)
        l1_peak = 152 * 128.0 * sm_mhz * 1e6 / 1e9
        l1_bytes = MIXED_L1_BYTES_PER_ENTRY * m["nb"]
        l1_ach = l1_bytes / (mforce_ms * 1e-3) / 1e9
        mtraffic = committed_traffic("k_force_mixed")
        mixed_roof = {"bound": "l1tex",
                      "kernel": "k_force_mixed_staged (EAM2 force pass, full rows, fused table "
                                "rows in shared memory)",
                      "achieved": l1_ach, "peak": l1_peak, "unit": "GB/s",
                      "frac": l1_ach / l1_peak, "traffic": mtraffic,
                      "peak_kind": "nominal: 128 B per SM per cycle x 152 SMs at the sampled "
                                   "SM clock",
                      "bytes_per_launch": l1_bytes, "bytes_per_entry": MIXED_L1_BYTES_PER_ENTRY,
                      "list_entries": m["nb"],
                      "ncu_l1tex_throughput": NCU_L1TEX_MIXED_FORCE,
                      "hbm": {"achieved": FORCE_BYTES_PER_ATOM * n / (mforce_ms * 1e-3) / 1e9,
                              "peak": hbm_peak, "unit": "GB/s", "peak_kind": peak_kind,
                              "bytes_per_atom": FORCE_BYTES_PER_ATOM,
                              "traffic_gbs": (mtraffic / (mforce_ms * 1e-3) / 1e9)
                              if mtraffic else None}}
        mixed_roof["hbm"]["frac"] = mixed_roof["hbm"]["achieved"] / hbm_peak
        line["mixed"] = {"value": mv, "unit": "atom-steps/s", "speedup_vs_fp64": mv / value,
                         "ms_per_step": m["ms"] / args.steps,
                         "kernels_ms_per_step": {"density": m["ms_density"] / args.steps,
                                                 "force": m["ms_force"] / args.steps,
                                                 "integrate": m["ms_integrate"] / args.steps,
                                                 "rebuild": m["ms_rebuild"] / args.steps},
                         "rebuilds_in_timed_steps": m["rebuilds"],
                         "autotuned_blocks": {"density": m["blocks"][0], "force": m["blocks"][1],
                                              "lanes_per_atom": m["blocks"][2]},
                         "graph_replay_wall": m["graph_rate"],
                         "energy_drift_per_atom": float((m["etot"][-1] - m["etot"][0]) / n),
                         "vs_fp64": prec, "roofline": mixed_roof, "clocks": m["clocks"]}
    if not args.no_batch:
        bc = run_batch(args, tabs, rank, world, dist)
        if rank == 0:
            line["batched_cg"] = bc
    if rank == 0 and not args.no_cpu:
        try:
            rate, _ = cpu_sample(tabs, args.cpu_steps, 1)
            line["cpu_baseline"] = {"value": rate, "unit": "atom-steps/s", "cores": 1,
                                    "kind": "port",
                                    "sample": "%d NVE steps of the 256000-atom system on one "
                                              "core (oracle/imd_oracle.c)" % args.cpu_steps}
        except Exception as e:  # the measurement itself stays valid
            line["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-cells", type=int, default=512)
    ap.add_argument("--no-seed4", action="store_true",
                    help="skip the plain relaxation of the seed-4 batching cells")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
