"""Learned starting guess for batched CG relaxation: data, training, use.

No counterpart in IMD, which starts every relaxation from the positions it
reads.  Every computation runs on the GPU through libimdgpu; this module is
the host-side sequencing only:

1. data: defect cells from the batched workload's generator are relaxed by
   the plain batched CG (imdgpu_batch_*); the target of every atom is its
   displacement, relaxed minus unrelaxed, unwrapped by the minimum image of
   its cell's box;
2. training: Adam on the per-pair MLP (imdgpu_ml_train_step: the project's
   own forward, backward and Adam kernels), one step per group of
   `batch_cells` cells; each group is one GpuBatch with its atoms at the
   unrelaxed positions, kept on the device when the training set is small
   enough and uploaded for its step otherwise, and the model's weights and
   Adam state move between the groups' handles;
3. use: imdgpu_batch_ml_start moves every cell to its predicted start where
   that lowers the cell's energy, and the plain batched CG finishes every
   cell to the same force tolerance.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import api

H, K1, NIN = 64, 32, 17
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * K1
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1

# Table interpolation of the batched relaxations: IMD's `spline` target.  With
# the default 3-point quadratic interpolation the force jumps by about
# 1e-4 eV/A where a pair crosses a grid point of a 2000-point table (the
# interpolant is continuous, its derivative is not), which is the size of
# the 1e-4 eV/A stopping force, and CG then spends most of its force calls
# in the last factor of two of the max force.
BATCH_INTERPOLATION = api.SPLINE


def init_weights(seed: int = 0) -> np.ndarray:
    """Initial parameters in the layout of imdgpu_ml_set_weights: normal
    weights scaled by 1/sqrt(fan-in) (inputs 17..31 of W1 are padding and
    stay zero), zero biases, a small output layer so that the first
    prediction is close to no displacement."""
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM, np.float32)
    w1 = rng.standard_normal((H, K1)) / np.sqrt(NIN)
    w1[:, NIN:] = 0.0
    w[OFF_W1:OFF_B1] = w1.ravel()
    w[OFF_W2:OFF_B2] = (rng.standard_normal((H, H)) / np.sqrt(H)).ravel()
    w[OFF_W3:OFF_B3] = 0.01 * rng.standard_normal(H)
    return w


def min_image(d: np.ndarray, box: np.ndarray) -> np.ndarray:
    """Displacements d (n,3) reduced to the nearest image of the periodic
    box whose rows are the box vectors."""
    s = d @ np.linalg.inv(box)
    s -= np.round(s)
    return s @ box


def make_batch(tables, cells, precision=api.FP64,
               interpolation: int = BATCH_INTERPOLATION, nbl_margin: float = 0.4) -> api.GpuBatch:
    b = api.GpuBatch(1, api.EAM2, precision, interpolation)
    b.read_tables(tables)
    b.set_cells(cells, nbl_margin)
    return b


@dataclass
class RelaxResult:
    seconds: float
    epot: np.ndarray
    fmax: np.ndarray
    nfc: np.ndarray
    steps: np.ndarray
    status: np.ndarray
    rounds: int
    used: np.ndarray | None = None
    e_start: np.ndarray | None = None
    e_pred: np.ndarray | None = None
    positions: list = field(default_factory=list)
    # (seconds since the start, rounds so far, cells finished, atoms of the
    # unfinished cells) after every advance call, when relax() was asked to
    # trace
    trace: list = field(default_factory=list)
    rebuilds: int = 0   # neighbour-list rebuilds of the batch during the relaxation

    @property
    def relaxations_per_s(self) -> float:
        return len(self.epot) / self.seconds

    def tail_histogram(self, ncells: int, natoms: int, bounds=(8, 32)) -> dict:
        """Wall time, rounds and atom-rounds (one force call of one atom)
        spent while at most 8, 9-32 and more than 32 cells were unfinished;
        each traced interval counts at the cells unfinished when it began and
        at the mean of the unfinished atoms at its two ends."""
        edges = sorted(bounds)
        names = ["unfinished<=%d" % edges[0]] + \
                ["%d<unfinished<=%d" % (a, b) for a, b in zip(edges, edges[1:])] + \
                ["unfinished>%d" % edges[-1]]
        out = {k: {"seconds": 0.0, "rounds": 0, "atom_rounds": 0.0} for k in names}
        t0, r0, left, a0 = 0.0, 0, ncells, natoms
        for t, r, done, active in self.trace:
            k = sum(left > e for e in edges)
            out[names[k]]["seconds"] += t - t0
            out[names[k]]["rounds"] += r - r0
            out[names[k]]["atom_rounds"] += 0.5 * (a0 + active) * (r - r0)
            t0, r0, left, a0 = t, r, ncells - done, active
        for v in out.values():
            v["ms_per_round"] = 1e3 * v["seconds"] / v["rounds"] if v["rounds"] else None
            v["ns_per_atom_round"] = 1e9 * v["seconds"] / v["atom_rounds"] \
                if v["atom_rounds"] else None
        return out


def relax(tables, cells, fmax: float = 1e-4, weights=None, precision=api.FP64,
          keep_positions: bool = False, chunk_rounds: int = 4096,
          interpolation: int = BATCH_INTERPOLATION, nbl_margin: float = 0.4,
          trace: bool = False, start_iters: int = 1) -> RelaxResult:
    """Relax every cell with the batched CG, from the learned start when
    `weights` are given.  The wall time covers the learned start (its two
    force calls and the prediction) and the CG, not the upload of the cells.
    Force calls per cell include the learned start's two.  trace: advance
    64 rounds per call and record the progress after each (RelaxResult.trace).
    start_iters > 1 applies the learned start again from the positions it
    chose (features recomputed there), each application kept only where it
    lowers the cell's energy; two more force calls each."""
    if trace:
        chunk_rounds = 64
    b = make_batch(tables, cells, precision, interpolation, nbl_margin)
    used = e0 = e1 = None
    api.lib()
    b.calc_forces(0)  # first list and geometry outside the timed region
    t0 = time.perf_counter()
    if weights is not None:
        b.ml_set_weights(weights)
        used, e0, e1 = b.ml_start()
        for _ in range(start_iters - 1):
            u2, _, e2 = b.ml_start()
            used = np.maximum(used, u2)
            e1 = np.where(u2 == 1, e2, e1)
    b.begin(fmax)
    rounds = 0
    tr = []
    while True:
        nd, rounds = b.advance(chunk_rounds)
        if trace:
            tr.append((time.perf_counter() - t0, rounds, nd, b.progress()[1]))
        if nd >= len(cells):
            break
        if rounds > 10_000_000:
            raise RuntimeError("batched CG did not finish")
    sec = time.perf_counter() - t0
    r = b.results()
    nfc = r["nfc"] + (2 * start_iters if weights is not None else 0)
    pos = b.positions() if keep_positions else []
    nreb = b.rebuilds()
    b.close()
    return RelaxResult(sec, r["epot"], r["fmax"], nfc, r["steps"], r["status"], rounds,
                       used, e0, e1, pos, tr, nreb)


def targets(cells, relaxed_positions) -> list:
    """Per cell (n,3) displacements relaxed - unrelaxed, minimum image."""
    return [min_image(xr - c.x, np.asarray(c.box)) for c, xr in zip(cells, relaxed_positions)]


# above this many training atoms the groups are not kept on the device
RESIDENT_ATOMS = 24_000_000


class Trainer:
    """Adam training of the per-pair MLP on groups of cells."""

    def __init__(self, tables, cells, disp, batch_cells: int = 64, seed: int = 0,
                 weights=None, interpolation: int = BATCH_INTERPOLATION,
                 core_weight: float = 0.0, core_disp: float = 0.2, resident=None):
        """core_weight > 0 weights the loss of every atom whose target
        displacement is at least core_disp (A) by 1 + core_weight: the few
        defect-core atoms that set the CG cost count as much as the many
        atoms of the elastic field.  resident: keep every group's batch on
        the device (default: when the cells hold at most RESIDENT_ATOMS);
        otherwise each step uploads its group and frees it afterwards."""
        self.tables, self.interpolation = tables, interpolation
        self.core_weight, self.core_disp = core_weight, core_disp
        if resident is None:
            resident = sum(c.n for c in cells) <= RESIDENT_ATOMS
        self.resident = resident
        self.groups = []
        for g0 in range(0, len(cells), batch_cells):
            gc = cells[g0:g0 + batch_cells]
            t = np.ascontiguousarray(np.concatenate(disp[g0:g0 + batch_cells]), np.float64)
            self.groups.append((self._batch(gc, t) if resident else gc, t))
        self.w = init_weights(seed) if weights is None else np.asarray(weights, np.float32)
        self.m = np.zeros(NPARAM, np.float32)
        self.v = np.zeros(NPARAM, np.float32)
        self.step = 0
        self.rng = np.random.default_rng(seed + 1)
        self.history = []

    def _batch(self, gc, t):
        b = make_batch(self.tables, gc, interpolation=self.interpolation)
        # training needs rho and the pairs, not fast forces: no 32-byte
        # per-entry pair cache beside every resident group's list
        b.set_pair_cache(False)
        if self.core_weight > 0.0:
            core = np.sqrt(np.sum(t * t, axis=1)) >= self.core_disp
            b.ml_set_loss_weights(1.0 + self.core_weight * core)
        return b

    def _step(self, gi, lr):
        """One Adam step (lr 0: the loss alone) on group gi."""
        g, t = self.groups[gi]
        b = g if self.resident else self._batch(g, t)
        try:
            self._load(b)
            loss = b.ml_train_step(t, lr)
            if lr > 0.0:
                self._store(b)
        finally:
            if not self.resident:
                b.close()
        return loss

    def _load(self, b):
        b.ml_set_weights(self.w)
        b.ml_set_adam(self.m, self.v, self.step)

    def _store(self, b):
        self.w = b.ml_get_weights()
        self.m, self.v, self.step = b.ml_get_adam()

    def epoch(self, lr: float = 1e-3) -> float:
        """One pass over the groups in random order; mean loss before each
        group's step."""
        losses = [self._step(gi, lr) for gi in self.rng.permutation(len(self.groups))]
        m = float(np.mean(losses))
        self.history.append(m)
        return m

    def loss(self) -> float:
        """Mean loss over all groups at the current weights (no update)."""
        return float(np.mean([self._step(gi, 0.0) for gi in range(len(self.groups))]))

    def close(self):
        if self.resident:
            for b, _ in self.groups:
                b.close()
        self.groups = []


def main(argv=None):
    """python -m imd_gb300.learned [--cells 512] [--seed 6] [--rounds 0]
    [--weights imd_gb300/data/start_mlp.npz] [--engine 1] [--pair-cache 1]
    [--partial-rebuild 0]

    Relax a batch of the defect-cell workload (Sutton-Chen Cu, spline tables)
    with the batched CG, from the learned start when --weights is given, and
    print one JSON line (seconds, rounds, rebuilds, force calls, status
    counts).  --rounds N stops after N rounds (0: until every cell is done),
    for profiling the early rounds."""
    import argparse
    import json
    import os
    import tempfile
    from . import workloads as wl
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=512)
    ap.add_argument("--seed", type=int, default=6)
    ap.add_argument("--rounds", type=int, default=0)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--engine", type=int, default=1)
    ap.add_argument("--pair-cache", type=int, default=1)
    ap.add_argument("--partial-rebuild", type=int, default=0)
    a = ap.parse_args(argv)
    tabs = wl.sutton_chen_tables(os.path.join(tempfile.mkdtemp(prefix="imdrelax"), "cu"),
                                 [wl.CU])
    cells = wl.defect_batch(a.cells, seed=a.seed)
    b = make_batch(tabs, cells)
    b.set_engine(bool(a.engine))
    b.set_pair_cache(bool(a.pair_cache))
    b.set_partial_rebuild(bool(a.partial_rebuild))
    b.calc_forces(0)
    t0 = time.perf_counter()
    if a.weights:
        b.ml_set_weights(np.load(a.weights)["w"])
        b.ml_start()
    b.begin(1e-4)
    rounds = nd = 0
    while nd < len(cells) and (a.rounds <= 0 or rounds < a.rounds):
        step = 4096 if a.rounds <= 0 else min(4096, a.rounds - rounds)
        nd, rounds = b.advance(step)
    sec = time.perf_counter() - t0
    r = b.results()
    out = {"cells": len(cells), "atoms": int(sum(c.n for c in cells)), "seed": a.seed,
           "seconds": sec, "rounds": rounds, "done": nd, "rebuilds": b.rebuilds(),
           "force_calls_mean": float(r["nfc"].mean()),
           "status_counts": np.bincount(r["status"], minlength=5).tolist(),
           "relaxations_per_s": len(cells) / sec if nd >= len(cells) else None}
    b.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
