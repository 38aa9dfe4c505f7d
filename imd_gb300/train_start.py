"""Train the learned CG start on the GPU and store its weights.

    python -m imd_gb300.train_start [--train-cells 2048] [--epochs 20]
        [--batch-cells 64] [--lr 1e-3] [--out imd_gb300/data/start_mlp.npz]
        [--eval-cells 512] [--relax-chunk 512] [--start-iters 1] [--max-mean-disp2 0]

Training cells come from the batched-relaxation generator with seed 5, held-out
cells with seed 6 (single-species Sutton-Chen Cu, 1-4 vacancies or <100>
dumbbells per cell, +-2% strain, 0.05 A noise, 500-20,000 atoms).  Every
training cell is relaxed by the plain batched CG to max |F| <= 1e-4 eV/A,
512 cells per batch.  Its relaxed-minus-unrelaxed displacements are the
targets.  Adam then trains the per-pair MLP on the device for `epochs`
passes over groups of `batch_cells` cells.  The output file holds the FP32
weights (`w`) and a record of the run; imd_gb300/learned.py and bench.py
load it.  With --eval-cells > 0 the held-out cells are relaxed once plainly
and once from the learned start, and the comparison is stored too.
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

from imd_gb300 import learned, workloads as wl  # noqa: E402

DEFAULT_OUT = os.path.join(HERE, "data", "start_mlp.npz")


def relax_targets(tabs, cells, chunk: int = 512, max_mean_disp2: float = 0.0):
    """Plain batched CG of `cells` in batches of `chunk`; displacement targets.
    A cell whose mean squared displacement exceeds max_mean_disp2 (A^2; 0:
    no limit) gives no target; every batch's record names its cells with the
    largest targets (index, atoms, mean |d|^2, max |d|, |mean d|, force calls)."""
    disp, stats = [], []
    for c0 in range(0, len(cells), chunk):
        part = cells[c0:c0 + chunk]
        r = learned.relax(tabs, part, keep_positions=True)
        # cells that did not relax (status != 0) give no target
        d = learned.targets(part, r.positions)
        m2 = np.array([float(np.mean(np.sum(x * x, axis=1))) for x in d])
        keep = (r.status == 0) & ((m2 <= max_mean_disp2) if max_mean_disp2 > 0 else True)
        disp += [d[k] if keep[k] else None for k in range(len(part))]
        top = np.argsort(-np.where(r.status == 0, m2, -1.0))[:8]
        stats.append({"cells": len(part), "seconds": r.seconds, "rounds": r.rounds,
                      "nfc_mean": float(r.nfc.mean()),
                      "status": np.bincount(r.status, minlength=5).tolist(),
                      "mean_disp2_cells": float(m2[r.status == 0].mean()),
                      "dropped_large": int(((r.status == 0) & ~keep).sum()),
                      "largest": [[int(c0 + k), int(part[k].n), float(m2[k]),
                                   float(np.sqrt(np.max(np.sum(d[k] ** 2, axis=1)))),
                                   float(np.linalg.norm(d[k].mean(axis=0))), int(r.nfc[k])]
                                  for k in top]})
        print("relaxed %d/%d cells: %.1f s, %d rounds, %.0f force calls per cell"
              % (c0 + len(part), len(cells), r.seconds, r.rounds, r.nfc.mean()), flush=True)
    return disp, stats


def evaluate(tabs, cells, w, start_iters: int = 1, plain=None):
    """Held-out cells relaxed plainly and from the learned start."""
    plain = plain or learned.relax(tabs, cells)
    ml = learned.relax(tabs, cells, weights=w, start_iters=start_iters)
    n = np.array([c.n for c in cells])
    both = (plain.status == 0) & (ml.status == 0)
    de = (ml.epot - plain.epot)[both] / n[both]
    return {
        "cells": len(cells), "atoms": int(n.sum()), "start_iters": start_iters,
        "plain_seconds": plain.seconds, "learned_seconds": ml.seconds,
        "plain_relaxations_per_s": plain.relaxations_per_s,
        "learned_relaxations_per_s": ml.relaxations_per_s,
        "speedup": ml.relaxations_per_s / plain.relaxations_per_s,
        "plain_converged": int((plain.status == 0).sum()),
        "learned_converged": int((ml.status == 0).sum()),
        "plain_nfc_mean": float(plain.nfc.mean()), "learned_nfc_mean": float(ml.nfc.mean()),
        "plain_nfc_sum_atoms": float((plain.nfc * n).sum()),
        "learned_nfc_sum_atoms": float((ml.nfc * n).sum()),
        "plain_rounds": plain.rounds, "learned_rounds": ml.rounds,
        "start_used": int(ml.used.sum()),
        "start_energy_gain_ev_per_atom_mean": float(((ml.e_start - ml.e_pred) / n)[ml.used == 1].mean())
        if ml.used.any() else 0.0,
        "final_energy_diff_ev_per_atom_max": float(np.abs(de).max()) if both.any() else None,
        "final_energy_diff_ev_per_atom_mean": float(de.mean()) if both.any() else None,
        "final_energy_within_1e-6": int((np.abs(de) <= 1e-6).sum()),
        "status_plain": np.bincount(plain.status, minlength=5).tolist(),
        "status_learned": np.bincount(ml.status, minlength=5).tolist(),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-cells", type=int, default=2048)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch-cells", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval-cells", type=int, default=512)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--core-weight", default="0",
                    help="extra loss weight of atoms displaced by >= --core-disp A; a comma "
                         "list trains one model per weight on the same targets, each written "
                         "to --out with _cw<weight> before the extension")
    ap.add_argument("--core-disp", type=float, default=0.2)
    ap.add_argument("--relax-chunk", type=int, default=512,
                    help="training cells relaxed per batch when making the targets")
    ap.add_argument("--max-mean-disp2", type=float, default=0.0,
                    help="drop cells whose mean squared target exceeds this (A^2; 0: keep all)")
    ap.add_argument("--start-iters", type=int, default=1,
                    help="also evaluate the learned start applied this many times")
    a = ap.parse_args(argv)
    tmp = tempfile.mkdtemp(prefix="imdtrain")
    tabs = wl.sutton_chen_tables(os.path.join(tmp, "cu"), [wl.CU])
    t0 = time.perf_counter()
    train = wl.defect_batch(a.train_cells, seed=5)
    disp, relax_stats = relax_targets(tabs, train, a.relax_chunk, a.max_mean_disp2)
    train = [c for c, d in zip(train, disp) if d is not None]
    disp = [d for d in disp if d is not None]
    t_data = time.perf_counter() - t0
    weights = [float(v) for v in str(a.core_weight).split(",")]
    held = plain = None
    if a.eval_cells > 0:
        held = wl.defect_batch(a.eval_cells, seed=6)
        plain = learned.relax(tabs, held)
    for cw in weights:
        out = a.out
        if len(weights) > 1:
            root, ext = os.path.splitext(a.out)
            out = "%s_cw%g%s" % (root, cw, ext)
        train_one(a, tabs, train, disp, cw, t_data, relax_stats, held, plain, out)


def train_one(a, tabs, train, disp, core_weight, t_data, relax_stats, held, plain, out):
    t1 = time.perf_counter()
    tr = learned.Trainer(tabs, train, disp, batch_cells=a.batch_cells, seed=a.seed,
                         core_weight=core_weight, core_disp=a.core_disp)
    loss0 = tr.loss()
    for ep in range(a.epochs):
        m = tr.epoch(a.lr)
        print("core weight %g, epoch %d: mean loss %.6e" % (core_weight, ep + 1, m), flush=True)
    loss1 = tr.loss()
    w = tr.w.copy()
    steps = tr.step
    resident = tr.resident
    tr.close()
    t_train = time.perf_counter() - t1
    # the same loss with zero displacement: mean |target|^2 per atom
    zero = float(np.mean([np.mean(np.sum(d * d, axis=1)) for d in disp]))
    rec = {"train_cells": a.train_cells, "train_cells_relaxed": len(train),
           "train_atoms": int(sum(c.n for c in train)),
           "epochs": a.epochs, "batch_cells": a.batch_cells, "lr": a.lr, "adam_steps": steps,
           "groups_resident": resident,
           "core_weight": core_weight, "core_disp": a.core_disp,
           "loss_weighted": core_weight > 0.0,
           "loss_initial": loss0, "loss_final": loss1, "loss_zero_prediction": zero,
           "loss_history": tr.history, "seconds_data": t_data, "seconds_train": t_train,
           "relax_batches": relax_stats}
    if held is not None:
        rec["eval"] = evaluate(tabs, held, w, plain=plain)
        print(json.dumps(rec["eval"]), flush=True)
        if a.start_iters > 1:
            rec["eval_iterated"] = evaluate(tabs, held, w, start_iters=a.start_iters, plain=plain)
            print(json.dumps(rec["eval_iterated"]), flush=True)
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    np.savez(out, w=w, record=json.dumps(rec))
    print("wrote %s (loss %.3e -> %.3e; zero prediction %.3e)" % (out, loss0, loss1, zero),
          flush=True)


if __name__ == "__main__":
    main()
