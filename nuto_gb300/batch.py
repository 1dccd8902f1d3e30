"""Batched independent specimens: many small problems of uneven size assembled and solved as one system.

A batch concatenates the specimens' meshes into one cell group: cells of specimen 0 first, then specimen 1, ...;
coordinate nodes offset likewise, and each specimen translated to its own place on a grid so that no two specimens
touch (NuTo's AddDofInterpolation merges DOF nodes at equal coordinates). Every kernel of the path -- residual,
tangent, history, the Krylov solver and its multigrid -- then runs once over all cells and DOFs of the batch per
launch. The work unit of every launch is the cell (or the node row), not the specimen, so specimens of uneven size
need no load balancing: a plate of 120 x 120 cells and one of 20 x 20 are the same stream of cells. The matrix is
block diagonal with one block per specimen; the multigrid's aggregates never cross a specimen because no matrix
entry does.

Equivalence to solving each specimen alone (what NuTo's QuasistaticSolver does per problem,
nuto/mechanics/tools/QuasistaticSolver.cpp:51-147):
- DOF numbering: the first-touch numbering of the concatenated cells (DofNumbering::Build,
  nuto/mechanics/dofs/DofNumbering.cpp:7-58) is every specimen's own numbering shifted by the DOF count of the
  specimens before it, per DOF type; `BatchSetup.split_state` undoes the shift.
- Newton test: with an absolute tolerance (newton_atol, newton_rtol = 0) the batch iterates until the combined
  |C^T r| < atol; every specimen's own |C^T r| is a part of that norm, so each meets the same tolerance alone.
  Specimens that converge early receive further Newton updates that keep them within it. (A relative tolerance
  refers to the combined first residual, which the largest specimens dominate.)
- Time steps are shared: a NoConvergence of the batch cuts the step back for every specimen (AdaptiveSolve,
  nuto/mechanics/tools/AdaptiveSolve.cpp:18-67, applied to the batch).

    python -m nuto_gb300.batch [--specimens 128] [--seed 0] [--steps 10]

solves a seeded batch of notched plates (side n ~ U{20..120} cells, notch depth ~ U[0.2, 0.5] of the width; the
per-specimen problem is configs.notched_plate) and prints one JSON line with its size and throughput.
"""

import argparse
import json
import time
from dataclasses import dataclass, field

import numpy as np

from . import configs
from . import mesh as M


@dataclass
class SpecimenRange:
    cells: tuple        # (first cell, end) in the batch
    dofs: list          # per DOF layer: (first DOF number, end) in that layer's numbering of the batch


@dataclass
class BatchSetup(configs.Setup):
    """A Setup whose mesh is the concatenation of several specimens' meshes."""

    specimens: list = field(default_factory=list)
    layer_dofs: list = field(default_factory=list)  # DOFs per layer (combined vector: [layer 0 | layer 1 | ...])

    def split_state(self, x):
        """Combined state vector of the batch -> list of each specimen's vector in its own [layer 0 | layer 1]
        order."""
        base = np.concatenate([[0], np.cumsum(self.layer_dofs)])
        out = []
        for r in self.specimens:
            out.append(np.concatenate([x[base[l] + a: base[l] + b] for l, (a, b) in enumerate(r.dofs)]))
        return out

    def split_history(self, kappa):
        """History [cell, ip] of the batch -> list of each specimen's history."""
        return [kappa[a:b] for a, b in (r.cells for r in self.specimens)]


def concatenate(setups, name=None):
    """One BatchSetup from specimens that share the cell type, the DOF layers, the integration order, the integrand
    and the load schedule. Each specimen keeps its own constraints (dependent DOFs and right-hand sides)."""
    if not setups:
        raise ValueError("a batch needs at least one specimen")
    s0 = setups[0]
    nl = len(s0.layers)
    for s in setups:
        if (s.mesh.dim, s.mesh.geo_interp, s.gauss, len(s.layers)) != (s0.mesh.dim, s0.mesh.geo_interp, s0.gauss, nl):
            raise ValueError("specimens differ in cell type, integration order or DOF layers")
        if s.integrand != s0.integrand or (s.load_steps, s.t_end) != (s0.load_steps, s0.t_end):
            raise ValueError("specimens differ in integrand or load schedule")
        for a, b in zip(s.layers, s0.layers):
            La, Lb = s.mesh.layers[a], s0.mesh.layers[b]
            if (La.ncomp, La.interp) != (Lb.ncomp, Lb.interp):
                raise ValueError("specimens differ in a DOF layer's components or interpolation")
    # specimen i at grid place (i % cols, i // cols) with a pitch of 1.5 times the largest extent
    lo = [s.mesh.coords.min(axis=0) for s in setups]
    ext = max(float((s.mesh.coords.max(axis=0) - l).max()) for s, l in zip(setups, lo))
    pitch = 1.5 * ext if ext > 0 else 1.0
    cols = int(np.ceil(np.sqrt(len(setups))))
    coords, conn, node0 = [], [], 0
    for i, (s, l) in enumerate(zip(setups, lo)):
        shift = np.zeros(s.mesh.dim)
        shift[0], shift[1] = (i % cols) * pitch, (i // cols) * pitch
        coords.append(s.mesh.coords - l + shift)
        conn.append(s.mesh.conn.astype(np.int64) + node0)
        node0 += s.mesh.coords.shape[0]
    m = M.MeshFem(s0.mesh.dim, s0.mesh.geo_interp, np.concatenate(coords), np.concatenate(conn))
    layers = [M.add_dof_interpolation(m, s0.mesh.layers[l].ncomp, s0.mesh.layers[l].interp) for l in s0.layers]
    # per layer: the specimens' constraints with their DOF numbers shifted by the DOFs of the specimens before
    cons, ranges = [], []
    offs = [0] * nl
    cell0 = 0
    for s in setups:
        r = SpecimenRange((cell0, cell0 + s.mesh.num_cells), [])
        for k in range(nl):
            nk = s.mesh.layers[s.layers[k]].num_dofs
            r.dofs.append((offs[k], offs[k] + nk))
        ranges.append(r)
        cell0 += s.mesh.num_cells
        cons.append([(c[0].astype(np.int64) + offs[k], c[1], c[2]) for k, c in enumerate(s.constraints)])
        for k in range(nl):
            offs[k] += s.mesh.layers[s.layers[k]].num_dofs
    merged = []
    for k in range(nl):
        parts = [c[k] for c in cons]
        merged.append((np.concatenate([p[0] for p in parts]).astype(np.int32),
                       np.concatenate([p[1] for p in parts]), np.concatenate([p[2] for p in parts])))
    # the first-touch numbering of the concatenation is the specimens' numberings shifted (checked, not assumed)
    for k in range(nl):
        shift = np.cumsum([0] + [q.mesh.layers[q.layers[k]].num_nodes for q in setups[:-1]])
        expect = np.concatenate([q.mesh.layers[q.layers[k]].conn.astype(np.int64) + o for q, o in zip(setups, shift)])
        if not np.array_equal(m.layers[layers[k]].conn, expect):
            raise AssertionError("first-touch numbering of the batch is not the shifted specimen numbering")
    h0 = None
    if any(s.history0 is not None for s in setups):
        n_ip = s0.gauss ** s0.mesh.dim
        h0 = np.concatenate([s.history0 if s.history0 is not None else np.zeros((s.mesh.num_cells, n_ip))
                             for s in setups])
    return BatchSetup(name or "batch_of_%d" % len(setups), m, layers, s0.gauss, dict(s0.integrand), merged,
                      s0.load_steps, s0.t_end, h0, ranges, list(offs))


def notched_plate_batch(count, seed=0, n_range=(20, 120), depth_range=(0.2, 0.5), u_end=2e-4, load_steps=10):
    """Seeded batch of notched plates: side n ~ U{n_range} cells (inclusive), notch depth ~ U[depth_range] of the
    width (numpy default_rng(seed): n drawn first for all specimens, then the depths)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=count)
    depths = rng.uniform(depth_range[0], depth_range[1], size=count)
    plates = [configs.notched_plate(int(n), float(d), u_end, load_steps) for n, d in zip(ns, depths)]
    return concatenate(plates, "notched_plates_%d_seed%d" % (count, seed)), ns, depths


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--specimens", type=int, default=128)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--precision", type=int, default=32, choices=(32, 64))
    a = p.parse_args()
    import torch

    from .adaptive import AdaptiveSolve

    t0 = time.perf_counter()
    b, ns, depths = notched_plate_batch(a.specimens, a.seed, load_steps=a.steps)
    g = b.build_gpu()
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    g.set_state(None, 0.0, True)
    o = g.default_options(precision=a.precision, newton_rtol=1e-8, krylov_rtol=1e-3, max_newton=20,
                          max_krylov=20000)
    dt = 1.0 / a.steps
    t_end = 0.0
    for _ in range(a.steps):  # the end time as the time steps add up, so that the last step ends on it
        t_end += dt
    solver = AdaptiveSolve(g, o, dt=dt, dt_max=dt)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    steps = solver.solve(t_end)
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    newton = sum(st["newton_iterations"] for st in solver.stats)
    krylov = sum(st["krylov_iterations"] for st in solver.stats)
    assemblies = sum(st["matrix_assemblies"] for st in solver.stats)
    damaged = sum(1 for k in b.split_history(g.history) if k.max() > b.integrand["kappa0"])
    print(json.dumps({
        "workload": b.name, "specimens": a.specimens, "cells": int(b.mesh.num_cells), "dofs": int(g.n_dofs),
        "nnz": int(g.nnz), "side_cells_min_max": [int(ns.min()), int(ns.max())],
        "precision": "FP%d tangent" % a.precision, "load_steps": steps, "cutbacks": solver.cutbacks,
        "newton_iterations": newton, "krylov_iterations": krylov, "tangent_assemblies": assemblies,
        "ms_total": ms, "ms_per_load_step": ms / max(steps, 1), "ms_per_newton_iteration": ms / max(newton, 1),
        "assembled_dofs_per_s": g.n_dofs * assemblies / (ms * 1e-3),
        "specimen_load_steps_per_s": a.specimens * steps / (ms * 1e-3), "specimens_damaged": damaged,
        "setup_s": t_setup, "device": torch.cuda.get_device_name(0)}))


if __name__ == "__main__":
    main()
