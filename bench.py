"""Benchmark: element assembly and quasistatic Newton solve of the 3D implicit gradient-damage beam (Hex8, 64^3 cells,
1.1 M DOFs) on GB300.

Headline (value, --steps / --warmup): a step is one assembly pass of the beam's Newton iteration, the FP32 tangent
(SimpleAssembler::BuildMatrix of GradientDamage::Hessian0) and the FP64 internal-force residual (BuildVector of
GradientDamage::Gradient), at a seeded damaged state (loading, unloading, damaged and undamaged integration points
mixed); state, history and the CSR values resident in HBM. value = DOFs x assembly passes / s ("assembled DOFs/s").
e2e        the same passes through the C ABI with host buffers: the state copied in from pinned host memory, the
           tangent's CSR values and the residual copied back to pinned host memory, every step.
roofline   the FP32 tangent kernel(s) of the pass: algorithmic bytes per assembly / mean CUDA-event duration.
cpu_baseline / --impl reference
           the oracle (the CPU restatement of NuTo's OpenMP SimpleAssembler with the same integrand and laws) doing
           the same passes on the same 64^3 beam at the same state, on the host cores.
newton     the benchmark spec's targets on the full load schedule: the 20 load steps to u_z = 2e-3 m from rest
           (QuasistaticSolver::DoStep each: trial state, Newton with line search to |C^T r| <= 1e-8 |C^T (r + K db)|,
           history update) once on the mixed-precision path (FP32 tangent, FP32 GMRES + multigrid, FP64 residual and
           history) and once on the plain FP64 GPU path, Newton-step times, the phase split, and both final states
           against an FP64 solution of the same schedule converged to 1e-11; plus the mixed schedule end to end
           through nuto_gpu_do_step_host.

--workload plates  (not the headline) the batched workload instead: --specimens seeded notched plates (2D
           gradient damage, side 20..120 cells) solved as one system through their 10 load steps; value = DOFs x
           load steps / s, next to the FP64 path and the oracle solving plates of the same batch one by one.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton-step time & assembled DOFs/s, FP32-tangent vs FP64 GPU at 1e-8 residual"
LOAD_STEPS = 20
# inexact Newton: each inner Krylov solve (both precisions) reduces its residual by 1e3; Newton on the FP64 residual
# then converges linearly at about max(1e-3, rounding of the FP32 tangent) per iteration
KRYLOV_RTOL = 1e-3
# mixed path: the Newton iterations with |C^T r| below 1e4 x the tolerance assemble the FP64 tangent and refine the
# FP32 solves against it (exact Jacobian for the last steps; the relative displacement error against the converged
# FP64 solution then stays below 1e-6, with the FP32 tangent alone it is about 1e-5 on the damaged beam)
EXACT_BELOW = 1.0e4
# forcing-term floor of both paths' Newton loops: the last linear solve of a load step leaves a linear residual of
# about FORCING_FLOOR x the Newton tolerance, so the converged state sits that far below the 1e-8 test
FORCING_FLOOR = 0.05
# the FP32 tangent's kernels per form the autotuner can choose (nuto_gpu_autotune_info)
TANGENT_KERNELS = {
    "cell_matrices": "k_cell_matrices_law<3,8,8,GD,W> + k_rows_from_cells32 (law and element matrix per cell, "
                     "then one warp per node adds its cells' slabs into its rows)",
    "node_rows": "k_point_records + k_tangent_fused<3,8,8,GD,STAGED,W> (per-point records, one warp per node "
                 "integrates its node-pair blocks)",
    "pipelined": "k_point_records + k_tangent_rows_pipe<3,8,8,GD,W> (node rows on resident blocks)",
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=None, help="cells per side (beam: 64, hex20: 80)")
    p.add_argument("--skip-fp64", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--skip-newton", action="store_true")
    p.add_argument("--skip-adjoint", action="store_true")
    p.add_argument("--load-steps", type=int, default=None,
                   help="run only the first N load steps of the 20-step Newton schedule (profiling of small cases)")
    p.add_argument("--workload", default="beam", choices=["beam", "plates", "hex20"])
    p.add_argument("--specimens", type=int, default=128)
    p.add_argument("--max-newton", type=int, default=None,
                   help="Newton iterations per load step before a cut-back (beam: 20, hex20: 50)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def aggregate_ranks(values, seconds, device):
    """Whole-job figures over replica ranks: each entry of `values` summed over the ranks (all_reduce SUM), and the
    slowest rank's time (all_reduce MAX). A single process, or no process group, returns its own figures."""
    import torch
    import torch.distributed as tdist

    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return [float(v) for v in values], float(seconds)
    w = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    tdist.all_reduce(w, op=tdist.ReduceOp.SUM)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(v) for v in w.tolist()], float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.idx)], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names[1:], f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [v for v in vis.split(",") if v.strip()]
        if local_rank < len(ids) and ids[local_rank].strip().isdigit():
            return int(ids[local_rank])
    return local_rank


def spmv_bytes(g, value_bytes):
    """Bytes the node SpMV on the padded pair layout must move once: the padded values, per slot pair and node the
    neighbour range (int64 pointer) and the block offset (int64), the neighbour columns (int32, replacing column
    indices), the constraint mask, x read once and y written once."""
    n = g.n_dofs
    padded, entries = g.solver_layout()
    layers = [g.mesh.layers[l] for l in g.layers]
    per_node = sum(L.num_nodes for L in layers) * len(layers) * (8 + 8)
    return padded * value_bytes + entries * 4 + per_node + n * (1 + 2 * value_bytes)


def tangent_bytes(setup, nnz, value_bytes):
    """Compulsory traffic of one tangent assembly: values written once, connectivity, coordinates, DOF values and
    history read once."""
    m = setup.mesh
    conn = sum(m.layers[l].conn.size for l in setup.layers) * 4 + m.conn.size * 4
    n_ip = setup.gauss ** m.dim
    return nnz * value_bytes + conn + m.coords.size * 8 + setup.n_dofs * 8 + m.num_cells * n_ip * 8


def residual_bytes(setup):
    """Compulsory traffic of one FP64 residual: the vector written once, connectivity, coordinates, DOF values and
    history read once."""
    m = setup.mesh
    conn = sum(m.layers[l].conn.size for l in setup.layers) * 4 + m.conn.size * 4
    n_ip = setup.gauss ** m.dim
    return setup.n_dofs * 8 + conn + m.coords.size * 8 + setup.n_dofs * 8 + m.num_cells * n_ip * 8


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        return json.load(open(path))
    return {}


AGG_KEYS = ("matrix_assemblies", "newton_iterations", "krylov_iterations", "ms_spmv", "spmv_launches",
            "kernel_launches", "ms_assemble_matrix", "ms_assemble_vector", "ms_krylov", "residual_evaluations")


def accumulate(t0, dt, k):
    """t0 + dt, t0 + dt + dt, ... (k values), summed as the time stepping sums them"""
    out, t = [], t0
    for _ in range(k):
        t = t + dt
        out.append(t)
    return out


def run_steps(g, opts, t_start, t_values, dt=None, progress=None, cutbacks=8):
    """Advances the load from t_start through every t in t_values with AdaptiveSolve (time step 1/LOAD_STEPS, cut
    back by halves on NoConvergence as the reference's AdaptiveSolve does). Returns the summed step statistics,
    failed attempts included (their work was done), the number of cut-backs and the per-load-step Newton counts.
    progress: a label; each finished load step then prints one line to stderr. cutbacks: halvings allowed below
    the load step."""
    from nuto_gb300.adaptive import AdaptiveSolve

    dt = dt or 1.0 / LOAD_STEPS
    ad = AdaptiveSolve(g, opts, dt=dt, dt_max=dt, dt_min=dt / 2 ** cutbacks)
    t = t_start
    per_step = []
    for tv in t_values:
        n0 = len(ad.stats)
        ad.solve(tv, t)
        per_step.append(sum(st["newton_iterations"] for st in ad.stats[n0:]))
        if progress:
            sys.stderr.write("%s: t = %.4f, %d Newton, %d Krylov iterations, %d cut-backs so far\n"
                             % (progress, tv, per_step[-1], sum(st["krylov_iterations"] for st in ad.stats[n0:]),
                                ad.cutbacks))
            sys.stderr.flush()
        t = tv
    agg = {k: 0 for k in AGG_KEYS}
    for st in ad.stats:
        for k in agg:
            agg[k] += st[k]
    agg["cutbacks"] = ad.cutbacks
    agg["do_steps"] = len(ad.stats)
    agg["newton_per_load_step"] = per_step
    return agg


# the seeded state of the assembly passes: the beam's uniaxial field at load factor 0.5 (u_z = eps z, lateral
# contraction -nu eps (x - 1/2), eps = 0.5 * 2e-3 / 4) with every displacement perturbed by up to +-20 % of eps times
# the cell size, nodal eeq ~ U(0, 4e-4) and history kappa ~ U(0, 4e-4) per integration point: loading and unloading
# points, damaged (kappa >= kappa0 = 1e-4) and undamaged ones, all mixed
STATE_SEED = 0
STATE_EPS = 0.5 * 2e-3 / 4.0


def beam_state(u_coords, u_dofs, e_dofs, n_dofs, n_cells, n_ip, n, seed=STATE_SEED):
    """(state vector, kappa[cell, ip]) of the assembly passes from plain arrays: displacement node coordinates and DOF
    numbers (n_nodes x 3), eeq DOF numbers (n_nodes), the problem's size. Both arms call it with the arrays of their
    own set-up (the DOF numbering is the same, bit for bit)."""
    rng = np.random.default_rng(seed)
    x = np.zeros(n_dofs)
    h = 1.0 / n
    eps = STATE_EPS
    field = np.stack([-0.2 * eps * (u_coords[:, 0] - 0.5), -0.2 * eps * (u_coords[:, 1] - 0.5),
                      eps * u_coords[:, 2]], axis=1)
    field += rng.uniform(-0.2, 0.2, field.shape) * eps * h
    x[np.asarray(u_dofs).reshape(-1)] = field.reshape(-1)
    x[np.asarray(e_dofs).reshape(-1)] = rng.uniform(0.0, 4e-4, np.asarray(e_dofs).size)
    kappa = rng.uniform(0.0, 4e-4, (n_cells, n_ip))
    return x, kappa


def oracle_beam(n):
    """The oracle's 64^3 beam (or n^3) and its assembly-pass state."""
    from oracle import setups

    om, layers, P, cons = setups.hex8_gradient_damage(n)
    d, e = layers
    x, kappa = beam_state(om.layer_node_coords(d), om.layer_dof_numbers(d, 3), om.layer_dof_numbers(e, 1), P.n_dofs,
                          P.n_el, P.n_ip, n)
    P.kappa = kappa
    return P, x


def oracle_pass(P, x):
    """One assembly pass of the oracle: BuildMatrix (triplets per thread, sorted and summed into the combined CSC
    matrix, released) and BuildVector. Returns (seconds of the matrix, seconds of the vector); oracle_pass.nnz holds
    the matrix's nonzeros."""
    from oracle.core import _dp

    xa = np.ascontiguousarray(x)
    t0 = time.perf_counter()
    nnz = P.L.oracle_build_matrix(P.h, _dp(xa))
    P.L.oracle_matrix_release(P.h)
    t1 = time.perf_counter()
    P.build_vector(xa)
    t2 = time.perf_counter()
    oracle_pass.nnz = int(nnz)
    return t1 - t0, t2 - t1


def cpu_baseline(n):
    """One oracle assembly pass of the same n^3 beam at the same state on all host threads (the bounded CPU sample
    of the headline workload)."""
    from oracle.core import lib

    threads = lib().oracle_max_threads()
    lib().oracle_set_threads(threads)
    P, x = oracle_beam(n)
    tm, tv = oracle_pass(P, x)
    t = tm + tv
    return {"value": P.n_dofs / t, "unit": "DOF/s", "cores": threads, "kind": "port",
            "sample": "one assembly pass (oracle BuildMatrix with OpenMP + sorted triplets into CSC, BuildVector) "
                      "of the same %d^3 beam at the same state: %.2f s (matrix %.2f s, vector %.2f s)"
                      % (n, t, tm, tv)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle

    oracle.build()
    if args.workload == "plates":
        run_reference_plates(args)
        return
    threads = oracle.lib().oracle_max_threads()
    oracle.lib().oracle_set_threads(threads)
    args.size = args.size or 64
    P, x = oracle_beam(args.size)
    # a CPU pass has nothing to warm up but page faults: one warm-up pass whatever --warmup asks for
    for _ in range(min(args.warmup, 1)):
        oracle_pass(P, x)
    tm = tv = 0.0
    for _ in range(args.steps):
        a, b = oracle_pass(P, x)
        tm, tv = tm + a, tv + b
    total = tm + tv
    value = P.n_dofs * args.steps / total
    out = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": beam_config(args.size, P.n_dofs, oracle_pass.nnz),
           "precision": "FP64 tangent and residual",
           "ms_matrix_per_step": 1e3 * tm / args.steps, "ms_vector_per_step": 1e3 * tv / args.steps,
           "cpu_baseline": {"value": value, "unit": "DOF/s", "cores": threads, "kind": "port",
                            "sample": "%d assembly passes of the %d^3 beam (oracle BuildMatrix + BuildVector, OpenMP "
                                      "over %d threads); the reference itself cannot be built here (Eigen/Boost "
                                      "absent)" % (args.steps, args.size, threads)},
           "e2e": {"value": value, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def beam_config(n, n_dofs, nnz, world=1):
    """The headline workload, the same dictionary in both arms."""
    return {"workload": "hex8_gradient_damage_%d^3 assembly pass: Hex8 2x2x2 Gauss, beam 1x1x4 m, u + eeq, "
                        "GradientDamage(c=0.01, LinearElasticDamage(30000, 0.2, FULL), DamageLawExponential(1e-4, 100, "
                        "0.99), ModifiedMises(k=10)); one step = BuildMatrix (tangent, Hessian0) + BuildVector "
                        "(residual, Gradient) at the seeded state (uniaxial field at t = 0.5 perturbed +-20 %%, eeq "
                        "and kappa ~ U(0, 4e-4), seed %d)" % (n, STATE_SEED),
            "n_dofs": int(n_dofs), "nnz": int(nnz),
            "l2": "inputs larger than L2 (the tangent's %.0f MB of FP32 values are written every step)" % (nnz * 4 / 1e6),
            "parallelism": "replicas" if world > 1 else "none"}


def run_newton(args, s, g, barrier):
    """The benchmark spec's targets on the beam's full load schedule: the LOAD_STEPS load steps from rest to t = 1
    (u_z = 2e-3 m) on the mixed-precision path and on the plain FP64 path, each timed with CUDA events; both final
    states against an FP64 solution of the same schedule converged to 1e-11 (untimed); and the mixed schedule end
    to end through nuto_gpu_do_step_host with the state and history in pinned host memory."""
    import torch

    import nuto_gb300

    n_dofs = g.n_dofs
    t_values = accumulate(0.0, 1.0 / LOAD_STEPS, LOAD_STEPS)[:args.load_steps or LOAD_STEPS]
    common = dict(newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL, max_newton=args.max_newton or 20, max_krylov=20000,
                  forcing_floor=FORCING_FLOOR)
    opts32 = g.default_options(precision=nuto_gb300.FP32, exact_tangent_below=EXACT_BELOW, **common)
    opts64 = g.default_options(precision=nuto_gb300.FP64, **common)

    def schedule(opts):
        g.set_state(None, 0.0, True)
        g.history = s.history0
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        agg = run_steps(g, opts, 0.0, t_values)
        e1.record()
        barrier()
        x, _ = g.get_state()
        return e0.elapsed_time(e1) / 1e3, agg, x

    def summary(sec, agg):
        na = max(agg["matrix_assemblies"], 1)
        return {"seconds": sec, "newton_step_ms": 1e3 * sec / na, "load_step_ms": 1e3 * sec / len(t_values),
                "tangent_solves": agg["matrix_assemblies"], "newton_iterations": agg["newton_iterations"],
                "newton_per_load_step": agg["newton_per_load_step"], "krylov_iterations": agg["krylov_iterations"],
                "cutbacks": agg["cutbacks"], "residual_evaluations": agg["residual_evaluations"],
                "kernel_launches": agg["kernel_launches"],
                "launches_per_krylov_iteration": agg["kernel_launches"] / max(agg["krylov_iterations"], 1),
                # where a Newton step's time goes (CUDA events around the phases, summed over the schedule)
                "ms_per_newton_step": {"tangent": agg["ms_assemble_matrix"] / na,
                                       "residual": agg["ms_assemble_vector"] / na,
                                       "krylov": agg["ms_krylov"] / na,
                                       "krylov_spmv": agg["ms_spmv"] / na},
                "spmv_launches": agg["spmv_launches"],
                "spmv_mean_us": 1e3 * agg["ms_spmv"] / max(agg["spmv_launches"], 1)}

    sec32, agg32, x32 = schedule(opts32)
    out = {"schedule": "%d of the %d load steps from rest to t = 1 (u_z = 2e-3 m), AdaptiveSolve cut-back, Newton "
                       "|C^T r| <= 1e-8 |C^T (r + K db)| per load step, Eisenstat-Walker forcing with floor %g"
                       % (len(t_values), LOAD_STEPS, FORCING_FLOOR),
           "mixed": summary(sec32, agg32)}
    out["mixed"]["path"] = ("FP32 tangent (k_tangent_fused), FP32 GMRES(80) with the FP32 "
                            "multigrid, FP64 residual, history, Newton test and refinement residual; iterations "
                            "with |C^T r| < %g tol use the FP64-accurate tangent (k_tangent, FP64 law, double-float "
                            "products) for the refinement" % EXACT_BELOW)
    if not args.skip_fp64:
        sec64, agg64, x64 = schedule(opts64)
        out["fp64"] = summary(sec64, agg64)
        out["fp64"]["path"] = ("FP64 tangent (k_tangent element kernel with FP64 atomics), FP64 GMRES(80) with the "
                               "FP64 multigrid, FP64 residual and history")
        opts_t = g.default_options(precision=nuto_gb300.FP64, newton_rtol=1e-11, krylov_rtol=1e-6, max_newton=40,
                                   max_krylov=20000)
        try:
            _, _, xt = schedule(opts_t)
        except Exception as exc:  # the converged solution is a diagnostic only
            xt = None
            out["converged_fp64_error"] = str(exc)

        def rel(a, b):
            return {"max": float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)),
                    "l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}

        t = {"speedup_newton_step_mixed_vs_fp64": out["fp64"]["newton_step_ms"] / out["mixed"]["newton_step_ms"],
             "speedup_schedule_mixed_vs_fp64": sec64 / sec32,
             "mixed_vs_fp64_path": rel(x32, x64)}
        if xt is not None:
            t["mixed_vs_converged_fp64"] = rel(x32, xt)
            t["fp64_path_vs_converged_fp64"] = rel(x64, xt)
        out["targets"] = t

    # the mixed schedule end to end: state and history uploaded from pinned host memory and downloaded every step
    n_hist = s.mesh.num_cells * g.n_ip
    xa = torch.zeros(n_dofs, dtype=torch.float64, pin_memory=True)
    xb = torch.empty(n_dofs, dtype=torch.float64, pin_memory=True)
    ka = torch.empty(n_hist, dtype=torch.float64, pin_memory=True)
    kb = torch.empty(n_hist, dtype=torch.float64, pin_memory=True)
    ka.numpy()[:] = s.history0.ravel()
    g.set_state(None, 0.0, False)
    barrier()
    h0 = time.perf_counter()
    assemblies, t, dt = 0, 0.0, 1.0 / LOAD_STEPS
    step = dt
    for tv in t_values:
        while t < tv - 1e-14:  # AdaptiveSolve's cut-back on the host-buffer entry point
            tn = min(tv, t + step)
            try:
                g.do_step_host(tn, xa, ka, xb, kb, opts32)
            except nuto_gb300.NoConvergence:
                assemblies += g.stats()["matrix_assemblies"]
                step *= 0.5
                continue
            assemblies += g.stats()["matrix_assemblies"]
            xa, xb = xb, xa
            ka, kb = kb, ka
            t = tn
            step = min(dt, step * 1.5) if g.stats()["newton_iterations"] < 3 else step
    barrier()
    sec_e2e = time.perf_counter() - h0
    out["mixed_e2e"] = {"seconds": sec_e2e, "newton_step_ms": 1e3 * sec_e2e / max(assemblies, 1),
                        "h2d_bytes_per_load_step": int((n_dofs + n_hist) * 8),
                        "d2h_bytes_per_load_step": int((n_dofs + n_hist) * 8)}
    return out


def run_adjoint(n=32, checkpoint_every=2):
    """The adjoint workload at n^3 cells (unit cube, seeded lognormal modulus, 10 load steps into the damaged range,
    squared displacement misfit at 256 observed surface nodes against the response of the seed + 1 field): one
    forward with checkpoints every `checkpoint_every` load steps and one reverse sweep (transposed tangent solves,
    per-point parameter derivatives, the segments' load steps recomputed), timed with CUDA events."""
    import torch

    from nuto_gb300 import configs
    from nuto_gb300.adjoint import AdjointLoadPath

    case = configs.hex8_adjoint(n)
    s = case.setup
    g = s.build_gpu()
    t_values = accumulate(0.0, 1.0 / s.load_steps, s.load_steps)
    obs = torch.as_tensor(case.obs_dofs, device="cuda")
    truth = AdjointLoadPath(g, s.integrand, t_values).forward(case.true_scale, 1e-4, 100.0)[obs].clone()
    path = AdjointLoadPath(g, s.integrand, t_values, checkpoint_every=checkpoint_every)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    e0.record()
    x = path.forward(case.scale, 1e-4, 100.0)
    e1.record()
    r = torch.zeros_like(x)
    r[obs] = x[obs] - truth
    gE, gk, gb = path.backward(2.0 * r)
    e2.record()
    torch.cuda.synchronize()
    return {"workload": "hex8_adjoint_%d^3: %d cells, %d DOFs, %d load steps, 256 observed surface nodes"
                        % (n, s.mesh.num_cells, g.n_dofs, s.load_steps),
            "forward_s": e0.elapsed_time(e1) / 1e3, "backward_s": e1.elapsed_time(e2) / 1e3,
            "checkpoint_every": checkpoint_every, "recomputed_load_steps": path.recomputed_steps,
            "loss": float((r[obs] ** 2).sum()), "dL_dkappa0": gk, "dL_dbeta": gb,
            "dL_dE_norm": float(gE.norm()),
            "method": "FP64 Newton to |C^T r| <= 1e-12, transposed tangent solved by FP64 GMRES + multigrid to 1e-13"}


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import nuto_gb300
    from nuto_gb300 import configs

    nuto_gb300.load()
    args.size = args.size or 64
    s = configs.hex8_gradient_damage(args.size, load_steps=LOAD_STEPS, imperfection=True)
    g = s.build_gpu(device=local)
    n_dofs, nnz = g.n_dofs, g.nnz
    Ld, Le = s.mesh.layers[s.layers[0]], s.mesh.layers[s.layers[1]]

    def barrier():
        if world > 1:
            import torch.distributed as tdist

            tdist.barrier()
        torch.cuda.synchronize()

    # ---- headline: assembly passes at the seeded state, everything resident in HBM ----------------------------
    x_h, kappa_h = beam_state(Ld.node_coords, Ld.dof_numbers, Le.dof_numbers, n_dofs, s.mesh.num_cells, g.n_ip,
                              args.size)
    g.history = kappa_h
    u = torch.as_tensor(x_h, device="cuda")
    k32 = torch.empty(nnz, dtype=torch.float32, device="cuda")
    f = torch.empty(n_dofs, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        g.build_system(u, nuto_gb300.FP32, out=k32, f_out=f)
    launches0 = g.stats()["kernel_launches"]
    clocks = ClockSampler(gpu_index(local))
    clocks.start()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):  # one step: the tangent and the residual at the state, the residual beside the tangent
        g.build_system(u, nuto_gb300.FP32, out=k32, f_out=f)
    e1.record()
    barrier()
    clk = clocks.stop()
    launches = g.stats()["kernel_launches"] - launches0
    sec = e0.elapsed_time(e1) / 1e3
    (work,), sec = aggregate_ranks([n_dofs * args.steps], sec, "cuda")
    value = work / sec
    fp32_check = float(k32.abs().max().item())  # touches the result (non-finite values would show here)

    # the same K steps with the two calls in sequence, each bracketed by events on the library's stream (torch's
    # current stream): the tangent's and the residual's own launch times (the roofline below), and the gain of
    # running them side by side
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    for a, b, c in ev:
        a.record()
        g.build_matrix(u, nuto_gb300.FP32, out=k32)
        b.record()
        g.build_vector(u, out=f)
        c.record()
    barrier()
    ms_matrix = [a.elapsed_time(b) for a, b, _ in ev]
    ms_vector = [b.elapsed_time(c) for _, b, c in ev]
    ms_sequential = float(np.mean([a.elapsed_time(c) for a, _, c in ev]))

    # the same passes end to end through the C ABI with host buffers (nuto_gpu_build_system_host): state in from
    # pinned memory, CSR values and residual out to pinned memory, every step
    xp = torch.empty(n_dofs, dtype=torch.float64, pin_memory=True)
    xp.numpy()[:] = x_h
    kp = torch.empty(nnz, dtype=torch.float32, pin_memory=True)
    fp = torch.empty(n_dofs, dtype=torch.float64, pin_memory=True)
    g.build_system_host(xp, kp, fp, nuto_gb300.FP32)  # allocates the context's host-io buffers (untimed)
    barrier()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        # state in, tangent values and residual out; the values' copy overlaps the residual
        g.build_system_host(xp, kp, fp, nuto_gb300.FP32)
    barrier()
    sec_e2e = time.perf_counter() - h0
    (work_e2e,), sec_e2e = aggregate_ranks([n_dofs * args.steps], sec_e2e, "cuda")
    # the bare copy of the CSR values to pinned host memory, for scale (the floor of the end-to-end pass)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record()
    kp.copy_(k32, non_blocking=True)
    c1.record()
    torch.cuda.synchronize()
    d2h_ms = c0.elapsed_time(c1)
    e2e = {"value": work_e2e / sec_e2e, "unit": "DOF/s", "h2d_bytes_per_step": int(n_dofs * 8),
           "d2h_bytes_per_step": int(nnz * 4 + n_dofs * 8), "ms_per_step": 1e3 * sec_e2e / args.steps,
           "call": "nuto_gpu_build_system_host (host buffers, page-locked)",
           "d2h_values_ms": d2h_ms, "d2h_values_gbs": nnz * 4 / (d2h_ms / 1e3) / 1e9}

    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    tb = tangent_bytes(s, nnz, 4)
    asm_s = float(np.mean(ms_matrix)) / 1e3
    form = g.autotune_info()["tangent_form"]
    roof = {"kernel": TANGENT_KERNELS[form], "bound": "hbm", "achieved": tb / asm_s / 1e9, "peak": peak, "unit": "GB/s",
            "frac": tb / asm_s / 1e9 / peak, "peak_kind": peak_kind,
            "traffic": traffic.get("tangent_%s_bytes_per_launch" % form),
            "algorithmic_bytes_per_launch": tb, "mean_launch_ms": asm_s * 1e3,
            "assembled_dofs_per_s": n_dofs / asm_s}
    rb = residual_bytes(s)
    res_s = float(np.mean(ms_vector)) / 1e3

    out = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "config": beam_config(args.size, n_dofs, nnz, world),
           "precision": "FP32 tangent (law branch decisions in FP64), FP64 residual",
           "ms_matrix_per_step": float(np.mean(ms_matrix)), "ms_vector_per_step": float(np.mean(ms_vector)),
           "ms_per_step_sequential": ms_sequential,
           "step_form": "nuto_gpu_build_system: the FP64 residual on a second stream (%s resident blocks per SM) "
                        "beside the FP32 tangent; ms_matrix/ms_vector_per_step and the rooflines from the same K "
                        "steps run as two calls in sequence" % os.environ.get("NUTO_GPU_SYSTEM_RES_BLOCKS", "6"),
           "max_abs_tangent_value": fp32_check,
           "roofline": roof,
           "roofline_residual": {"kernel": "k_residual (FP64 internal-force vector)", "bound": "fp64",
                                 "algorithmic_bytes_per_launch": rb, "mean_launch_ms": res_s * 1e3,
                                 "achieved_gbs": rb / res_s / 1e9},
           "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if not args.skip_newton:
        out["newton"] = run_newton(args, s, g, barrier)
    # launch shapes the autotuner chose (first tangent, first Krylov products) with the times it measured, and the
    # gain over the default shapes (4 warps per block, 8 lanes per node)
    tune = g.autotune_info()
    tms = tune["tangent_ms"] + tune["tangent_pipelined_ms"] + tune["tangent_cells_ms"]
    if tune["tangent_warps"] and min(tms) > 0:
        tune["tangent_gain_over_default"] = tms[1] / min(tms)
    for k, ms in tune["spmv_ms"].items():
        if tune["spmv_lanes"][k] and min(ms) > 0:
            tune.setdefault("spmv_gain_over_default", {})[k] = ms[1] / ms[[4, 8, 16].index(tune["spmv_lanes"][k])]
    out["autotune"] = tune
    if not args.skip_adjoint and world == 1:
        try:
            out["adjoint"] = run_adjoint()
        except Exception as exc:  # an extra key: it must not hide the headline
            out["adjoint"] = {"error": str(exc)}
    if rank == 0 and world == 1 and not args.skip_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline(args.size)
        except Exception as exc:  # the CPU leg must not hide the GPU result
            out["cpu_baseline"] = {"value": None, "error": str(exc)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as tdist

        tdist.destroy_process_group()


PLATES_METRIC = "batched notched plates: DOF load steps/s (DOFs of every plate x load steps at 1e-8 residual / s)"
PLATE_STEPS = 10


def plates_cpu_sample(ns, depths, threads, budget_s=15.0):
    """The oracle (OpenMP assembly, SuperLU) solving plates of the batch one by one through the 10 load steps,
    nearest to the batch's median size first, until budget_s seconds have been spent (at least one plate); Newton to
    |C^T r| < 1e-10 (absolute; the forces are of order 1). Returns (seconds, DOF load steps, plates, iterations)."""
    from oracle import setups
    from oracle.core import lib
    from oracle.quasistatic import QuasistaticOracle

    lib().oracle_set_threads(threads)
    order = np.argsort(np.abs(ns - np.median(ns)), kind="stable")
    spent, work, count, its = 0.0, 0, 0, 0
    for i in order:
        om, layers, P, cons = setups.notched_plate(int(ns[i]), float(depths[i]))
        Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-10, max_iterations=20)
        t0 = time.perf_counter()
        for t in accumulate(0.0, 1.0 / PLATE_STEPS, PLATE_STEPS):
            its += Q.do_step(t)
        spent += time.perf_counter() - t0
        work += P.n_dofs * PLATE_STEPS
        count += 1
        if spent >= budget_s:
            break
    return spent, work, count, its


def run_reference_plates(args):
    """The reference arm of the batched workload: the oracle solving plates of the same seeded batch one by one
    (each step a bounded sample, plates nearest the median size first)."""
    from nuto_gb300 import batch
    from oracle.core import lib

    _, ns, depths = batch.notched_plate_batch(args.specimens, seed=0, load_steps=PLATE_STEPS)
    threads = lib().oracle_max_threads()
    i = int(np.argmin(ns))
    for _ in range(args.warmup):  # the smallest plate
        plates_cpu_sample(ns[i:i + 1], depths[i:i + 1], threads, budget_s=0.0)
    sec, work, count, its = 0.0, 0, 0, 0
    for _ in range(args.steps):
        s_, w_, c_, i_ = plates_cpu_sample(ns, depths, threads, budget_s=5.0)
        sec, work, count, its = sec + s_, work + w_, count + c_, its + i_
    value = work / sec
    out = {"metric": PLATES_METRIC, "value": value, "unit": "DOF load steps/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": "%d notched plates (seed 0), solved one by one" % args.specimens,
                      "parallelism": "host OpenMP"},
           "cpu_baseline": {"value": value, "unit": "DOF load steps/s", "cores": threads, "kind": "port",
                            "sample": "%d plate solves (10 load steps each; oracle assembly + SuperLU), %d Newton "
                                      "iterations; the reference itself cannot be built (Eigen/Boost absent)"
                                      % (count, its)},
           "e2e": {"value": value, "unit": "DOF load steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_plates(args):
    """The batched workload on one GPU (replicas under torchrun: rank r solves the batch of seed r)."""
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import nuto_gb300
    from nuto_gb300 import batch
    from nuto_gb300.adaptive import AdaptiveSolve

    nuto_gb300.load()
    b, ns, depths = batch.notched_plate_batch(args.specimens, seed=rank, load_steps=PLATE_STEPS)
    g = b.build_gpu(device=local)
    n_dofs, nnz = g.n_dofs, g.nnz
    dt = 1.0 / PLATE_STEPS
    t_values = accumulate(0.0, dt, PLATE_STEPS)
    opts = {32: g.default_options(precision=nuto_gb300.FP32, newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL,
                                  max_newton=20, max_krylov=20000, exact_tangent_below=EXACT_BELOW),
            64: g.default_options(precision=nuto_gb300.FP64, newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL,
                                  max_newton=20, max_krylov=20000)}

    def barrier():
        if world > 1:
            import torch.distributed as tdist

            tdist.barrier()
        torch.cuda.synchronize()

    def solve(o, t_end):
        g.set_state(None, 0.0, True)
        ad = AdaptiveSolve(g, o, dt=dt, dt_max=dt, dt_min=dt / 256)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        ad.solve(t_end)
        e1.record()
        barrier()
        agg = {k: sum(st[k] for st in ad.stats) for k in AGG_KEYS}
        agg["cutbacks"] = ad.cutbacks
        return e0.elapsed_time(e1) / 1e3, agg

    if args.warmup > 0:  # warm-up load steps from rest
        solve(opts[32], t_values[min(args.warmup, PLATE_STEPS) - 1])
    clocks = ClockSampler(gpu_index(local))
    clocks.start()
    sec32, agg32 = solve(opts[32], t_values[-1])
    clk = clocks.stop()
    x32, _ = g.get_state()
    # replicas: every rank solved its own batch (seed = rank); whole-job work over the slowest rank's time
    sec32_rank = sec32
    (work, assembled, plates), sec32 = aggregate_ranks(
        [n_dofs * PLATE_STEPS, n_dofs * agg32["matrix_assemblies"], args.specimens * PLATE_STEPS], sec32, "cuda")
    out = {"metric": PLATES_METRIC, "value": work / sec32, "unit": "DOF load steps/s",
           "n_gpus": world, "steps": PLATE_STEPS, "warmup": args.warmup, "ms_per_step": 1e3 * sec32 / PLATE_STEPS,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
           "data": "synthetic",
           "config": {"workload": "%d notched plates (seed %d): Quad4 2x2 Gauss on the unit square, side n ~ "
                                  "U{20..120} cells, notch one cell high from the left edge at mid height, depth ~ "
                                  "U[0.2, 0.5] of the width; plane-strain GradientDamage(c=0.01, "
                                  "LinearElasticDamage(30000, 0.2, FULL), DamageLawExponential(1e-4, 100, 0.99), "
                                  "ModifiedMises(k=10)); bottom u_y = 0, top u_y = 2e-4 t, 10 load steps, all plates "
                                  "in one cell group" % (args.specimens, rank),
                      "specimens": args.specimens, "cells": int(b.mesh.num_cells), "n_dofs": n_dofs, "nnz": nnz,
                      "side_cells_min_max": [int(ns.min()), int(ns.max())],
                      "newton_tolerance": "|C^T r| <= 1e-8 |C^T (r + K db)| of the load step (whole batch)",
                      "l2": "inputs larger than L2 (FP32 tangent %.0f MB)" % (nnz * 4 / 1e6),
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "newton_iterations": agg32["newton_iterations"], "tangent_solves": agg32["matrix_assemblies"],
           "krylov_iterations": agg32["krylov_iterations"], "cutbacks": agg32["cutbacks"],
           "assembled_dofs_per_s": assembled / sec32,
           "specimen_load_steps_per_s": plates / sec32,
           "gpu_launches": int(agg32["kernel_launches"]), "clocks": clk}
    if not args.skip_fp64:
        sec64, agg64 = solve(opts[64], t_values[-1])
        x64, _ = g.get_state()
        out["fp64"] = {"value": n_dofs * PLATE_STEPS / sec64, "unit": "DOF load steps/s",
                       "ms_per_step": 1e3 * sec64 / PLATE_STEPS, "newton_iterations": agg64["newton_iterations"],
                       "krylov_iterations": agg64["krylov_iterations"], "cutbacks": agg64["cutbacks"],
                       "speedup_mixed_vs_fp64": sec64 / sec32_rank,
                       "max_rel_displacement_difference_mixed_vs_fp64": float(
                           np.abs(x32 - x64).max() / max(np.abs(x64).max(), 1e-300))}
    if rank == 0 and world == 1 and not args.skip_cpu:
        try:
            from oracle.core import lib

            threads = lib().oracle_max_threads()
            sec, work, count, its = plates_cpu_sample(ns, depths, threads)
            out["cpu_baseline"] = {"value": work / sec, "unit": "DOF load steps/s", "cores": threads, "kind": "port",
                                   "sample": "%d plate(s) of the same batch nearest its median size, each solved "
                                             "alone through the 10 load steps by the oracle (OpenMP assembly, "
                                             "SuperLU, Newton to 1e-10 absolute): %.1f s, %d Newton iterations"
                                             % (count, sec, its)}
        except Exception as exc:  # the CPU leg must not hide the GPU result
            out["cpu_baseline"] = {"value": None, "error": str(exc)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as tdist

        tdist.destroy_process_group()


HEX20_METRIC = "Hex20 local damage: Newton-step time & assembled DOFs/s, FP32 tangent vs FP64 GPU"
HEX20_STEPS = 5


def run_hex20(args):
    """The large configuration: Hex20 displacements (3x3x3 Gauss) with the local exponential damage law on an n^3
    cube (80^3: 6.3 M DOFs, 1.09 G nonzeros), its 5 load steps to u_z = 5e-5 from rest on the mixed path (FP32
    tangent and Krylov, FP64 residual and history) and on the FP64 path, each timed with CUDA events; the two final
    states compared. Not the headline."""
    import torch

    import nuto_gb300
    from nuto_gb300 import configs

    torch.cuda.set_device(0)
    nuto_gb300.load()
    n = args.size or 80
    s = configs.hex20_local_damage(n, load_steps=HEX20_STEPS)
    g = s.build_gpu(device=0)
    t_values = accumulate(0.0, 1.0 / HEX20_STEPS, HEX20_STEPS)
    # local softening localises into one layer of cells in the step where damage starts; Newton needs more
    # iterations there the finer the mesh (the oracle's exact Newton: 6 at 4^3, 12 at 8^3)
    common = dict(newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL, max_newton=args.max_newton or 50, max_krylov=50000,
                  forcing_floor=FORCING_FLOOR)
    runs = {"mixed": g.default_options(precision=nuto_gb300.FP32, exact_tangent_below=EXACT_BELOW, **common),
            "fp64": g.default_options(precision=nuto_gb300.FP64, **common)}
    out, states = {}, {}
    for name, o in runs.items():
        if name == "fp64" and args.skip_fp64:
            continue
        g.set_state(None, 0.0, True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        agg = run_steps(g, o, 0.0, t_values, dt=1.0 / HEX20_STEPS, progress=name, cutbacks=3)
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        states[name], _ = g.get_state()
        na = max(agg["matrix_assemblies"], 1)
        out[name] = {"seconds": sec, "newton_step_ms": 1e3 * sec / na, "tangent_solves": agg["matrix_assemblies"],
                     "newton_per_load_step": agg["newton_per_load_step"], "krylov_iterations": agg["krylov_iterations"],
                     "cutbacks": agg["cutbacks"],
                     "ms_per_newton_step": {"tangent": agg["ms_assemble_matrix"] / na,
                                            "residual": agg["ms_assemble_vector"] / na,
                                            "krylov": agg["ms_krylov"] / na}}
    res = {"metric": HEX20_METRIC, "value": g.n_dofs * out["mixed"]["tangent_solves"] / out["mixed"]["seconds"],
           "unit": "DOF/s", "n_gpus": 1, "steps": HEX20_STEPS, "warmup": 0,
           "ms_per_step": 1e3 * out["mixed"]["seconds"] / HEX20_STEPS, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": "hex20_local_damage_%d^3: Hex20 3x3x3 Gauss on the unit cube, MomentumBalance + "
                                  "LocalIsotropicDamage(30000, 0.2, kappa0 1e-4, beta 100, alpha 0.99, k 10), z = 0 "
                                  "fixed, z = 1 u_z = 5e-5 t, %d load steps from rest" % (n, HEX20_STEPS),
                      "n_dofs": int(g.n_dofs), "nnz": int(g.nnz)},
           "runs": out}
    if "fp64" in states:
        a, b = states["mixed"], states["fp64"]
        res["mixed_vs_fp64_path"] = {"max": float(np.abs(a - b).max() / np.abs(b).max()),
                                     "l2": float(np.linalg.norm(a - b) / np.linalg.norm(b))}
        res["speedup_newton_step_mixed_vs_fp64"] = out["fp64"]["newton_step_ms"] / out["mixed"]["newton_step_ms"]
    # the FP32 tangent (tensor cores: k_tc20_points + k_tangent_tc20 + k_tc20_rows) at the final state of the last
    # run (damaged points at the fixed face's edges), timed with CUDA events, and its error against the FP64
    # tangent (element kernel, FP64 law and products) at the same state
    x_end = torch.as_tensor(g.get_state()[0], device="cuda")
    k64 = g.build_matrix(x_end, nuto_gb300.FP64)
    k32 = torch.empty(g.nnz, dtype=torch.float32, device="cuda")
    for _ in range(2):
        g.build_matrix(x_end, nuto_gb300.FP32, out=k32)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record()
    for _ in range(reps):
        g.build_matrix(x_end, nuto_gb300.FP32, out=k32)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    err = float((k32.double() - k64).abs().max() / k64.abs().max())
    tb = tangent_bytes(s, g.nnz, 4)
    peak, peak_kind = load_peaks()
    res["tangent_fp32"] = {"kernels": "k_tc20_points + k_tangent_tc20 (tcgen05.mma kind::tf32, three-product split, "
                                      "accumulators in tensor memory) + k_tc20_rows",
                           "ms_per_assembly": ms, "assembled_dofs_per_s": g.n_dofs / (ms / 1e3),
                           "algorithmic_bytes": tb, "hbm_frac": tb / (ms / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                           "max_rel_error_vs_fp64_tangent": err,
                           "tc_tflops": 2.0 * 128 * 64 * 64 * 3 * s.mesh.num_cells / (ms / 1e3) / 1e12}
    print(json.dumps(res))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "plates":
        run_plates(args)
    elif args.workload == "hex20":
        run_hex20(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
