"""Benchmark: quasistatic load steps of the 3D implicit gradient-damage beam (Hex8, 64^3 cells, 1.1 M DOFs) on GB300.

A step is one load step of the 20-step schedule to u_z = 2e-3 m (QuasistaticSolver::DoStep: trial state, Newton
with line search to |C^T r| <= 1e-8 |C^T (r + K db)|, history update), run through the C ABI with the state and
history resident in HBM. W warm-up load steps from rest come first, then exactly K timed load steps.

value      DOFs x tangent solves / s of the mixed-precision path (FP32 tangent + FP32 GMRES, FP64 residual): the
           assembled-and-solved DOFs per second; ms_per_step is the time of one load step and newton_step_ms the
           time of one tangent assembly + Krylov solve + residual update.
fp64       the same K load steps on the plain FP64 GPU path, from the same warm state, and the speed-up.
e2e        the same metric through nuto_gpu_do_step_host with the state vector and history in pinned host memory
           (copied in and out every step).
roofline   the Krylov SpMV (dominant kernel): algorithmic bytes per launch / mean CUDA-event duration.
cpu_baseline / --impl reference
           the oracle (CPU restatement of NuTo's assembly, OpenMP) plus scipy SuperLU as the stand-in for
           Eigen::SparseLU, timed on a bounded sample of the same problem on the host cores.

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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=64)
    p.add_argument("--skip-fp64", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--workload", default="beam", choices=["beam", "plates"])
    p.add_argument("--specimens", type=int, default=128)
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


def run_steps(g, opts, t_start, t_values):
    """Advances the load from t_start through every t in t_values with AdaptiveSolve (time step 1/LOAD_STEPS, cut
    back by halves on NoConvergence as the reference's AdaptiveSolve does). Returns the summed step statistics,
    failed attempts included (their work was done), and the number of cut-backs."""
    from nuto_gb300.adaptive import AdaptiveSolve

    dt = 1.0 / LOAD_STEPS
    ad = AdaptiveSolve(g, opts, dt=dt, dt_max=dt, dt_min=dt / 256)
    t = t_start
    for tv in t_values:
        ad.solve(tv, t)
        t = tv
    agg = {k: 0 for k in AGG_KEYS}
    for st in ad.stats:
        for k in agg:
            agg[k] += st[k]
    agg["cutbacks"] = ad.cutbacks
    agg["do_steps"] = len(ad.stats)
    return agg


def cpu_sample(n_s, threads):
    """One Newton iteration of the oracle (BuildMatrix + BuildVector + SuperLU solve of C^T K C) on an n_s^3 beam of
    the same problem, after two elastic load steps. Returns (seconds, n_dofs)."""
    import scipy.sparse.linalg as spla

    from oracle import setups
    from oracle.core import lib
    from oracle.quasistatic import QuasistaticOracle

    lib().oracle_set_threads(threads)
    om, layers, P, cons = setups.hex8_gradient_damage(n_s)
    Q = QuasistaticOracle(P, cons[0], cons[1], cons[2], tolerance=1e-10, max_iterations=20)
    x = np.zeros(P.n_dofs)
    t0 = time.perf_counter()
    K = Q.derivative(x)
    r = Q.residual(x)
    t1 = time.perf_counter()
    db = Q.global_rhs(1.0 / LOAD_STEPS) - Q.global_rhs(0.0)
    rhs = r + K @ db
    Kr = K[Q.indep][:, Q.indep].tocsc()
    spla.spsolve(Kr, rhs[Q.indep])
    t2 = time.perf_counter()
    cpu_sample.last = (t1 - t0, t2 - t1)
    return t2 - t0, P.n_dofs


def cpu_baseline(steps=1, n_s=16):
    from oracle.core import lib

    threads = lib().oracle_max_threads()
    times = []
    for _ in range(steps):
        dt, n = cpu_sample(n_s, threads)
        times.append(dt)
    t = float(np.median(times))
    return {"value": n / t, "unit": "DOF/s", "cores": threads, "kind": "port",
            "sample": "one Newton iteration (oracle BuildMatrix + BuildVector with OpenMP, SuperLU solve of C^T K C) "
                      "of the same gradient-damage beam at %d^3 cells (%d DOFs); %.2f s, of which assembly %.2f s "
                      "and SuperLU %.2f s" % (n_s, n, t, cpu_sample.last[0], cpu_sample.last[1]),
            "assembly_dofs_per_s": n / cpu_sample.last[0],
            "ms_per_newton_step": 1e3 * t}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle

    oracle.build()
    if args.workload == "plates":
        run_reference_plates(args)
        return
    for _ in range(args.warmup):
        cpu_sample(16, oracle.lib().oracle_max_threads())
    times = []
    n = None
    for _ in range(args.steps):
        dt, n = cpu_sample(16, oracle.lib().oracle_max_threads())
        times.append(dt)
    total = float(sum(times))
    value = n * args.steps / total
    cores = oracle.lib().oracle_max_threads()
    out = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": "hex8_gradient_damage beam 1x1x4, 16^3 cells sample of the 64^3 workload",
                      "n_dofs": n, "parallelism": "host OpenMP"},
           "cpu_baseline": {"value": value, "unit": "DOF/s", "cores": cores, "kind": "port",
                            "sample": "one Newton iteration per step (oracle assembly + SuperLU) on a 16^3 cell "
                                      "sample; the reference itself cannot be built (Eigen/Boost absent)"},
           "e2e": {"value": value, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


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
    s = configs.hex8_gradient_damage(args.size, load_steps=LOAD_STEPS, imperfection=True)
    g = s.build_gpu(device=local)
    n_dofs, nnz = g.n_dofs, g.nnz
    opts32 = g.default_options(precision=nuto_gb300.FP32, newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL, max_newton=20,
                               max_krylov=20000, exact_tangent_below=EXACT_BELOW)
    opts64 = g.default_options(precision=nuto_gb300.FP64, newton_rtol=1e-8, krylov_rtol=KRYLOV_RTOL, max_newton=20,
                               max_krylov=20000)
    dt = 1.0 / LOAD_STEPS
    g.set_state(None, 0.0, True)
    g.history = s.history0
    # load-step end times by accumulation, as AdaptiveSolve advances the time (t += dt), so that every step ends
    # exactly on its end time (k * dt can differ from the accumulated sum in the last bit)
    run_steps(g, opts32, 0.0, accumulate(0.0, dt, args.warmup))
    x_w, t_w = g.get_state()
    kappa_w = g.history
    t_values = accumulate(t_w, dt, args.steps)

    def barrier():
        if world > 1:
            import torch.distributed as tdist

            tdist.barrier()
        torch.cuda.synchronize()

    def timed(opts):
        g.set_state(x_w, t_w, False)
        g.history = kappa_w
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        agg = run_steps(g, opts, t_w, t_values)
        e1.record()
        barrier()
        return e0.elapsed_time(e1) / 1e3, agg

    clocks = ClockSampler(gpu_index(local))
    clocks.start()
    sec32, agg32 = timed(opts32)
    clk = clocks.stop()
    x32, _ = g.get_state()
    sec32_rank = sec32  # this rank's own time, for the ratios to this rank's FP64 run
    (work,), sec32 = aggregate_ranks([n_dofs * agg32["matrix_assemblies"]], sec32, "cuda")
    value = work / sec32

    fp64 = None
    if not args.skip_fp64:
        sec64, agg64 = timed(opts64)
        x64, _ = g.get_state()
        err = float(np.abs(x32 - x64).max() / max(np.abs(x64).max(), 1e-300))
        err_l2 = float(np.linalg.norm(x32 - x64) / max(np.linalg.norm(x64), 1e-300))
        fp64 = {"value": n_dofs * agg64["matrix_assemblies"] / sec64, "unit": "DOF/s",
                "ms_per_step": 1e3 * sec64 / args.steps,
                "newton_step_ms": 1e3 * sec64 / max(agg64["matrix_assemblies"], 1),
                "newton_iterations": agg64["newton_iterations"], "krylov_iterations": agg64["krylov_iterations"],
                "ms_assemble_matrix_per_launch": agg64["ms_assemble_matrix"] / max(agg64["matrix_assemblies"], 1),
                "speedup_mixed_vs_fp64_newton_step": (sec64 / max(agg64["matrix_assemblies"], 1))
                / (sec32_rank / max(agg32["matrix_assemblies"], 1)),
                "speedup_mixed_vs_fp64_load_step": sec64 / sec32_rank,
                "max_rel_displacement_error_mixed_vs_fp64": err,
                "l2_rel_displacement_error_mixed_vs_fp64": err_l2}
        # both results against an FP64 solution of the same steps converged to 1e-11 (untimed): the displacement
        # uncertainty that the 1e-8 residual tolerance itself leaves is the scale for the mixed path's error
        opts_t = g.default_options(precision=nuto_gb300.FP64, newton_rtol=1e-11, krylov_rtol=1e-6, max_newton=40,
                                   max_krylov=20000)
        try:
            g.set_state(x_w, t_w, False)
            g.history = kappa_w
            run_steps(g, opts_t, t_w, t_values)
            xt, _ = g.get_state()
            sc = max(np.abs(xt).max(), 1e-300)
            fp64["max_rel_displacement_error_vs_fp64_1e-11"] = {
                "mixed": float(np.abs(x32 - xt).max() / sc), "fp64": float(np.abs(x64 - xt).max() / sc)}
            nt = max(np.linalg.norm(xt), 1e-300)
            fp64["l2_rel_displacement_error_vs_fp64_1e-11"] = {
                "mixed": float(np.linalg.norm(x32 - xt) / nt), "fp64": float(np.linalg.norm(x64 - xt) / nt)}
        except Exception as exc:  # the reference solution is a diagnostic only
            fp64["max_rel_displacement_error_vs_fp64_1e-11"] = {"error": str(exc)}

    # end to end through the C ABI with pinned host buffers (state + history copied in and out every step)
    n_hist = s.mesh.num_cells * g.n_ip
    xa = torch.empty(n_dofs, dtype=torch.float64, pin_memory=True)
    xb = torch.empty(n_dofs, dtype=torch.float64, pin_memory=True)
    ka = torch.empty(n_hist, dtype=torch.float64, pin_memory=True)
    kb = torch.empty(n_hist, dtype=torch.float64, pin_memory=True)
    xa.numpy()[:] = x_w
    ka.numpy()[:] = kappa_w.ravel()
    g.set_state(x_w, t_w, False)
    barrier()
    h0 = time.perf_counter()
    assemblies = 0
    t, step = t_w, dt
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
    (work_e2e,), sec_e2e = aggregate_ranks([n_dofs * assemblies], sec_e2e, "cuda")
    e2e = {"value": work_e2e / sec_e2e, "unit": "DOF/s",
           "h2d_bytes_per_step": int((n_dofs + n_hist) * 8), "d2h_bytes_per_step": int((n_dofs + n_hist) * 8),
           "ms_per_step": 1e3 * sec_e2e / args.steps}

    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    per_launch = agg32["ms_spmv"] / max(agg32["spmv_launches"], 1) / 1e3
    sb = spmv_bytes(g, 4)
    achieved = sb / per_launch / 1e9
    roof = {"kernel": "k_spmv_nb<float,float,0> (Krylov SpMV of the whole FP32 tangent, padded pair layout)",
            "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "traffic": traffic.get("k_spmv_fp32_bytes_per_launch"), "algorithmic_bytes_per_launch": sb,
            "mean_launch_us": per_launch * 1e6, "launches": agg32["spmv_launches"]}
    tb = tangent_bytes(s, nnz, 4)
    # FP32 tangent assemblies timed alone (the step statistics also count the exact final phase's FP64
    # assemblies): five assemblies at the warm state, CUDA events on the library's stream (the current stream)
    u_dev = torch.as_tensor(x_w, device="cuda")
    k32 = torch.empty(nnz, dtype=torch.float32, device="cuda")
    g.build_matrix(u_dev, nuto_gb300.FP32, out=k32)
    torch.cuda.synchronize()
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record()
    for _ in range(5):
        g.build_matrix(u_dev, nuto_gb300.FP32, out=k32)
    a1.record()
    torch.cuda.synchronize()
    asm_launch = a0.elapsed_time(a1) / 5 / 1e3
    del k32
    assembly = {"kernel": "k_tangent<float,REC> + k_tangent_rows<float> (FP32 tangent: records + row gather)",
                "bound": "hbm",
                "achieved": tb / asm_launch / 1e9, "peak": peak, "unit": "GB/s",
                "frac": tb / asm_launch / 1e9 / peak, "algorithmic_bytes_per_launch": tb,
                "mean_launch_ms": asm_launch * 1e3, "assembled_dofs_per_s": n_dofs / asm_launch,
                "traffic": traffic.get("k_tangent_fp32_bytes_per_launch")}

    out = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * sec32 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": "hex8_gradient_damage_%d^3: Hex8 2x2x2 Gauss, beam 1x1x4 m, u + eeq, "
                                  "GradientDamage(c=0.01, LinearElasticDamage(30000, 0.2, FULL), "
                                  "DamageLawExponential(1e-4, 100, 0.99), ModifiedMises(k=10)), 20 load steps to "
                                  "u_z=2e-3 (AdaptiveSolve cut-back), imperfection kappa=3 kappa0 in the two middle "
                                  "cell layers; timed load steps %d..%d" % (args.size, args.warmup + 1,
                                                                           args.warmup + args.steps),
                      "n_dofs": n_dofs, "nnz": nnz,
                      "precision": "FP32 tangent + FP32 GMRES(80) and multigrid, FP64 residual, history and Newton "
                                   "test; the iterations with |C^T r| < %g tol assemble the FP64 tangent and refine "
                                   "the FP32 solves against it" % EXACT_BELOW,
                      "newton_tolerance": "|C^T r| <= 1e-8 |C^T (r + K db)| of the load step",
                      "krylov_rtol": KRYLOV_RTOL,
                      "l2": "inputs larger than L2 (FP32 tangent %.0f MB)" % (nnz * 4 / 1e6),
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "newton_step_ms": 1e3 * sec32 / max(agg32["matrix_assemblies"], 1),
           "newton_iterations": agg32["newton_iterations"], "tangent_solves": agg32["matrix_assemblies"],
           "do_steps": agg32["do_steps"], "cutbacks": agg32["cutbacks"],
           "krylov_iterations": agg32["krylov_iterations"],
           "roofline": roof, "roofline_assembly": assembly, "fp64": fp64, "e2e": e2e,
           "gpu_launches": int(agg32["kernel_launches"]), "clocks": clk}
    if fp64 is not None:
        # the two targets side by side: Newton-step speed-up over the FP64 GPU path, and the relative displacement
        # error against the converged FP64 solution (1e-11 residual; the FP64 path at 1e-8 shown for scale) and
        # against the FP64 path's own 1e-8 result
        tight = fp64.get("max_rel_displacement_error_vs_fp64_1e-11", {})
        tight_l2 = fp64.get("l2_rel_displacement_error_vs_fp64_1e-11", {})
        out["targets"] = {
            "speedup_newton_step_mixed_vs_fp64": fp64["speedup_mixed_vs_fp64_newton_step"],
            "mixed_vs_converged_fp64": {"max": tight.get("mixed"), "l2": tight_l2.get("mixed")},
            "fp64_path_vs_converged_fp64": {"max": tight.get("fp64"), "l2": tight_l2.get("fp64")},
            "mixed_vs_fp64_path": {"max": fp64["max_rel_displacement_error_mixed_vs_fp64"],
                                   "l2": fp64["l2_rel_displacement_error_mixed_vs_fp64"]}}
    if rank == 0 and world == 1 and not args.skip_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline()
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


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "plates":
        run_plates(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
