"""Kernel timeline of one load step of the gradient-damage benchmark, recorded with the CUDA activity trace of the
PyTorch profiler (device start/end of every kernel, memset and copy, including the kernels of CUDA graphs).

    python -m nuto_gb300.trace_step [--size 64] [--warmup 3]

Runs --warmup load steps of the benchmark schedule (FP32 tangent, exact final phase), then traces load step
warmup + 1 and prints: wall time, GPU busy time and the gaps between operations; the device time per kernel; and
per Krylov iteration (delimited by the GMRES projection kernel) the time by class. Unlike a serialised ncu launch
list the times are the ones of the real run (warm caches, back-to-back launches). Two limits: with programmatic
dependent launch a kernel's interval includes its wait for the predecessor (intervals overlap), and the activity
buffers can drop records on steps with tens of thousands of launches (compare the operation count with the
step's kernel_launches statistic); both are reported.
"""

import argparse
import collections
import json
import os
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _name(e):
    return e["name"].split("(")[0].replace("void nuto_gpu::", "").replace("nuto_gpu::", "")


def _grid(e):
    g = e.get("args", {}).get("grid", [0])
    return g[0] if isinstance(g, list) else 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--size", type=int, default=64)
    p.add_argument("--warmup", type=int, default=3)
    a = p.parse_args()
    import numpy as np
    import torch
    from torch.profiler import ProfilerActivity, profile

    import nuto_gb300
    from nuto_gb300 import configs

    load_steps = 20
    s = configs.hex8_gradient_damage(a.size, load_steps=load_steps, imperfection=True)
    g = s.build_gpu()
    g.set_state(None, 0.0, True)
    g.history = s.history0
    o = g.default_options(precision=nuto_gb300.FP32, newton_rtol=1e-8, krylov_rtol=1e-3, max_newton=20,
                          max_krylov=20000)
    dt = 1.0 / load_steps
    for k in range(1, a.warmup + 1):
        g.do_step(dt * k, o)
    x, t = g.get_state()
    kappa = g.history
    g.do_step(t + dt, o)  # the same step once untraced (graphs captured, buffers allocated)
    torch.cuda.synchronize()
    g.set_state(x, t, False)
    g.history = kappa
    with profile(activities=[ProfilerActivity.CUDA, ProfilerActivity.CPU]) as prof:
        t0 = time.perf_counter()
        g.do_step(t + dt, o)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    st = g.stats()
    fd, path = tempfile.mkstemp(suffix=".json")
    os.close(fd)
    prof.export_chrome_trace(path)
    ev = json.load(open(path))["traceEvents"]
    os.unlink(path)
    ks = sorted([e for e in ev if e.get("cat") in ("kernel", "gpu_memcpy", "gpu_memset") and "dur" in e],
                key=lambda e: e["ts"])
    busy = sum(e["dur"] for e in ks)
    span = ks[-1]["ts"] + ks[-1]["dur"] - ks[0]["ts"]
    gaps = [ks[i + 1]["ts"] - ks[i]["ts"] - ks[i]["dur"] for i in range(len(ks) - 1)]
    print("size %d, load step %d: %d Newton iterations, %d Krylov iterations, %d tangent assemblies, "
          "%d kernel launches (%d device operations recorded)"
          % (a.size, a.warmup + 1, st["newton_iterations"], st["krylov_iterations"], st["matrix_assemblies"],
             st["kernel_launches"], len(ks)))
    print("wall %.1f ms, GPU span %.1f ms, GPU busy %.1f ms, %d operations, gaps %.1f ms (median %.2f us)" %
          (1e3 * (t1 - t0), span / 1e3, busy / 1e3, len(ks), sum(x for x in gaps if x > 0) / 1e3,
           float(np.median([x for x in gaps if x > 0]))))
    per = collections.defaultdict(lambda: [0, 0.0])
    for e in ks:
        per[_name(e)][0] += 1
        per[_name(e)][1] += e["dur"]
    print("\n| kernel | launches | total ms | mean us | share |\n|---|---|---|---|---|")
    for k, (n, d) in sorted(per.items(), key=lambda x: -x[1][1])[:24]:
        print("| `%s` | %d | %.2f | %.2f | %.1f%% |" % (k, n, d / 1e3, d / n, 100 * d / busy))
    idx = [i for i, e in enumerate(ks) if _name(e).startswith("k_gm_proj")]
    if len(idx) > 2:
        cls = collections.defaultdict(float)
        for i0, i1 in zip(idx[:-1], idx[1:]):
            for e in ks[i0:i1]:
                n, gsz = _name(e), _grid(e)
                kind = "spmv" if "spmv" in n else ("gmres" if n.startswith("k_gm") else "other")
                size = "fine" if gsz >= 8000 else ("level 1-2" if gsz >= 1000 else "small")
                cls["%s (%s)" % (kind, size)] += e["dur"]
            cls["gaps"] += sum(max(0, ks[j + 1]["ts"] - ks[j]["ts"] - ks[j]["dur"]) for j in range(i0, i1 - 1))
        ni = len(idx) - 1
        span_it = (ks[idx[-1]]["ts"] - ks[idx[0]]["ts"]) / ni
        print("\nper Krylov iteration (%d iterations, %.1f us each; classes by grid size):" % (ni, span_it))
        print("| class | us per iteration |\n|---|---|")
        for k, v in sorted(cls.items(), key=lambda x: -x[1]):
            print("| %s | %.1f |" % (k, v / ni))


if __name__ == "__main__":
    main()
