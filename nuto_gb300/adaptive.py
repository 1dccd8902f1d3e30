"""Adaptive load stepping: AdaptiveSolve::Solve (nuto/mechanics/tools/AdaptiveSolve.cpp:18-67) over
nuto_gpu_do_step (host logic only; tests/test_adaptive.py checks it against scripted step outcomes).

A step that ends in NewtonRaphson::NoConvergence (NUTO_GPU_ENOCONV; the library leaves state and history
unchanged) is retried with the time step times decrease_factor; after a step that converged in fewer than three
Newton iterations the time step grows by increase_factor up to dt_max. Defaults are the reference's
(AdaptiveSolve.h: dt = dt_max = 0.1, dt_min = 1e-6, factors 1.5 / 0.5).
"""

from ._lib import NoConvergence


class AdaptiveSolve:
    def __init__(self, group, options, dt=0.1, dt_max=0.1, dt_min=1e-6, increase_factor=1.5, decrease_factor=0.5,
                 post_process=None):
        self.g = group
        self.options = options
        self.dt = dt
        self.dt_max = dt_max
        self.dt_min = dt_min
        self.increase_factor = increase_factor
        self.decrease_factor = decrease_factor
        self.post_process = post_process
        self.steps = 0
        self.cutbacks = 0
        self.stats = []

    def solve(self, t_end, t_start=0.0):
        """Advances the group's state from t_start to t_end; returns the number of converged steps.

        Follows AdaptiveSolve::Solve step by step: the time step is state (kept across calls, clipped so that the
        last step ends at t_end), at least one step is attempted, a NoConvergence halves it without advancing the
        time, and after a step that converged in fewer than three Newton iterations it grows by increase_factor up
        to dt_max."""
        t = t_start
        steps = 0
        if self.post_process:
            self.post_process(t)
        while True:
            try:
                its = self.g.do_step(t + self.dt, self.options)
            except NoConvergence:
                self.dt *= self.decrease_factor
                self.cutbacks += 1
                self.stats.append(self.g.stats())
                if self.dt < self.dt_min:
                    raise RuntimeError("time step smaller than the prescribed minimal time step %g" % self.dt_min)
                continue  # without updating the global time
            t += self.dt
            steps += 1
            self.stats.append(self.g.stats())
            if self.post_process:
                self.post_process(t)
            if t >= t_end:
                break
            if its < 3 and self.dt < self.dt_max:
                self.dt = min(self.dt * self.increase_factor, self.dt_max)
            if t + self.dt > t_end:
                self.dt = t_end - t
        self.steps += steps
        return steps
