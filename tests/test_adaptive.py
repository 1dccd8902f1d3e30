"""AdaptiveSolve (AdaptiveSolve.cpp:18-67) over scripted step outcomes: cut-back, growth, clipping to the end time
and the minimal-step error, on the host (no GPU)."""

import pytest

from nuto_gb300._lib import NoConvergence
from nuto_gb300.adaptive import AdaptiveSolve


class FakeGroup:
    """do_step(t_new) converges with the scripted iteration count, or raises NoConvergence when the step is larger
    than max_dt; records the attempted times."""

    def __init__(self, max_dt=1.0, iterations=5):
        self.t = 0.0
        self.max_dt = max_dt
        self.iterations = iterations
        self.attempts = []

    def do_step(self, t_new, options):
        self.attempts.append(t_new)
        if t_new - self.t > self.max_dt + 1e-15:
            raise NoConvergence(4, "No convergence")
        self.t = t_new
        return self.iterations

    def stats(self):
        return {"newton_iterations": self.iterations}


def test_fixed_steps_reach_the_end_exactly():
    g = FakeGroup()
    ad = AdaptiveSolve(g, None, dt=0.25, dt_max=0.25)
    assert ad.solve(1.0) == 4
    assert g.attempts == [0.25, 0.5, 0.75, 1.0]
    assert ad.cutbacks == 0


def test_cutback_halves_and_keeps_the_time():
    # steps above 0.1 fail: 0.4 -> 0.2 -> 0.1, then steps of 0.1 (slow convergence: no growth)
    g = FakeGroup(max_dt=0.1, iterations=5)
    ad = AdaptiveSolve(g, None, dt=0.4, dt_max=0.4)
    assert ad.solve(0.3) == 3
    assert ad.cutbacks == 2
    assert g.attempts[:3] == [0.4, 0.2, 0.1]
    assert g.t == pytest.approx(0.3)
    assert ad.dt == pytest.approx(0.1)  # the reduced step is kept


def test_growth_after_fast_convergence_is_capped():
    # two Newton iterations per step: dt grows by 1.5 up to dt_max; the last step is clipped to t_end
    g = FakeGroup(iterations=2)
    ad = AdaptiveSolve(g, None, dt=0.1, dt_max=0.2)
    ad.solve(0.6)
    steps = [b - a for a, b in zip([0.0] + g.attempts[:-1], g.attempts)]
    assert steps[0] == pytest.approx(0.1)
    assert steps[1] == pytest.approx(0.15)
    assert all(s <= 0.2 + 1e-15 for s in steps)
    assert g.attempts[-1] == pytest.approx(0.6)


def test_minimal_step_raises():
    g = FakeGroup(max_dt=1e-9)
    ad = AdaptiveSolve(g, None, dt=0.1, dt_max=0.1, dt_min=1e-4)
    with pytest.raises(RuntimeError):
        ad.solve(1.0)
