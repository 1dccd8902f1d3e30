"""CPU tests of the batched-specimen set-up (nuto_gb300.batch): the concatenated mesh's DOF numbering equals the
oracle's first-touch numbering of the same cells bit for bit, the state splits back into the specimens, and the
oracle's Newton on the whole batch (block-diagonal system, one absolute tolerance) reproduces the oracle's
separate solves of every specimen."""

import numpy as np
import pytest

import oracle
from oracle import setups as osetups
from oracle.quasistatic import QuasistaticOracle


def _batch(specs):
    from nuto_gb300 import batch, configs

    return batch.concatenate([configs.notched_plate(n, d) for n, d in specs])


def _oracle_of_batch(b):
    """The oracle's restatement run on the product's concatenated arrays."""
    m = oracle.Mesh.from_arrays(2, oracle.QUAD4, b.mesh.coords, b.mesh.conn)
    d = m.add_dof(2)
    e = m.add_dof(1)
    integ = oracle.Integrand.make(oracle.GRADIENT_DAMAGE, 2, E=30000.0, nu=0.2, damage_application=oracle.FULL,
                                  kappa0=1e-4, beta=100.0, alpha=0.99, k=10.0, c=0.01)
    return m, [d, e], oracle.Problem(m, 2, [d, e], integ)


def test_notched_plate_matches_oracle_setup():
    from nuto_gb300 import configs

    for n, depth in ((4, 0.2), (8, 0.4), (12, 0.5), (9, 0.33)):
        s = configs.notched_plate(n, depth)
        om, layers, P, cons = osetups.notched_plate(n, depth)
        assert s.n_dofs == P.n_dofs
        for k in range(2):
            assert np.array_equal(s.mesh.layers[s.layers[k]].conn, om.layer_conn(layers[k]))
        assert np.array_equal(s.constraints[0][0], cons[0])
        assert np.array_equal(s.constraints[0][2], cons[2])
        assert s.mesh.num_cells == n * n - min(max(round(depth * n), 1), n - 2)


def test_batch_numbering_is_shifted_specimen_numbering():
    specs = [(6, 0.25), (4, 0.5), (9, 0.3)]
    b = _batch(specs)
    om, layers, P = _oracle_of_batch(b)
    for k in range(2):
        assert np.array_equal(b.mesh.layers[b.layers[k]].conn, om.layer_conn(layers[k]))
    assert b.n_dofs == P.n_dofs
    from nuto_gb300 import configs

    plates = [configs.notched_plate(n, d) for n, d in specs]
    assert [r.cells for r in b.specimens] == [(0, 34), (34, 48), (48, 126)]  # 36 - 2, 16 - 2, 81 - 3 cells
    assert b.layer_dofs == [sum(p.mesh.layers[0].num_dofs for p in plates),
                            sum(p.mesh.layers[1].num_dofs for p in plates)]
    assert len(b.constraints[0][0]) == sum(len(p.constraints[0][0]) for p in plates)
    # split_state inverts the combined [u of all | eeq of all] order
    xs = [np.random.default_rng(i).uniform(size=p.n_dofs) for i, p in enumerate(plates)]
    nu = [p.mesh.layers[0].num_dofs for p in plates]
    x = np.concatenate([xi[:n] for xi, n in zip(xs, nu)] + [xi[n:] for xi, n in zip(xs, nu)])
    for a, c in zip(b.split_state(x), xs):
        assert np.array_equal(a, c)


def test_batch_rejects_mixed_specimens():
    from nuto_gb300 import batch, configs

    with pytest.raises(ValueError):
        batch.concatenate([configs.notched_plate(6), configs.quad4_elastic(6)])
    with pytest.raises(ValueError):
        batch.concatenate([])


def test_seeded_plate_batch_is_reproducible():
    from nuto_gb300 import batch

    b1, n1, d1 = batch.notched_plate_batch(6, seed=4, n_range=(4, 10))
    b2, n2, d2 = batch.notched_plate_batch(6, seed=4, n_range=(4, 10))
    assert np.array_equal(n1, n2) and np.array_equal(d1, d2)
    assert np.array_equal(b1.mesh.conn, b2.mesh.conn)
    assert n1.min() >= 4 and n1.max() <= 10 and d1.min() >= 0.2 and d1.max() <= 0.5


def test_batched_newton_reproduces_separate_solves():
    """Six load steps (damage from step 4) of three plates solved as one batch by the oracle's Newton (direct solve,
    absolute tolerance on the combined |C^T r|) against each plate solved alone: the same states to 1e-9."""
    specs = [(6, 0.25), (4, 0.5), (8, 0.4)]
    b = _batch(specs)
    om, layers, P = _oracle_of_batch(b)
    dep, a, s = b.constraints[0]
    Qb = QuasistaticOracle(P, dep, a, s, tolerance=1e-12, max_iterations=20)
    alone = []
    for n, d in specs:
        _, _, Pi, ci = osetups.notched_plate(n, d)
        alone.append((Pi, QuasistaticOracle(Pi, ci[0], ci[1], ci[2], tolerance=1e-12, max_iterations=20)))
    for k in range(1, 7):
        Qb.do_step(0.1 * k)
        for Pi, Qi in alone:
            Qi.do_step(0.1 * k)
    xs = b.split_state(Qb.x)
    ks = b.split_history(P.kappa)
    for (Pi, Qi), x, kap in zip(alone, xs, ks):
        assert np.abs(x - Qi.x).max() <= 1e-9 * np.abs(Qi.x).max()
        assert np.abs(kap - Pi.kappa).max() <= 1e-9 * np.abs(Pi.kappa).max()
        assert Pi.kappa.max() > 1e-4  # damaged


def test_plates_cpu_sample_counts_work():
    """The CPU baseline of the batched workload (bench.py): plates nearest the median size first, at least one."""
    import bench

    ns, depths = np.array([4, 6, 5]), np.array([0.3, 0.4, 0.25])
    sec, work, count, its = bench.plates_cpu_sample(ns, depths, 1, budget_s=0.0)
    _, _, P, _ = osetups.notched_plate(5, 0.25)
    assert count == 1 and work == P.n_dofs * bench.PLATE_STEPS and sec > 0 and its > 0

