"""The adjoint workload's inputs (nuto_gb300.configs.hex8_adjoint): the seeded lognormal modulus field, the truth
field and the observed surface nodes."""

import numpy as np


def test_adjoint_case_field_and_observations():
    """The adjoint workload's inputs: a lognormal modulus field with the prescribed mean, CoV and Gaussian
    correlation, a different truth field, and 256 distinct observed surface nodes off the fixed face."""
    from nuto_gb300 import configs

    c = configs.hex8_adjoint(32, seed=0)
    assert c.setup.n_dofs == 143748 and c.scale.size == 32 ** 3
    assert not np.allclose(c.scale, c.true_scale)
    xyz = c.setup.mesh.layers[0].node_coords[c.obs_nodes]
    assert len(set(c.obs_nodes.tolist())) == 256
    assert np.all(np.any((np.abs(xyz) < 1e-10) | (np.abs(xyz - 1) < 1e-10), axis=1))
    assert np.all(xyz[:, 2] > 1e-10)
    assert np.array_equal(c.obs_dofs, c.setup.mesh.layers[0].dof_numbers[c.obs_nodes].reshape(-1))
    # statistics over seeds: the standard field has unit variance and correlation exp(-r^2 / (2 l^2)) along x
    n, lags = 16, (1, 2, 3)
    acc, var, m, cv = np.zeros(len(lags)), 0.0, [], []
    for sd in range(24):
        g = configs.gaussian_cell_field(n, np.random.default_rng(sd))
        var += (g * g).mean() / 24
        for i, k in enumerate(lags):
            acc[i] += (g[:, :, k:] * g[:, :, :-k]).mean() / 24
        E = configs.lognormal_cell_field(n, np.random.default_rng(sd))
        m.append(E.mean())
        cv.append(E.std() / E.mean())
    assert abs(var - 1) < 0.1
    for i, k in enumerate(lags):
        assert abs(acc[i] - np.exp(-((k / n) ** 2) / (2 * 0.1 ** 2))) < 0.08, (k, acc[i])
    assert abs(np.mean(m) / 30000 - 1) < 0.03 and abs(np.mean(cv) - 0.3) < 0.03
