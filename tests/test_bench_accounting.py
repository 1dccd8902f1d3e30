"""The benchmark's byte accounting and time stepping on the CPU: the algorithmic bytes of one FP32 tangent assembly of
the 64^3 beam (values written once, connectivity, coordinates, state and history read once) and the load-step end
times summed as the adaptive stepping sums them."""

import bench


def test_tangent_bytes_of_the_beam():
    from nuto_gb300 import configs

    s = configs.hex8_gradient_damage(64)
    nnz = 16 * 193 ** 3  # node pairs (3n+1)^3 x 16 entries per pair of [u | eeq] nodes
    cells, nodes = 64 ** 3, 65 ** 3
    expect = (nnz * 4                      # FP32 values written once
              + 3 * cells * 8 * 4          # int32 connectivity: displacement, eeq and coordinate cells
              + nodes * 3 * 8              # FP64 coordinates
              + 4 * nodes * 8              # FP64 state (u and eeq)
              + cells * 8 * 8)             # FP64 history per integration point
    assert bench.tangent_bytes(s, nnz, 4) == expect == 517421688


def test_accumulated_end_times():
    t = bench.accumulate(0.0, 0.05, 20)
    acc = 0.0
    for k in range(20):
        acc += 0.05
        assert t[k] == acc
    assert len(bench.accumulate(0.3, 0.1, 0)) == 0


def test_both_arms_assemble_the_same_state():
    """The headline's seeded state built from the product's set-up and from the oracle's set-up (the reference arm)
    is the same vector and history, bit for bit."""
    import numpy as np

    from nuto_gb300 import configs

    n = 4
    s = configs.hex8_gradient_damage(n)
    Ld, Le = s.mesh.layers[s.layers[0]], s.mesh.layers[s.layers[1]]
    x, kappa = bench.beam_state(Ld.node_coords, Ld.dof_numbers, Le.dof_numbers, s.n_dofs, s.mesh.num_cells, 8, n)
    P, xo = bench.oracle_beam(n)
    assert np.array_equal(x, xo)
    assert np.array_equal(kappa, P.kappa)
    # a mix of branches: loading and unloading points, damaged and undamaged ones
    assert 0.2 < np.mean(kappa > 1e-4) < 0.9
