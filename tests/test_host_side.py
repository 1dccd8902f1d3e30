"""CPU tests of the product's host side: the C ABI library loads and exports every declared symbol, and the
product's mesh / DOF numbering / constraint selection equals the oracle's restatement of NuTo bit for bit."""

import os
import re

import numpy as np
import pytest

import oracle
from oracle import setups as osetups

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "nuto_gpu.h")).read()
    return sorted(set(re.findall(r"\b(nuto_gpu_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_loads_and_exports_every_declared_symbol():
    import ctypes

    from nuto_gb300 import _lib

    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    raw = ctypes.CDLL(_lib.LIB_PATH)
    assert raw.nuto_gpu_version() == 1


def _cmp_layers(pm, om, layers, ncomps):
    for pl, ol, nc in zip(layers, layers, ncomps):
        PL = pm.layers[pl]
        assert PL.num_nodes == om.layer_num_nodes(ol)
        assert np.array_equal(PL.conn, om.layer_conn(ol))
        assert np.array_equal(PL.dof_numbers, om.layer_dof_numbers(ol, nc))
        assert np.allclose(PL.node_coords, om.layer_node_coords(ol), atol=1e-15)


@pytest.mark.parametrize("n", [1, 3, 8])
def test_quad4_numbering_and_constraints_match_oracle(n):
    from nuto_gb300 import configs

    s = configs.quad4_elastic(n)
    om, layers, P, cons = osetups.quad4_elastic(n)
    assert np.allclose(s.mesh.coords, om.coords(2))
    assert np.array_equal(s.mesh.conn, om.conn(4))
    _cmp_layers(s.mesh, om, layers, [2])
    assert np.array_equal(s.constraints[0][0], cons[0])
    assert np.array_equal(s.constraints[0][1], cons[1])


@pytest.mark.parametrize("n", [1, 2, 5])
def test_hex8_gradient_damage_numbering_and_constraints_match_oracle(n):
    from nuto_gb300 import configs

    s = configs.hex8_gradient_damage(n)
    om, layers, P, cons = osetups.hex8_gradient_damage(n)
    assert np.allclose(s.mesh.coords, om.coords(3))
    _cmp_layers(s.mesh, om, layers, [3, 1])
    assert np.array_equal(s.constraints[0][0], cons[0])
    assert np.array_equal(s.constraints[0][2], cons[2])
    assert s.n_dofs == P.n_dofs


@pytest.mark.parametrize("n", [1, 2, 3])
def test_hex20_numbering_matches_oracle(n):
    from nuto_gb300 import configs

    s = configs.hex20_local_damage(n)
    om, layers, P, cons = osetups.hex20_local_damage(n)
    _cmp_layers(s.mesh, om, layers, [3])
    assert np.array_equal(s.constraints[0][0], cons[0])
    # node count of the 20-node serendipity lattice
    assert s.mesh.layers[0].num_nodes == (n + 1) ** 3 + 3 * n * (n + 1) ** 2


def test_benchmark_sizes():
    """DOF counts of the benchmark meshes (survey table: 80,802 / 1,098,500 / 6,318,243)."""
    from nuto_gb300 import mesh as M

    m = M.create_quads(200, 200)
    assert M.add_dof_interpolation(m, 2) == 0 and m.layers[0].num_dofs == 80802
    assert 3 * 65 ** 3 + 65 ** 3 == 1098500
    n = 80
    assert 3 * ((n + 1) ** 3 + 3 * n * (n + 1) ** 2) == 6318243
