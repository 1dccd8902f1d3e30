"""nuto_gpu_build_matrix_noalloc: the FP32 tangent with its integration-point records in the library's static device
array (the call allocates nothing), checked against nuto_gpu_build_matrix on the same state."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _group(n):
    pytest.importorskip("torch")
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from nuto_gb300 import configs

    s = configs.hex8_gradient_damage(n)
    return s, s.build_gpu()


def _state(s, g, seed):
    rng = np.random.default_rng(seed)
    n_u = 3 * s.mesh.layers[s.layers[0]].num_nodes
    u = rng.uniform(-2e-4, 2e-4, g.n_dofs)
    u[n_u:] = rng.uniform(0.0, 4e-4, g.n_dofs - n_u)
    kappa = rng.uniform(0.0, 3e-4, (s.mesh.num_cells, g.n_ip))
    return u, kappa


def _unchanged_memory(fn):
    """Runs fn() and checks that the device memory in use did not change: torch's allocator holds the same
    bytes and cudaMemGetInfo reports the same free memory (nothing was allocated on the device)."""
    import gc

    import torch

    # contexts of earlier tests that the garbage collector has not reached yet would free their device memory at an
    # arbitrary point: collect them first and keep the collector off while measuring
    gc.collect()
    gc.disable()
    try:
        torch.cuda.synchronize()
        held = torch.cuda.memory_allocated()
        free0, _ = torch.cuda.mem_get_info()
        fn()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
    finally:
        gc.enable()
    assert torch.cuda.memory_allocated() == held
    assert free1 == free0


def test_noalloc_tangent_matches_build_matrix_twice():
    import torch

    import nuto_gb300

    s, g = _group(4)
    u, kappa = _state(s, g, 7)
    g.history = kappa
    ref = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    scale = np.abs(ref).max()
    ud = torch.as_tensor(u, device="cuda")
    out = torch.empty(g.nnz, dtype=torch.float32, device="cuda")
    for _ in range(2):  # two calls in a row reuse the static records
        _unchanged_memory(lambda: g.build_matrix_noalloc(ud, out=out))
        v = out.double().cpu().numpy()
        assert np.abs(v - ref).max() <= 1e-6 * scale
    # a second state after the first: nothing of the previous call leaks into the next one
    u2, kappa2 = _state(s, g, 8)
    g.history = kappa2
    ref2 = g.build_matrix(u2, nuto_gb300.FP32).double().cpu().numpy()
    v2 = g.build_matrix_noalloc(u2).double().cpu().numpy()
    assert np.abs(v2 - ref2).max() <= 1e-6 * np.abs(ref2).max()


def test_noalloc_tangent_hex20_local_damage():
    """The other record layout: Hex20 displacements with the local damage law (3x3x3 points, 2,099 cells at most),
    two calls in a row against nuto_gpu_build_matrix."""
    import torch

    import nuto_gb300
    from nuto_gb300 import configs

    s = configs.hex20_local_damage(3)
    g = s.build_gpu()
    rng = np.random.default_rng(12)
    u = rng.uniform(-3e-4, 3e-4, g.n_dofs)
    g.history = rng.uniform(0.0, 3e-4, (s.mesh.num_cells, g.n_ip))
    ref = g.build_matrix(u, nuto_gb300.FP32).double().cpu().numpy()
    ud = torch.as_tensor(u, device="cuda")
    out = torch.empty(g.nnz, dtype=torch.float32, device="cuda")
    for _ in range(2):
        _unchanged_memory(lambda: g.build_matrix_noalloc(ud, out=out))
        assert np.abs(out.double().cpu().numpy() - ref).max() <= 1e-6 * np.abs(ref).max()


def test_noalloc_tangent_needs_setup_and_rejects_large_meshes():
    import nuto_gb300

    s, g = _group(3)
    u, kappa = _state(s, g, 9)
    with pytest.raises(nuto_gb300.NutoGpuError) as e:
        g.build_matrix_noalloc(u)  # the allocating set-up has not run yet
    assert e.value.code == nuto_gb300._lib.ESTATE
    s, g = _group(24)  # 13,824 Hex8 gradient-damage cells: above the 12,192 the static array holds
    u, kappa = _state(s, g, 10)
    g.build_matrix(u, nuto_gb300.FP32)
    with pytest.raises(nuto_gb300.NutoGpuError) as e:
        g.build_matrix_noalloc(u)
    assert e.value.code == nuto_gb300._lib.EINVAL
