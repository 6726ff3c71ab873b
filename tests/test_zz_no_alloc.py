"""mo_ed_lanczos_iteration_noalloc against mo_ed_lanczos_iteration.

The no-allocation entry point serves hosts that cannot call cudaMalloc while
they run: a DMFT driver whose memory pool owns the whole GPU, or a loop that
cannot absorb the device-wide synchronisation of cudaFree.  It runs the same
Lanczos kernels on the library's fixed 32 MiB device region, so its a, b and
nstep_calc must equal those of the allocating entry point.  Each case makes
two calls in a row with different start vectors: the region keeps the first
call's contents, which must not leak into the second.

This file is collected last so that a stop at the first failure has already
run every other test; it builds its own context, so it passes alone as well.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_STATE, ERR_CAPACITY = 7, 8


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(1e-300, np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def fresh(pkg):
    s = pkg.EDSolver(0)
    yield s
    s.close()


def c3_model(pkg):
    cfg = pkg.configs.config("C3")   # 3 orbitals x 3 bath levels, sector (6,6): D = 853,776
    ek, vk = cfg.model()
    return cfg, ek, vk


def free_device_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_matches_lanczos_iteration(fresh, pkg, precision):
    """Same a, b, nstep_calc as the allocating entry point on two calls in a
    row, and no device memory taken by either call: the 32 MiB region was
    committed when the context was created."""
    cfg, ek, vk = c3_model(pkg)
    fresh.set_options(precision=precision, nstep=60)
    fresh.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    nu = nd = 6
    D = fresh.sector_dims(nu, nd)[2]
    rng = np.random.default_rng(21)
    vs = [rng.standard_normal(D) for _ in range(2)]
    ref = [fresh.lanczos_iteration(nu, nd, v) for v in vs]   # also prepares the sector
    for call in range(2):
        free0 = free_device_bytes()
        n1, a1, b1 = fresh.lanczos_iteration_noalloc(nu, nd, vs[call])
        assert free_device_bytes() == free0, call
        n0, a0, b0 = ref[call]
        assert n1 == n0 == 60, call
        assert rel(a1, a0) < 1e-12 and rel(b1, b0) < 1e-12, (call, rel(a1, a0), rel(b1, b0))
        assert b1[0] == 0.0


def test_noalloc_breakdown_small_sector(fresh, pkg):
    """Dimension-5 sector: the recurrence stops early and the unused a, b stay 0
    although the region still holds the previous call's longer run."""
    rng = np.random.default_rng(22)
    fresh.set_options(precision="fp64", nstep=30)
    ek = np.concatenate([[-1.0], rng.uniform(-1, 1, 4)])
    fresh.set_model(1, 4, 2.0, 0.0, ek, rng.uniform(0.1, 0.6, (1, 4)))
    for call in range(2):
        v = rng.standard_normal(5)
        n0, a0, b0 = fresh.lanczos_iteration(1, 0, v)
        n1, a1, b1 = fresh.lanczos_iteration_noalloc(1, 0, v)
        assert n1 == n0 <= 6
        assert rel(a1, a0) < 1e-12 and rel(b1, b0) < 1e-12
        assert not a1[n1 + 1:].any() and not b1[n1 + 1:].any()


def test_noalloc_refuses_unprepared_and_oversized(fresh, pkg):
    cfg, ek, vk = c3_model(pkg)
    fresh.set_options(precision="fp64", nstep=20)
    fresh.set_model(cfg.norb, cfg.nbath, cfg.U, cfg.J, ek, vk)
    D = fresh.sector_dims(5, 7)[2]
    with pytest.raises(pkg.EDError) as e:              # no earlier call prepared (5,7) in FP64
        fresh.lanczos_iteration_noalloc(5, 7, np.ones(D))
    assert e.value.code == ERR_STATE

    c4 = pkg.configs.config("C4")                       # sector (7,8): 41.6e6 padded elements
    ek4, vk4 = c4.model()
    fresh.set_model(c4.norb, c4.nbath, c4.U, c4.J, ek4, vk4)
    fresh.hv_tuning(7, 8, pkg.FP64)                     # prepares the sector, FP64 shape
    D4 = fresh.sector_dims(7, 8)[2]
    with pytest.raises(pkg.EDError) as e:
        fresh.lanczos_iteration_noalloc(7, 8, np.zeros(D4))
    assert e.value.code == ERR_CAPACITY
