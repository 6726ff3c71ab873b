"""Failure paths through the C-ABI (the reference's only one is die -> MPI_Abort,
sys.F:5-41): non-finite model input is refused with MO_ED_ERR_ARG, and a
zero-norm start vector ends the Lanczos recurrence at once.  Every case makes
the error on the host; nothing here faults a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_STATE = 1, 7


@pytest.mark.parametrize("where", ["ek", "vk", "U", "J"])
def test_nan_model_input_refused(solver, pkg, where):
    ek = np.array([-1.0, -0.5, 0.3, 0.7])
    vk = np.full((1, 3), 0.3)
    U, J = 2.0, 0.0
    if where == "ek":
        ek[2] = np.nan
    elif where == "vk":
        vk[0, 1] = np.inf
    elif where == "U":
        U = np.nan
    else:
        J = -np.inf
    with pytest.raises(pkg.EDError) as e:
        solver.set_model(1, 3, U, J, ek, vk)
    assert e.value.code == ERR_ARG
    assert "non-finite" in str(e.value)
    # the context stays usable
    solver.set_model(1, 3, 2.0, 0.0, np.array([-1.0, -0.5, 0.3, 0.7]), np.full((1, 3), 0.3))
    assert solver.sector_dims(2, 2)[2] == 36


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_zero_norm_start_vector(solver, pkg, precision):
    """b(0) = |v|^2 = 0: no step is taken (nstep_calc = 0, a = b = 0); the
    reference would divide by zero here (ed_lanczos.F90:33-36)."""
    solver.set_options(precision=precision, nstep=20)
    solver.set_model(1, 3, 2.0, 0.0, np.array([-1.0, -0.5, 0.3, 0.7]), np.full((1, 3), 0.3))
    n, a, b = solver.lanczos_iteration(2, 2, np.zeros(36))
    assert n == 0 and not a.any() and not b.any()
    # and a proper start vector afterwards runs normally
    n, a, b = solver.lanczos_iteration(2, 2, np.ones(36))
    assert n > 0 and b[1] > 0


def test_calls_before_model_refused(pkg):
    s = pkg.EDSolver(0)
    try:
        with pytest.raises(pkg.EDError) as e:
            s.sector_dims(1, 1)
        assert e.value.code == ERR_STATE
        with pytest.raises(pkg.EDError) as e:
            s.ed_solve()
        assert e.value.code == ERR_STATE
    finally:
        s.close()
