"""The adjoint chi^2 gradient of the bath fit through a torch.autograd.Function.

The wrapper lives here, in the test harness only: forward and backward both
call mo_ed_chi2_grad_dev (the device FUNC / dfunc of func.f90:1-142) on device
tensors, the gradient being the hand-written adjoint kernel.  It is checked
with torch.autograd.gradcheck, against 5-point central differences of the
device chi^2 to 1e-7 relative (the reference carries a commented-out
finite-difference check of dfunc, func.f90:63-70), and against the oracle's
dfunc.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(1e-300, np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def chi2(pkg):
    import torch

    P = pkg.configs.fit_config(seed=4, nbatch=4)
    # the solver's kernels run on their own torch stream, ordered against
    # torch's current stream on both sides of every call (a null stream would
    # give the context a private non-blocking stream)
    st = torch.cuda.Stream()
    s = pkg.EDSolver(0, st.cuda_stream)
    om = torch.tensor(P["omega"], dtype=torch.float64, device="cuda")
    dev = torch.tensor(pkg.ed._dev_f(P["dev"]), dtype=torch.float64, device="cuda")
    norb, nbath = P["norb"], P["nbath"]
    nw = len(P["omega"])

    class Chi2(torch.autograd.Function):
        """chi^2(x) per parameter set x[b] (nbatch, nxsize) float64 on the device."""

        @staticmethod
        def forward(ctx, x):
            x = x.contiguous()
            nb, nx = x.shape
            f = torch.empty(nb, dtype=torch.float64, device=x.device)
            g = torch.empty_like(x)
            cur = torch.cuda.current_stream()
            st.wait_stream(cur)
            s.chi2_grad_dev(nb, x.data_ptr(), nw, nx, om.data_ptr(), dev.data_ptr(), nbath, norb, f.data_ptr(),
                            g.data_ptr())
            cur.wait_stream(st)
            for t in (x, f, g):
                t.record_stream(st)
            ctx.save_for_backward(g)
            return f

        @staticmethod
        def backward(ctx, gf):
            (g,) = ctx.saved_tensors
            return gf[:, None] * g

    yield Chi2, P
    s.close()


def test_gradcheck(chi2):
    import torch

    Chi2, P = chi2
    x = torch.tensor(P["X0"][:2], dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(Chi2.apply, (x,), eps=1e-7, atol=1e-8, rtol=1e-6)


def test_backward_vs_finite_differences_1e7(chi2):
    """5-point central differences (error O(h^4)) of the device chi^2 against the
    backward gradient, every parameter of two starts, to 1e-7 relative."""
    import torch

    Chi2, P = chi2
    X = torch.tensor(P["X0"][:2], dtype=torch.float64, device="cuda", requires_grad=True)
    Chi2.apply(X).sum().backward()
    G = X.grad.cpu().numpy()
    X0 = P["X0"][:2]
    nx = X0.shape[1]
    worst = 0.0
    for i in range(nx):
        h = 1e-5 * max(1.0, np.abs(X0[:, i]).max())   # well below the smallest |i w_n - eps_k|
        pts = []
        for k in (2, 1, -1, -2):
            Xk = X0.copy()
            Xk[:, i] += k * h
            pts.append(Chi2.apply(torch.tensor(Xk, dtype=torch.float64, device="cuda")).cpu().numpy())
        fd = (-pts[0] + 8 * pts[1] - 8 * pts[2] + pts[3]) / (12 * h)
        scale = np.maximum(np.abs(G[:, i]), 1e-3 * np.abs(G).max(axis=1))
        worst = max(worst, float(np.max(np.abs(fd - G[:, i]) / scale)))
    print("largest relative difference", worst)
    assert worst < 1e-7


def test_backward_vs_oracle_dfunc(chi2, oracle):
    import torch

    Chi2, P = chi2
    norb, nbath = P["norb"], P["nbath"]
    X = torch.tensor(P["X0"], dtype=torch.float64, device="cuda", requires_grad=True)
    f = Chi2.apply(X)
    f.sum().backward()
    for b in range(X.shape[0]):
        go = oracle.dfunc(P["X0"][b], norb + nbath, P["omega"], P["dev"], nbath, norb)
        fo = oracle.func(P["X0"][b], norb + nbath, P["omega"], P["dev"], nbath, norb)
        assert rel(X.grad[b].cpu().numpy(), go) < 1e-12
        assert abs(f[b].item() - fo) < 1e-12 * abs(fo)
