"""The Acc adjoint (tg_acc_vjp) and the differentiable leapfrog.

* VJP against PyTorch FP64 autograd through a naive O(N^2) restatement of
  the softened acceleration: FP64 to 1e-10 relative, split FP32 to 1e-4.
* Gradient of a leapfrog trajectory loss with respect to initial positions,
  velocities and masses (adjoint, checkpointed) against FP64 central finite
  differences of the same forward map: 1e-6 relative.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ad():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import autodiff
    return autodiff


def system(n, seed, e2=1e-4):
    g = torch.Generator().manual_seed(seed)
    r = torch.randn(3, n, generator=g, dtype=torch.float64) * 0.6
    v = torch.randn(3, n, generator=g, dtype=torch.float64) * 0.3
    m = torch.rand(n, generator=g, dtype=torch.float64) / n + 0.5 / n
    e = torch.full((n,), e2 / 2, dtype=torch.float64)
    return [t.cuda() for t in (r, v, m, e)]


def naive_acc(r, m, e2):
    d = r[:, :, None] - r[:, None, :]                       # r_i - r_j
    r2 = (d * d).sum(0)
    s = r2 + e2[:, None] + e2[None, :]
    mask = r2 > 0
    q3 = torch.where(mask, s ** -1.5, torch.zeros_like(s))
    return -(d * (m[None, :] * q3)[None]).sum(2)


@pytest.mark.parametrize("prec,tol", [("float64", 1e-10), ("ds32", 1e-4)])
def test_vjp_matches_torch_autograd(ad, prec, tol):
    r, v, m, e2 = system(300, seed=1)
    g = torch.randn(3, 300, dtype=torch.float64, device="cuda")
    rr = r.clone().requires_grad_(True)
    mm = m.clone().requires_grad_(True)
    naive_acc(rr, mm, e2).backward(g)
    rb, mb = ad.acc_vjp(r, m, e2, g, ad.PREC[prec])
    assert (rb - rr.grad).norm() <= tol * rr.grad.norm()
    assert (mb - mm.grad).norm() <= tol * mm.grad.norm()


def test_forward_matches_naive(ad):
    r, v, m, e2 = system(200, seed=2)
    a = ad.acc_forward(r, m, e2, ad.PREC["float64"])
    ref = naive_acc(r, m, e2)
    assert (a - ref).norm() <= 1e-12 * ref.norm()


def test_leapfrog_gradient_matches_finite_differences(ad):
    n, steps, dt = 256, 16, 1.0 / 256
    r0, v0, m, e2 = system(n, seed=3)
    target, _ = ad.leapfrog(r0 + 0.01, v0, m * 1.01, e2, dt, steps, "float64")

    def loss(r, v, mm):
        rf, _ = ad.leapfrog(r, v, mm, e2, dt, steps, "float64", checkpoint_every=4)
        return ad.loss_to_target(rf, target)

    r = r0.clone().requires_grad_(True)
    v = v0.clone().requires_grad_(True)
    mm = m.clone().requires_grad_(True)
    loss(r, v, mm).backward()
    rng = np.random.default_rng(4)
    with torch.no_grad():
        for which, base, grad, h in (("r", r0, r.grad, 1e-6), ("v", v0, v.grad, 1e-6), ("m", m, mm.grad, 1e-9)):
            for _ in range(4):
                idx = tuple(int(rng.integers(0, s)) for s in base.shape)
                plus, minus = base.clone(), base.clone()
                plus[idx] += h
                minus[idx] -= h
                args_p = {"r": r0, "v": v0, "m": m}
                args_m = dict(args_p)
                args_p[which], args_m[which] = plus, minus
                fd = (loss(args_p["r"], args_p["v"], args_p["m"]) - loss(args_m["r"], args_m["v"], args_m["m"])) / (2 * h)
                g = grad[idx]
                assert abs(float(fd - g)) <= 1e-6 * max(abs(float(g)), 1e-3 * float(grad.abs().max())), (which, idx)
