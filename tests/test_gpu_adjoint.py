"""The Acc adjoint (tg_acc_vjp) and the differentiable leapfrog.

* VJP against PyTorch FP64 autograd through a naive O(N^2) restatement of
  the softened acceleration: FP64 to 1e-10 relative, split FP32 (the
  double-single adjoint kernel) to 1e-9.
* Gradient of a leapfrog trajectory loss with respect to initial positions,
  velocities and masses (adjoint, checkpointed) against FP64 central finite
  differences of the same forward map: 1e-6 relative, in FP64 and in split
  FP32 (ordered Acc forward, double-single adjoint).
* TG_PREC_DS32X (double-single forces and adjoint): the forward within 1e-10
  of FP64 at N = 65536 (ordered-path size), the VJP within 1e-9 of autograd,
  the leapfrog gradient within 1e-8 of the FP64 adjoint; other kernels
  refuse it.
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


@pytest.mark.parametrize("prec,tol", [("float64", 1e-10), ("ds32", 1e-9), ("ds32x", 1e-9)])
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


def naive_leapfrog(r, v, m, e2, dt, steps):
    """Kick-drift-kick with the naive acceleration, differentiated by torch."""
    a = naive_acc(r, m, e2)
    for _ in range(steps):
        v = v + a * (0.5 * dt)
        r = r + v * dt
        a = naive_acc(r, m, e2)
        v = v + a * (0.5 * dt)
    return r, v


def test_leapfrog_adjoint_matches_torch_autograd(ad):
    """The checkpointed adjoint leapfrog against PyTorch FP64 autograd
    through the naive O(N^2) leapfrog: the same discrete map, 1e-10."""
    n, steps, dt = 192, 12, 1.0 / 256
    r0, v0, m, e2 = system(n, seed=6)
    target = r0 + 0.01
    grads = []
    for fn in ("adjoint", "naive"):
        r = r0.clone().requires_grad_(True)
        v = v0.clone().requires_grad_(True)
        mm = m.clone().requires_grad_(True)
        if fn == "adjoint":
            rf, _ = ad.leapfrog(r, v, mm, e2, dt, steps, "float64", checkpoint_every=4)
        else:
            rf, _ = naive_leapfrog(r, v, mm, e2, dt, steps)
        ad.loss_to_target(rf, target).backward()
        grads.append((r.grad, v.grad, mm.grad))
    for g1, g2 in zip(*grads):
        assert (g1 - g2).norm() <= 1e-10 * g2.norm()


def test_leapfrog_gradient_matches_finite_differences(ad):
    """Richardson-extrapolated central differences (h and 2h) of the FP64
    forward map against the FP64 adjoint, on a smooth problem (pair
    softening 1e-2): 1e-6 relative."""
    n, steps, dt = 128, 8, 1.0 / 256
    r0, v0, m, e2 = system(n, seed=3, e2=1e-2)
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
        for which, base, grad, h in (("r", r0, r.grad, 1e-4), ("v", v0, v.grad, 1e-4), ("m", m, mm.grad, 1e-6)):
            for _ in range(4):
                idx = tuple(int(rng.integers(0, s)) for s in base.shape)

                def central(step):
                    plus, minus = base.clone(), base.clone()
                    plus[idx] += step
                    minus[idx] -= step
                    ap = {"r": r0, "v": v0, "m": m}
                    am = dict(ap)
                    ap[which], am[which] = plus, minus
                    return float(loss(ap["r"], ap["v"], ap["m"]) - loss(am["r"], am["v"], am["m"])) / (2 * step)

                fd = (4 * central(h) - central(2 * h)) / 3
                g = float(grad[idx])
                assert abs(fd - g) <= 1e-6 * abs(g) + 1e-9 * float(grad.abs().max()), (which, idx, fd, g)


def test_ds32_leapfrog_gradient_matches_fp64_finite_differences(ad):
    """The split-FP32 leapfrog (Acc on the ordered split-FP32 path at
    N = 4096, the double-single adjoint) differentiated by the adjoint,
    against Richardson-extrapolated FP64 central differences of the FP64
    forward map: 1e-6 relative, on 12 coordinates of r0, v0 and m."""
    n, steps, dt = 4096, 4, 1.0 / 256
    r0, v0, m, e2 = system(n, seed=8, e2=1e-4)
    target, _ = ad.leapfrog(r0 + 0.01, v0, m * 1.01, e2, dt, steps, "float64")

    def loss(r, v, mm, prec):
        rf, _ = ad.leapfrog(r, v, mm, e2, dt, steps, prec, checkpoint_every=2)
        return ad.loss_to_target(rf, target)

    r = r0.clone().requires_grad_(True)
    v = v0.clone().requires_grad_(True)
    mm = m.clone().requires_grad_(True)
    loss(r, v, mm, "ds32").backward()
    rng = np.random.default_rng(9)
    with torch.no_grad():
        for which, base, grad, h in (("r", r0, r.grad, 1e-4), ("v", v0, v.grad, 1e-4), ("m", m, mm.grad, 1e-7)):
            for _ in range(4):
                idx = tuple(int(rng.integers(0, s)) for s in base.shape)

                def central(step):
                    plus, minus = base.clone(), base.clone()
                    plus[idx] += step
                    minus[idx] -= step
                    ap = {"r": r0, "v": v0, "m": m}
                    am = dict(ap)
                    ap[which], am[which] = plus, minus
                    return float(loss(ap["r"], ap["v"], ap["m"], "float64")
                                 - loss(am["r"], am["v"], am["m"], "float64")) / (2 * step)

                fd = (4 * central(h) - central(2 * h)) / 3
                g = float(grad[idx])
                assert abs(fd - g) <= 1e-6 * abs(g) + 1e-9 * float(grad.abs().max()), (which, idx, fd, g)


def test_ds32x_forward_at_ordered_size(ad):
    """N = 65536 takes the ordered path in ds32; ds32x runs the double-single
    kernel for every particle: per-particle error against FP64 <= 1e-10."""
    r, v, m, e2 = system(65536, seed=10, e2=1e-6)
    a64 = ad.acc_forward(r, m, e2, ad.PREC["float64"])
    ax = ad.acc_forward(r, m, e2, ad.PREC["ds32x"])
    err = ((ax - a64).norm(dim=0) / a64.norm(dim=0)).max()
    assert float(err) <= 1e-10, float(err)


def test_ds32x_leapfrog_gradient_matches_fp64_adjoint(ad):
    n, steps, dt = 4096, 8, 1.0 / 256
    r0, v0, m, e2 = system(n, seed=11, e2=1e-4)
    target, _ = ad.leapfrog(r0 + 0.01, v0, m * 1.01, e2, dt, steps, "float64")
    grads = {}
    for prec in ("float64", "ds32x"):
        r = r0.clone().requires_grad_(True)
        v = v0.clone().requires_grad_(True)
        mm = m.clone().requires_grad_(True)
        rf, _ = ad.leapfrog(r, v, mm, e2, dt, steps, prec, checkpoint_every=4)
        ad.loss_to_target(rf, target).backward()
        grads[prec] = (r.grad, v.grad, mm.grad)
    for gx, g64 in zip(grads["ds32x"], grads["float64"]):
        assert float((gx - g64).norm() / g64.norm()) <= 1e-8


def test_ds32x_refused_by_other_kernels(ad):
    from tupan_gb300 import _native
    r, v, m, e2 = system(64, seed=12)
    out = torch.empty(64, dtype=torch.float64, device="cuda")
    p = [m.data_ptr(), r[0].data_ptr(), r[1].data_ptr(), r[2].data_ptr(), e2.data_ptr()]
    with pytest.raises(_native.TupanGB300Error, match="DS32X"):
        _native.call_device("phi", 64, p, 64, p, (), [out.data_ptr()], _native.PREC_DS32X, _native.current_stream())
