"""Hand-written adjoints against float64 central finite differences.

The loss is the differentiation workload's: the MSE between an aggregate and
the aggregate of the same series with y perturbed, NaN pixels masked with
nan_to_num on both sides.  Gradients with respect to v and y from the
adjoint kernels are compared with central differences of (a) the GPU forward
and (b) the CPU oracle forward (the reference algorithm) on random
coordinates.  Coordinates where the one-sided differences disagree sit on a
kink of the piecewise-smooth coverage (a clamp edge, a scanline limit, the
previous-segment choice); they are reported and excluded, and must be rare.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import autograd as ag
from datashader_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _series(nseries=12, length=160, seed=0):
    x, y, v, _ = synthetic.time_series_np(nseries, length, seed)
    return x, y, v


def _canvas(y):
    lo, hi = float(np.nanmin(y)), float(np.nanmax(y))
    pad = 0.05 * (hi - lo)
    return ds.Canvas(plot_width=160, plot_height=80, x_range=(0.0, 1.0), y_range=(lo - pad, hi + pad))


def _loss_gpu(x, y, v, target, cvs, lw=1.5):
    agg = ag.line_sum(x, y, v, cvs, lw)
    return torch.mean((torch.nan_to_num(agg) - target) ** 2)


def _loss_oracle(x, y, v, target_np, cvs, lw=1.5):
    agg = oracle.line_axis0({"x": x, "y": y, "v": v}, "x", "y", cvs.plot_width, cvs.plot_height,
                            cvs.x_range, cvs.y_range, [oracle.spec("sum", "v")], line_width=lw)[0]
    return float(np.mean((np.nan_to_num(agg) - target_np) ** 2))


def test_line_sum_adjoint_vs_finite_differences():
    x, y, v = _series()
    rng = np.random.default_rng(7)
    y_t = y + rng.normal(0, 0.005, y.shape)
    cvs = _canvas(y)
    X = torch.from_numpy(x).cuda()
    target = torch.nan_to_num(ag.line_sum(X, torch.from_numpy(y_t).cuda(), torch.from_numpy(v).cuda(), cvs)).detach()
    target_np = target.cpu().numpy()
    Y = torch.from_numpy(y).cuda().requires_grad_(True)
    V = torch.from_numpy(v).cuda().requires_grad_(True)
    loss = _loss_gpu(X, Y, V, target, cvs)
    loss.backward()
    gy, gv = Y.grad.cpu().numpy(), V.grad.cpu().numpy()
    valid = np.flatnonzero(~np.isnan(y))
    picks = rng.choice(valid, 64, replace=False)

    def loss_at(which, k, d):
        arr = (y if which == "y" else v).copy()
        arr[k] += d
        yy, vv = (arr, v) if which == "y" else (y, arr)
        return float(_loss_gpu(X, torch.from_numpy(yy).cuda(), torch.from_numpy(vv).cuda(), target, cvs))

    kinks, checked = [], 0
    for which, grad, base in (("y", gy, y), ("v", gv, v)):
        for k in picks[:32] if which == "y" else picks[32:]:
            # The loss is exactly quadratic in v (the coverage does not depend
            # on v): no kinks, and the central difference is exact.  In y it is
            # piecewise smooth: the one-sided asymmetry a(h) = (f(h) + f(-h) -
            # 2 f(0)) / h shrinks like h on a smooth piece and stays at the
            # slope jump on a kink.
            h = 1e-6 if which == "y" else 1e-3
            f0, fp, fm = loss_at(which, k, 0.0), loss_at(which, k, h), loss_at(which, k, -h)
            central = (fp - fm) / (2 * h)
            scale = max(abs(central), abs(grad[k]), 1e-12)
            if which == "y":
                a1 = (fp + fm - 2 * f0) / h
                q = h / 8
                a2 = (loss_at(which, k, q) + loss_at(which, k, -q) - 2 * f0) / q
                if abs(a2) > 0.5 * abs(a1) and abs(a1) > 1e-6 * scale:
                    kinks.append((which, int(k)))
                    continue
            checked += 1
            assert abs(grad[k] - central) <= 1e-4 * scale + 1e-10, (which, k, grad[k], central)
            # the reference algorithm's own finite difference (CPU oracle forward)
            arrp, arrm = base.copy(), base.copy()
            arrp[k] += h
            arrm[k] -= h
            if which == "y":
                ref = (_loss_oracle(x, arrp, v, target_np, cvs) - _loss_oracle(x, arrm, v, target_np, cvs)) / (2 * h)
            else:
                ref = (_loss_oracle(x, y, arrp, target_np, cvs) - _loss_oracle(x, y, arrm, target_np, cvs)) / (2 * h)
            assert abs(grad[k] - ref) <= 1e-4 * max(abs(ref), abs(grad[k]), 1e-12) + 1e-10, (which, k, grad[k], ref)
    assert checked >= 56, f"too many kink coordinates: {kinks}"


def test_line_sum_adjoint_value_linearity():
    """The aggregate is linear in v: the v-gradient of <w, agg> is exact."""
    x, y, v = _series(6, 120, seed=3)
    cvs = _canvas(y)
    X, Y = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    V = torch.from_numpy(v).cuda().requires_grad_(True)
    agg = ag.line_sum(X, Y, V, cvs)
    w = torch.randn_like(agg)
    (torch.nan_to_num(agg) * w).sum().backward()
    # <w, agg(v)> = sum_i v_i * c_i, so c_i = <w, agg(e_i)>
    for i in (5, 40, 77):
        e = np.zeros_like(v)
        e[i] = 1.0
        ai = torch.nan_to_num(ag.line_sum(X, Y, torch.from_numpy(e).cuda(), cvs))
        assert abs(float((ai * w).sum()) - float(V.grad[i])) <= 1e-10 * max(1.0, abs(float(V.grad[i])))


@pytest.mark.parametrize("mean", [False, True])
def test_points_adjoint_vs_finite_differences(mean):
    rng = np.random.default_rng(11)
    n = 20_000
    x, y = synthetic.gaussian_mixture_np(n, seed=2, dtype=np.float32)
    v = rng.lognormal(0, 1, n)
    cvs = ds.Canvas(plot_width=64, plot_height=64, x_range=(-4, 4), y_range=(-4, 4))
    X, Y = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    V = torch.from_numpy(v).cuda().requires_grad_(True)
    f = ag.points_mean if mean else ag.points_sum
    w = torch.randn(64, 64, dtype=torch.float64, device="cuda")
    (torch.nan_to_num(f(X, Y, V, cvs)) * w).sum().backward()
    for i in rng.choice(n, 16, replace=False):
        h = 1e-3
        vp, vm = v.copy(), v.copy()
        vp[i] += h
        vm[i] -= h
        lp = float((torch.nan_to_num(f(X, Y, torch.from_numpy(vp).cuda(), cvs)) * w).sum())
        lm = float((torch.nan_to_num(f(X, Y, torch.from_numpy(vm).cuda(), cvs)) * w).sum())
        assert abs((lp - lm) / (2 * h) - float(V.grad[i])) <= 1e-7 * max(1.0, abs(float(V.grad[i])))


def test_line_adjoint_work_order_matches_row_order():
    """The adjoint with a workspace recomputes segments in work order; without
    one, in row order.  The pixels of a warp's 32 segments are worked off by
    case, so a segment's dL/dv terms (float64) and its float32 tangent terms
    are summed in an order that depends on its warp's other segments: equal
    up to float64 rounding (dL/dv, 1e-12 relative) and float32 rounding of
    the tangent sums (dL/dy, 1e-5 relative)."""
    import ctypes
    from datashader_gb300 import _native as N
    from datashader_gb300.autograd import _canvas_desc
    from datashader_gb300.core import dsgb_dtype
    x, y, v = _series(nseries=40, length=400, seed=5)
    cvs = _canvas(y)
    dev = torch.device("cuda")
    xt, yt, vt = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (x, y, v))
    rng = np.random.default_rng(5)
    grad = torch.from_numpy(rng.standard_normal((cvs.plot_height, cvs.plot_width))).to(dev)
    n = vt.numel()
    cv = _canvas_desc(cvs, cvs.x_range, cvs.y_range)
    cols = (N.Column * 3)(N.Column(xt.data_ptr(), dsgb_dtype(xt), 0), N.Column(yt.data_ptr(), dsgb_dtype(yt), 0),
                          N.Column(vt.data_ptr(), dsgb_dtype(vt), 0))
    L = N.lib()
    st = torch.cuda.current_stream().cuda_stream
    out = []
    for ordered in (False, True):
        gv = torch.empty(n, dtype=torch.float64, device=dev)
        gy = torch.empty(n, dtype=torch.float64, device=dev)
        if ordered:
            wsz = int(L.dsgb_line_workspace_size(n))
            ws = torch.empty(wsz, dtype=torch.uint8, device=dev)
            N.check(L.dsgb_line_axis0_backward_ws(cols, 3, n, 0, 1, 2, ctypes.byref(cv), 1.5, 1, grad.data_ptr(),
                                                  None, gv.data_ptr(), gy.data_ptr(), ws.data_ptr(), wsz, st),
                    "dsgb_line_axis0_backward_ws")
        else:
            N.check(L.dsgb_line_axis0_backward(cols, 3, n, 0, 1, 2, ctypes.byref(cv), 1.5, 1, grad.data_ptr(),
                                               None, gv.data_ptr(), gy.data_ptr(), st), "dsgb_line_axis0_backward")
        out.append((gv.cpu().numpy(), gy.cpu().numpy()))
    (gv0, gy0), (gv1, gy1) = out
    np.testing.assert_allclose(gv1, gv0, rtol=1e-12, atol=1e-12 * np.abs(gv0).max())
    np.testing.assert_allclose(gy1, gy0, rtol=1e-5, atol=1e-6 * np.abs(gy0).max())
    assert np.abs(gv0).max() > 0 and np.abs(gy0).max() > 0


@pytest.mark.parametrize("mean", [False, True])
def test_points_adjoint_strided_and_host_inputs(mean):
    """Strided views (columns of an (n, 2) array), a stride-0 expanded value
    column and host x/y give the gradients of the contiguous device inputs:
    the backward reads the frame's device copies, not the caller's tensors."""
    n = 4096
    x, y = synthetic.gaussian_mixture_np(n, seed=6, dtype=np.float32)
    v = np.random.default_rng(6).lognormal(0, 1, n)
    cvs = ds.Canvas(plot_width=32, plot_height=32, x_range=(-4, 4), y_range=(-4, 4))
    f = ag.points_mean if mean else ag.points_sum
    w = torch.randn(32, 32, dtype=torch.float64, device="cuda")
    X, Y = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    V = torch.from_numpy(v).cuda().requires_grad_(True)
    (torch.nan_to_num(f(X, Y, V, cvs)) * w).sum().backward()
    ref = V.grad.clone()
    xy = torch.stack([X, Y], dim=1)                     # x, y as stride-2 views
    V2 = torch.from_numpy(v).cuda().requires_grad_(True)
    (torch.nan_to_num(f(xy[:, 0], xy[:, 1], V2, cvs)) * w).sum().backward()
    assert torch.equal(V2.grad, ref)
    V3 = torch.from_numpy(v).cuda().requires_grad_(True)
    (torch.nan_to_num(f(X.cpu(), Y.cpu(), V3, cvs)) * w).sum().backward()   # host x/y, device v
    assert torch.equal(V3.grad, ref)
    c = torch.tensor([1.5], dtype=torch.float64, device="cuda", requires_grad=True)
    (torch.nan_to_num(f(X, Y, c.expand(n), cvs)) * w).sum().backward()        # stride-0 value column
    assert c.grad is not None and torch.isfinite(c.grad).all()
    if not mean:   # d/dc of sum_px w * (c * count) is sum_i w[pixel(i)]
        torch.testing.assert_close(c.grad, ref.sum().reshape(1), rtol=1e-12, atol=0)


def test_line_adjoint_strided_inputs():
    x, y, v = _series(4, 100, seed=9)
    cvs = _canvas(y)
    X, Y0, V0 = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, y, v))
    Y = Y0.clone().requires_grad_(True)
    V = V0.clone().requires_grad_(True)
    w = torch.randn(cvs.plot_height, cvs.plot_width, dtype=torch.float64, device="cuda")
    (torch.nan_to_num(ag.line_sum(X, Y, V, cvs)) * w).sum().backward()
    big = torch.stack([X, Y0, V0], dim=1)               # every column a stride-3 view
    Ys = big[:, 1].detach().requires_grad_(True)
    Vs = big[:, 2].detach().requires_grad_(True)
    (torch.nan_to_num(ag.line_sum(big[:, 0], Ys, Vs, cvs)) * w).sum().backward()
    # the work order's ties fall by atomics, and a segment's dL/dv terms sum in
    # an order set by its warp's other segments: equal up to rounding
    torch.testing.assert_close(Vs.grad, V.grad, rtol=1e-12, atol=1e-12 * float(V.grad.abs().max()))
    torch.testing.assert_close(Ys.grad, Y.grad, rtol=1e-5, atol=1e-6 * float(Y.grad.abs().max()))
