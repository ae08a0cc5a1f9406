"""Reverse-mode adjoint of the Hydro step against the oracle's FP64
tangent-linear model (dot-product test) and against central finite
differences of the forward.  States carry small noise on every field so the
CFL minimum has a unique arg-min (at a tie the step is not differentiable)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4
CFL = 0.4


def noisy_kh(oracle, size, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    return tuple(a * (1 + amp * rng.standard_normal(a.shape))
                 for a in oracle.hydro_init_kh(size[0], size[1], seed))


def make(pg, size, precision, **kw):
    h = pg.Hydro(size, precision=precision, gamma=GAMMA, **kw)
    h.set_scalar("cfl", CFL)
    h.set_scalar("dR0", 1.0 / size[0])
    h.set_scalar("dR1", 1.0 / size[1])
    return h


@pytest.mark.parametrize("size", [(32, 24), (64, 64)])
def test_vjp_dot_product_fp64(om_lib, oracle, size):
    st = noisy_kh(oracle, size, 3)
    rng = np.random.default_rng(11)
    ub = tuple(rng.standard_normal(a.shape) for a in st)
    d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st, (0.1, 0.05, 0.05, 0.1)))
    h = make(om_lib, size, 64)
    h.set_state(st)
    pb = h.vjp(ub)
    _, dout, _ = oracle.hydro_tl_run(st, d, 1, gamma=GAMMA, cfl=CFL)
    lhs = sum(float((a * b).sum()) for a, b in zip(ub, dout))
    rhs = sum(float((a * b).sum()) for a, b in zip(pb, d))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1e-30), (lhs, rhs)
    h.close()


def loss_of(h, st, steps, target):
    h.set_state(st)
    h.set_scalar("time", 0.0)
    h.proceed(steps)
    r = h.read("density").astype(np.float64)
    return float(((r - target) ** 2).mean())


@pytest.mark.parametrize("precision,steps,tol", [(64, 12, 1e-4), (32, 12, 2e-3)])
def test_gradient_vs_finite_differences(om_lib, oracle, precision, steps, tol):
    # The loss is piecewise smooth (the CFL arg-min, wave-speed cases and
    # limiter picks switch): a perturbation of 1e-6 already crosses such
    # switches on this grid (the difference quotient moves by ~4e-4 between
    # eps 1e-6 and 1e-7 while the tangent-linear value stays put), so the
    # difference step is 1e-7 (FP64 forward).
    size = (48, 40)
    st = noisy_kh(oracle, size, 5)
    dt = np.float64 if precision == 64 else np.float32
    st = tuple(a.astype(dt) for a in st)
    x = (np.arange(size[0]) + 0.5) / size[0]
    y = (np.arange(size[1]) + 0.5) / size[1]
    target = (1.5 + 0.1 * np.sin(2 * np.pi * (x[None, :] + 2 * y[:, None]))).astype(dt)
    h = make(om_lib, size, precision)
    h.set_state(st)
    loss, grad = h.adjoint_run(steps, target, checkpoint_every=4)
    assert loss > 0
    fd_h = make(om_lib, size, 64)     # finite differences of the FP64 forward
    st64 = tuple(a.astype(np.float64) for a in st)
    assert abs(loss_of(fd_h, st64, steps, target.astype(np.float64)) - loss) < 1e-5 * loss
    rng = np.random.default_rng(7)
    for _ in range(3):
        d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st64, (0.1, 0.05, 0.05, 0.1)))
        eps = 1e-7
        lp = loss_of(fd_h, tuple(a + eps * b for a, b in zip(st64, d)), steps, target)
        lm = loss_of(fd_h, tuple(a - eps * b for a, b in zip(st64, d)), steps, target)
        fd = (lp - lm) / (2 * eps)
        ad = sum(float((g.astype(np.float64) * b).sum()) for g, b in zip(grad, d))
        assert abs(ad - fd) <= tol * abs(fd), (ad, fd)
    h.close()
    fd_h.close()


def test_adjoint_leaves_final_state(om_lib, oracle):
    size = (32, 32)
    st = noisy_kh(oracle, size, 9)
    h = make(om_lib, size, 64)
    h.set_state(st)
    target = np.full(st[0].shape, 1.5)
    h.adjoint_run(5, target)
    ref, t, _ = oracle.hydro_run(st, 5, cyclic=True, gamma=GAMMA, cfl=CFL)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    h.close()


@pytest.mark.parametrize("ck", [1, 4, 0])
def test_multistep_gradient_vs_tangent_linear(om_lib, oracle, ck):
    # <grad, d> against the oracle's FP64 tangent-linear run (which follows
    # the dt of every step through its arg-min cell): equal to rounding
    size = (48, 40)
    steps = 10
    st = noisy_kh(oracle, size, 5)
    x = (np.arange(size[0]) + 0.5) / size[0]
    y = (np.arange(size[1]) + 0.5) / size[1]
    target = 1.5 + 0.1 * np.sin(2 * np.pi * (x[None, :] + 2 * y[:, None]))
    h = make(om_lib, size, 64)
    h.set_state(st)
    loss, grad = h.adjoint_run(steps, target, checkpoint_every=ck)
    rng = np.random.default_rng(3)
    for _ in range(2):
        d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st, (0.1, 0.05, 0.05, 0.1)))
        fin, dfin, _ = oracle.hydro_tl_run(st, d, steps, gamma=GAMMA, cfl=CFL)
        tl = float((2 * (fin[0] - target) * dfin[0]).sum() / fin[0].size)
        ad = sum(float((g * b).sum()) for g, b in zip(grad, d))
        assert abs(ad - tl) <= 1e-12 * abs(tl), (ad, tl)
    h.close()


def test_forward_backward_pair(om_lib, oracle):
    # om_hydro_forward / om_hydro_backward with an arbitrary cotangent on all
    # four fields: <cot, TL(d)> == <backward(cot), d>; the same tape serves a
    # second cotangent, and the loss cotangent reproduces adjoint_run
    size = (48, 40)
    steps = 7
    st = noisy_kh(oracle, size, 11)
    h = make(om_lib, size, 64)
    h.set_state(st)
    rng = np.random.default_rng(17)
    with h.forward(steps, checkpoint_every=3) as tape:
        ref, _, _ = oracle.hydro_run(st, steps, cyclic=True, gamma=GAMMA, cfl=CFL)
        for a, b in zip(h.state(), ref):
            assert np.array_equal(a, b)
        d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st, (0.1, 0.05, 0.05, 0.1)))
        _, dfin, _ = oracle.hydro_tl_run(st, d, steps, gamma=GAMMA, cfl=CFL)
        for _ in range(2):
            cot = tuple(rng.standard_normal(a.shape) for a in st)
            grad = tape.backward(cot)
            tl = sum(float((c * t).sum()) for c, t in zip(cot, dfin))
            ad = sum(float((g * b).sum()) for g, b in zip(grad, d))
            assert abs(ad - tl) <= 1e-12 * abs(tl), (ad, tl)
        for a, b in zip(h.state(), ref):     # left at the final state
            assert np.array_equal(a, b)
        target = np.full(st[0].shape, 1.5)
        loss_cot = (2 * (ref[0] - target) / ref[0].size, np.zeros_like(ref[0]),
                    np.zeros_like(ref[0]), np.zeros_like(ref[0]))
        g1 = tape.backward(loss_cot)
    h.set_state(st)
    h.set_scalar("time", 0.0)
    _, g2 = h.adjoint_run(steps, target, checkpoint_every=3)
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    h.close()


def test_backward_rejects_foreign_tape(om_lib, oracle):
    size = (32, 32)
    st = noisy_kh(oracle, size, 2)
    a, b = make(om_lib, size, 64), make(om_lib, size, 64)
    a.set_state(st)
    b.set_state(st)
    with a.forward(2) as tape:
        with pytest.raises(om_lib.OMError):
            b.backward(tape, [np.zeros(st[0].shape)] * 4)
    a.close()
    b.close()


@pytest.mark.parametrize("precision,size,tile,limit", [(32, (64, 48), 0, 0), (64, (64, 48), 0, 0),
                                                       (32, (128, 96), 0, 0),
                                                       (32, (128, 96), 16, 0),
                                                       (32, (128, 96), 32, 0),
                                                       (32, (256, 128), 0, 1)])
def test_segment_tapes_match_retaping(om_lib, oracle, monkeypatch, precision, size, tile, limit):
    # The backward pass recomputes each segment with the taped step, keeping
    # one tape per step; when those tapes cannot be allocated it recomputes
    # with the plain step and tapes each step again before its reverse.  The
    # taped step writes the same states as the plain one, so both paths give
    # the same gradient bit for bit.  128 x 96 FP32 runs the persistent
    # 32 x 32 kernel (plain and taped; paired with tile_x 0 and 16, one wall
    # per thread with tile_x 32), 64 x 48 the tile kernels; 256 x 128 with
    # one CTA (32 tiles, 16 per group) its two-group form.
    steps = 9
    st = noisy_kh(oracle, size, 21)
    if precision == 32:
        st = tuple(a.astype(np.float32) for a in st)
    rng = np.random.default_rng(5)
    cot = tuple(rng.standard_normal(a.shape).astype(st[0].dtype) for a in st)
    grads = []
    for retape in (False, True):
        h = make(om_lib, size, precision, tile_x=tile, grid_limit=limit)
        h.set_state(st)
        if retape:
            monkeypatch.setenv("OM_FAIL_ALLOC_AFTER", "0")
        tape = h.forward(steps, checkpoint_every=4)
        monkeypatch.delenv("OM_FAIL_ALLOC_AFTER", raising=False)
        with tape:
            grads.append(tape.backward(cot))
        h.close()
    for a, b in zip(*grads):
        assert np.array_equal(a, b)


def test_adjoint_step_timers(om_lib, oracle):
    st = tuple(a.astype(np.float32) for a in noisy_kh(oracle, (128, 96), 4))
    h = make(om_lib, (128, 96), 32)
    h.set_state(st)
    assert h.time_tape(2) > 0 and h.time_vjp(2) > 0
    for a, b in zip(h.state(), st):            # neither timer moves the handle
        assert np.array_equal(a, b)
    h.close()
