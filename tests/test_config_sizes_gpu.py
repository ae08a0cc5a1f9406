"""Parity at the benchmark configurations' own sizes.

The bit-exact tests elsewhere run on small meshes; these run the Hydro
configurations at full size:
  * the FP64 fused step at 4096^2 reproduces the CPU oracle bit for bit;
  * the production FP32 step over 1000 steps at 4096^2, the 64-instance FP32
    ensemble over 200 steps and the 1024^2 adjoint workload's FP32 forward
    over 200 steps stay within the relative density L1 error of 1e-5 against
    the FP64 path (itself bit-exact with the oracle), with L1 and Linf of
    every conserved field stated;
  * the FP64 adjoint at 1024^2 agrees with the oracle's FP64 tangent-linear
    model (dot-product test), and the FP32 adjoint within 1e-3.
Scheme: examples/Hydro/HydroMain.hs:134-276, Hydro.hs:37-127."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4
CFL = 0.4
FIELDS = ("density", "momentum0", "momentum1", "energy")


def make(pg, size, precision, **kw):
    h = pg.Hydro(size, precision=precision, gamma=GAMMA, **kw)
    dt = np.float64 if precision == 64 else np.float32
    h.set_scalar("cfl", CFL)
    h.set_scalar("time", 0.0)
    h.set_scalar("dR0", float(dt(1.0) / dt(size[0])))
    h.set_scalar("dR1", float(dt(1.0) / dt(size[1])))
    return h


def conserved(st):
    r, u, v, p = (a.astype(np.float64) for a in st)
    return {"density": r, "momentum0": r * u, "momentum1": r * v,
            "energy": 0.5 * r * (u * u + v * v) + p / (GAMMA - 1.0)}


def field_errors(got, ref):
    """L1 (relative to the mean magnitude of the reference) and Linf of every
    conserved field."""
    a, b = conserved(got), conserved(ref)
    out = {}
    for k in FIELDS:
        d = np.abs(a[k] - b[k])
        out[k] = (float(d.mean() / np.abs(b[k]).mean()), float(d.max()))
    return out


def flat(errs):
    return {f"{k}_{w}": v for k, (l1, li) in errs.items() for w, v in (("l1", l1), ("linf", li))}


def test_hydro_fp64_bit_exact_at_4096(om_lib, oracle, figures):
    size = (4096, 4096)
    st = oracle.hydro_init_kh(size[0], size[1], 1)
    h = make(om_lib, size, 64)
    h.set_state(st)
    h.proceed(3)
    d = np.float64(1.0) / np.float64(4096)
    ref, t, dts = oracle.hydro_run(st, 3, cyclic=True, gamma=GAMMA, cfl=CFL, dR=(d, d))
    got = h.state()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert np.array_equal(h.dt_history(3), np.array(dts))
    assert h.get_scalar("time") == t
    figures("hydro 4096^2 FP64 x3 vs CPU oracle", bit_exact=True, time=t)
    h.close()


@pytest.mark.slow
def test_hydro_fp32_1000_steps_at_4096(om_lib, figures):
    size = (4096, 4096)
    a = make(om_lib, size, 32)
    b = make(om_lib, size, 64)
    a.init_kh(1)
    b.init_kh(1)
    for x in (a, b):
        x.set_scalar("cfl", CFL)
    m0 = b.totals()
    a.proceed(1000)
    b.proceed(1000)
    errs = field_errors(a.state(), b.state())
    ta, tb = a.totals(), b.totals()
    figures("hydro 4096^2 FP32 x1000 vs FP64", **flat(errs),
            mass_rel=float((ta[0] - tb[0]) / tb[0]))
    assert errs["density"][0] <= 1e-5, errs
    assert abs(tb[0] - m0[0]) <= 1e-12 * m0[0]
    assert abs(ta[0] - m0[0]) <= 1e-6 * m0[0]
    a.close()
    b.close()


@pytest.mark.slow
def test_ensemble_64_instances_fp32_vs_fp64(om_lib, figures):
    sizes = om_lib.ensemble_sizes(64, 1)
    e32 = om_lib.Ensemble(sizes, precision=32, gamma=GAMMA)
    e64 = om_lib.Ensemble(sizes, precision=64, gamma=GAMMA)
    e32.init_kh(1000)
    e64.init_kh(1000)
    e32.step(200)
    e64.step(200)
    worst = {k: [0.0, 0.0] for k in FIELDS}
    for k in range(len(sizes)):
        errs = field_errors(e32.state(k), e64.state(k))
        assert errs["density"][0] <= 1e-5, (k, sizes[k], errs)
        for f, (l1, li) in errs.items():
            worst[f][0] = max(worst[f][0], l1)
            worst[f][1] = max(worst[f][1], li)
        t32, t64 = e32.scalar(k, "time"), e64.scalar(k, "time")
        assert abs(t32 - t64) <= 1e-4 * t64, (k, t32, t64)
    figures("ensemble 64 KH FP32 x200 vs FP64, worst instance",
            **flat({f: tuple(v) for f, v in worst.items()}))
    e32.close()
    e64.close()


def noisy_kh(oracle, size, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    return tuple(a * (1 + amp * rng.standard_normal(a.shape))
                 for a in oracle.hydro_init_kh(size[0], size[1], seed))


def adjoint_target(n, seed=7):
    x = (np.arange(n) + 0.5) / n
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(x, x)
    t = np.full((n, n), 1.5)
    amps = rng.uniform(0.2, 1.0, 8)
    amps *= 0.1 / amps.sum()
    for a in amps:
        p, q = rng.integers(-4, 5, 2)
        t += a * np.sin(2 * np.pi * (p * X + q * Y) + rng.uniform(0, 2 * np.pi))
    return t


@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 1e-3)])
def test_adjoint_tangent_linear_at_1024(om_lib, oracle, figures, precision, tol):
    size = (1024, 1024)
    steps = 3
    st = noisy_kh(oracle, size, 5)
    target = adjoint_target(1024)
    dt = np.float64 if precision == 64 else np.float32
    h = make(om_lib, size, precision)
    h.set_state(tuple(a.astype(dt) for a in st))
    loss, grad = h.adjoint_run(steps, target.astype(dt))
    st64 = tuple(a.astype(dt).astype(np.float64) for a in st)
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(2):
        d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st64, (0.1, 0.05, 0.05, 0.1)))
        fin, dfin, _ = oracle.hydro_tl_run(st64, d, steps, gamma=GAMMA, cfl=CFL)
        tl = float((2 * (fin[0] - target) * dfin[0]).sum() / fin[0].size)
        ad = sum(float((g.astype(np.float64) * b).sum()) for g, b in zip(grad, d))
        worst = max(worst, abs(ad - tl) / abs(tl))
    figures(f"adjoint 1024^2 FP{precision} x{steps} vs FP64 tangent-linear", rel=worst)
    assert worst <= tol
    h.close()


@pytest.mark.slow
def test_adjoint_workload_forward_fp32_vs_fp64(om_lib, figures):
    # the 1024^2 x 200 adjoint workload's forward in production FP32
    size = (1024, 1024)
    a = make(om_lib, size, 32)
    b = make(om_lib, size, 64)
    a.init_kh(1)
    b.init_kh(1)
    for x in (a, b):
        x.set_scalar("cfl", CFL)
    a.proceed(200)
    b.proceed(200)
    errs = field_errors(a.state(), b.state())
    figures("adjoint workload forward 1024^2 FP32 x200 vs FP64", **flat(errs))
    assert errs["density"][0] <= 1e-5, errs
    a.close()
    b.close()
