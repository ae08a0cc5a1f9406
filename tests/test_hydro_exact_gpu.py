"""The GPU Hydro paths against exact solutions (the cases of the reference's
exact-solution harness, attic/GA.reproduce/massive-test.cu:52-118, on
periodic meshes): entropy waves along an axis and at 45 degrees, a sound
wave and Sod's shock tube, in FP64 and in the production FP32 build."""
import numpy as np
import pytest

from oracle import riemann_exact as RX

pytestmark = pytest.mark.gpu


def run_until(pg, state, T, g, precision, cfl=0.4):
    h = pg.Hydro((state[0].shape[1], state[0].shape[0]), precision=precision, gamma=g)
    h.set_state(tuple(a.astype(np.float64 if precision == 64 else np.float32) for a in state))
    h.set_scalar("cfl", cfl)
    h.set_scalar("time", 0.0)
    h.set_scalar("dR0", 1.0 / state[0].shape[1])
    h.set_scalar("dR1", 1.0 / state[0].shape[0])
    while h.get_scalar("time") < T:
        h.proceed(1)
    out, t = [a.astype(np.float64) for a in h.state()], h.get_scalar("time")
    h.close()
    return out, t


def strip(n):
    return np.tile((np.arange(n) + 0.5) / n, (4, 1))


@pytest.mark.parametrize("precision", [64, 32])
def test_entropy_wave_converges(om_lib, precision):
    err = []
    for n in (128, 256, 512):
        X = strip(n)
        st, t = run_until(om_lib, RX.entropy_wave(X, 0.5, 0.0), 0.5, 1.4, precision)
        err.append(np.abs(st[0] - RX.entropy_wave(X, 0.5, t)[0]).mean())
    assert err[2] < 3e-4 and err[0] / err[1] > 3.0 and err[1] / err[2] > 3.0, err


def test_oblique_entropy_wave(om_lib):
    # the harness's Oblique case at 45 degrees: wave vector (1, 1), velocity
    # (0.5, 0.5), periodic on the unit square
    n = 128
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    st, t = run_until(om_lib, RX.entropy_wave(X, Y, 0.0, 0.5, 0.5, 1, 1), 0.5, 1.4, 64)
    err = np.abs(st[0] - RX.entropy_wave(X, Y, t, 0.5, 0.5, 1, 1)[0]).mean()
    assert err < 1e-2, err
    assert np.abs(st[1] - st[2]).max() < 1e-10      # the diagonal symmetry holds


@pytest.mark.parametrize("precision", [64, 32])
def test_sod_shock_tube(om_lib, precision):
    err = []
    for n in (256, 1024):
        X = strip(n)
        r, u, p = RX.sod_periodic(X, 1e-12, 1.4)
        st, t = run_until(om_lib, (r, u, np.zeros_like(r), p), 0.1, 1.4, precision)
        re, ue, pe = RX.sod_periodic(X, t, 1.4)
        err.append(np.abs(st[0] - re).mean())
        assert np.abs(st[3] - pe).mean() < 0.006 and np.abs(st[1] - ue).mean() < 0.012
    assert err[1] < 0.0025 and err[0] / err[1] > 2.5, err


def test_sound_wave(om_lib):
    g = 5.0 / 3.0
    X = strip(256)
    st, t = run_until(om_lib, RX.sound_wave(X, 0.0, g), 0.5, g, 64)
    assert np.abs(st[1] - RX.sound_wave(X, t, g)[1]).mean() < 0.005 * 1e-5
