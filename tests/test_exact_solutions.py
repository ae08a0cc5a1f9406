"""Known-answer tests of the Hydro scheme against exact solutions, the cases
of the reference's exact-solution harness (attic/GA.reproduce/
massive-test.cu:52-118) on periodic meshes: an entropy wave (converges at
second order away from the minmod clipping), a linear sound wave and Sod's
shock tube (first order at the discontinuities), run by the oracle."""
import numpy as np
import pytest

from oracle import riemann_exact as RX


def run_until(oracle, st, T, g, cfl=0.4):
    t = 0.0
    while t < T:
        st, t, _ = oracle.hydro_run(st, 1, cyclic=True, gamma=g, cfl=cfl, time=t)
    return st, t


def strip(n):
    x = (np.arange(n) + 0.5) / n
    return np.tile(x, (4, 1))


def test_riemann_solver_known_values():
    # Sod's star state (Toro, table 4.2 test 1): p* = 0.30313, u* = 0.92745
    p, u = RX.star_state(RX.SOD_L, RX.SOD_R, 1.4)
    assert abs(p - 0.30313) < 5e-5 and abs(u - 0.92745) < 5e-5
    r, uu, pp = RX.sample(RX.SOD_L, RX.SOD_R, 1.4, np.array([-10.0, 10.0, u]))
    assert r[0] == 1.0 and r[1] == 0.125 and abs(pp[2] - p) < 1e-12


def test_entropy_wave_converges(oracle):
    err = []
    for n in (64, 128):
        X = strip(n)
        st, t = run_until(oracle, RX.entropy_wave(X, 0.5, 0.0), 0.5, 1.4)
        err.append(np.abs(st[0] - RX.entropy_wave(X, 0.5, t)[0]).mean())
    assert err[1] < 4e-3 and err[0] / err[1] > 3.0, err


def test_sod_shock_tube(oracle):
    err = []
    for n in (128, 256):
        X = strip(n)
        r, u, p = RX.sod_periodic(X, 1e-12, 1.4)
        st, t = run_until(oracle, (r, u, np.zeros_like(r), p), 0.1, 1.4)
        re, ue, pe = RX.sod_periodic(X, t, 1.4)
        err.append(np.abs(st[0] - re).mean())
        assert np.abs(st[3] - pe).mean() < 0.012 and np.abs(st[1] - ue).mean() < 0.025
    assert err[1] < 0.008 and err[0] / err[1] > 1.5, err


def test_sound_wave(oracle):
    g = 5.0 / 3.0
    X = strip(128)
    st, t = run_until(oracle, RX.sound_wave(X, 0.0, g), 0.5, g)
    assert np.abs(st[1] - RX.sound_wave(X, t, g)[1]).mean() < 0.01 * 1e-5
