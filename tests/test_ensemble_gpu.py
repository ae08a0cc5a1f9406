"""Batched Hydro ensembles: uneven grids in one persistent launch per step,
each instance matching the single-grid path and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4
CFL = 0.4
SIZES = [(64, 32), (96, 128), (256, 64), (32, 32), (160, 96), (40, 72)]


def oracle_instance(oracle, st, steps, size, dtype):
    d0 = dtype(1.0) / dtype(size[0])
    d1 = dtype(1.0) / dtype(size[1])
    return oracle.hydro_run(st, steps, cyclic=True, gamma=GAMMA, cfl=CFL, dR=(d0, d1),
                            dtype=dtype)


@pytest.mark.parametrize("precision,variant", [(64, 0), (32, 2)])
def test_ensemble_bit_exact_per_instance(om_lib, oracle, precision, variant):
    dtype = np.float64 if precision == 64 else np.float32
    e = om_lib.Ensemble(SIZES, precision=precision, variant=variant, gamma=GAMMA)
    e.init_kh(100)
    init = [e.state(k) for k in range(len(SIZES))]
    # instance k holds the Kelvin-Helmholtz state of seed 100 + k
    for k, s in enumerate(SIZES):
        ref = oracle.hydro_init_kh(s[0], s[1], 100 + k, dtype=dtype)
        for a, b in zip(init[k], ref):
            np.testing.assert_allclose(a, b, rtol=0, atol=2e-16 if precision == 64 else 1e-7)
    for k, s in enumerate(SIZES):  # dR in the OM's Real type, as the oracle forms it
        e.set_scalar(k, "dR0", float(dtype(1.0) / dtype(s[0])))
        e.set_scalar(k, "dR1", float(dtype(1.0) / dtype(s[1])))
    e.step(7)
    assert e.last_launch_count() == 14
    dts = set()
    for k, s in enumerate(SIZES):
        ref, t, d = oracle_instance(oracle, init[k], 7, s, dtype)
        for a, b in zip(e.state(k), ref):
            assert np.array_equal(a, b), (k, s)
        # time accumulates the Real-typed dt of every step in FP64
        t64 = 0.0
        for x in d:
            t64 += float(x)
        assert abs(e.scalar(k, "time") - t64) <= 1e-14 * t64
        dts.add(e.scalar(k, "dt"))
    assert len(dts) > 1          # every instance has its own CFL dt
    e.close()


@pytest.mark.parametrize("tile", [(0, 0), (16, 0), (32, 0), (0, 32), (0, 16)])
def test_ensemble_fast_matches_single_grids(om_lib, tile):
    # (0, 0), (16, 0) and (32, 0): the persistent 32 x 32 kernel, paired as
    # two groups per CTA, paired, and one wall per thread, each item's box
    # prefetched (TMA inside an instance,
    # wrapped copies at its edges) while the block computes the item before;
    # (0, 32) and (0, 16): tile kernels; small instances: every block walks
    # several instances
    sizes = om_lib.ensemble_sizes(5, 42, lo=64, hi=320)
    e = om_lib.Ensemble(sizes, precision=32, gamma=GAMMA, tile_x=tile[0], tile_y=tile[1],
                        grid_limit=7)
    e.init_kh(7)
    e.step(3)       # graph captured
    e.step(3)       # replayed
    for k, s in enumerate(sizes):
        h = om_lib.Hydro(s, precision=32, gamma=GAMMA, tile_x=tile[0], tile_y=tile[1])
        h.init_kh(7 + k)
        h.set_scalar("cfl", CFL)
        h.proceed(6)
        for a, b in zip(e.state(k), h.state()):
            assert np.array_equal(a, b), (k, s)
        assert e.scalar(k, "time") == h.get_scalar("time")
        np.testing.assert_allclose(e.totals(k), h.totals(), rtol=1e-12)
        h.close()
    e.close()


def test_ensemble_two_groups_matches_single_grids(om_lib):
    # grid_limit 2: two CTAs of two groups for about 100 items, so the
    # two-group form of the persistent kernel runs; every instance equals its
    # single-grid production run (the same arithmetic) bit for bit
    sizes = om_lib.ensemble_sizes(4, 9, lo=128, hi=256)
    e = om_lib.Ensemble(sizes, precision=32, gamma=GAMMA, grid_limit=2)
    e.init_kh(3)
    e.step(4)
    for k, s in enumerate(sizes):
        h = om_lib.Hydro(s, precision=32, gamma=GAMMA)
        h.init_kh(3 + k)
        h.set_scalar("cfl", CFL)
        h.proceed(4)
        for a, b in zip(e.state(k), h.state()):
            assert np.array_equal(a, b), (k, s)
        assert e.scalar(k, "time") == h.get_scalar("time")
        h.close()
    e.close()


def test_ensemble_sizes_helper(om_lib):
    s = om_lib.ensemble_sizes(64, 1)
    assert len(s) == 64
    assert all(256 <= a <= 2048 and a % 32 == 0 and 256 <= b <= 2048 and b % 32 == 0 for a, b in s)
    assert s == om_lib.ensemble_sizes(64, 1)
    assert len(set(s)) > 32


def test_ensemble_rejects_bad_sizes(om_lib):
    with pytest.raises(om_lib.OMError):
        om_lib.Ensemble([(0, 5)])
