"""The autotuner measures candidates through the C ABI and returns a
configuration that runs, and that is at least as fast as the default one
measured the same way (the default configuration is always a candidate; 5 %
is left for the run-to-run spread of two separate measurements)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_life(om_lib, oracle):
    cfg, rate = om_lib.autotune("life", (2048, 1024))
    assert rate > 0
    life = om_lib.Life((2048, 1024), config=cfg)
    init = oracle.life_bernoulli(2048, 1024, 3, 0.3)
    life.write("cell", init)
    life.proceed(40)
    ref, pops = oracle.life_run(init, 40, cyclic=True)
    assert np.array_equal(life.read("cell"), ref)
    life.close()
    cfg2, rate2 = om_lib.autotune("life", (2048, 1024))   # cached
    assert rate2 == rate and cfg2.depth == cfg.depth and cfg2.tile_y == cfg.tile_y


def test_autotune_life_unpackable_size(om_lib):
    cfg, rate = om_lib.autotune("life", (100, 60))
    assert rate > 0


def test_autotune_hydro_and_ensemble(om_lib):
    cfg, rate = om_lib.autotune("hydro", (512, 384), precision=32, gamma=1.4)
    assert rate > 0 and cfg.precision == 32
    h = om_lib.Hydro((512, 384), config=cfg)
    h.init_kh(1)
    h.proceed(3)
    assert np.isfinite(h.totals()).all()
    h.close()
    sizes = om_lib.ensemble_sizes(6, 3, lo=64, hi=256)
    ecfg, erate = om_lib.autotune_ensemble(sizes, precision=32, gamma=1.4)
    assert erate > 0
    e = om_lib.Ensemble(sizes, config=ecfg)
    e.init_kh(1)
    e.step(2)
    e.close()


NOISE = 0.95


def test_autotune_beats_defaults(om_lib):
    pg = om_lib
    cfg, _ = pg.autotune("life", (2048, 1024))
    assert pg.measure_rate("life", (2048, 1024), cfg, 96) >= \
        NOISE * pg.measure_rate("life", (2048, 1024), pg.default_config(), 96)
    base = pg.default_config(precision=32, gamma=1.4)
    cfg, _ = pg.autotune("hydro", (1024, 768), precision=32, gamma=1.4)
    assert pg.measure_rate("hydro", (1024, 768), cfg, 8) >= \
        NOISE * pg.measure_rate("hydro", (1024, 768), base, 8)
    sizes = pg.ensemble_sizes(12, 5, lo=128, hi=768)
    ecfg, _ = pg.autotune_ensemble(sizes, precision=32, gamma=1.4)
    assert pg.ensemble_rate(sizes, ecfg) >= NOISE * pg.ensemble_rate(sizes, base)
