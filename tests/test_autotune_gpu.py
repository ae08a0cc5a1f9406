"""The autotuner measures candidates through the C ABI and returns a
configuration that runs (and is at least as fast as the defaults)."""
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
