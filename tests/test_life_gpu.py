"""Life on the GPU through the C ABI, bit-exact against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the profile name of the kernel the automatic choice takes on large grids
WANT_WS = "life_ws_tma_kernel"


def run_gpu(pg, size, init, steps, **cfg):
    life = pg.Life(size, **cfg)
    life.write("cell", init)
    life.proceed(steps)
    cells = life.read("cell")
    pops = life.population_history(steps)
    out = (cells, pops, life.population, life.generation, life.last_launch_count())
    life.close()
    return out


def test_life_128_bernoulli_1000(om_lib, oracle):
    # the 128x128 cyclic, Bernoulli(0.3), 1000-generation workload
    pg = om_lib
    life = pg.Life((128, 128))
    life.fill_random(1, 0.3)
    init = life.read("cell")
    assert np.array_equal(init, oracle.life_bernoulli(128, 128, 1, 0.3))
    life.proceed(1000)
    ref_cells, ref_pops = oracle.life_run(init, 1000, cyclic=True)
    assert np.array_equal(life.read("cell"), ref_cells)
    assert np.array_equal(life.population_history(1000), ref_pops)
    assert life.population == ref_pops[-1]
    assert life.generation == 1000
    life.close()


@pytest.mark.parametrize("size", [(37, 29), (1, 7), (5, 1), (80, 48), (33, 64), (130, 17),
                                  (96, 5000), (160, 3)])
def test_life_general_path_odd_sizes(om_lib, oracle, size):
    init = oracle.life_bernoulli(size[0], size[1], 5, 0.35)
    cells, pops, pop, gen, _ = run_gpu(om_lib, size, init, 25)
    rc, rp = oracle.life_run(init, 25, cyclic=True)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)
    assert pop == rp[-1] and gen == 25


@pytest.mark.parametrize("size", [(128, 128), (96, 40), (200, 130)])
def test_life_open_boundary(om_lib, oracle, size):
    init = oracle.life_bernoulli(size[0], size[1], 9, 0.3, cyclic=False)
    init[0, :] = 1   # margins written by the host are zeroed by the first step
    cells, pops, pop, gen, _ = run_gpu(om_lib, size, init, 40, boundary=1)
    rc, rp = oracle.life_run(init, 40, cyclic=False)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)


@pytest.mark.parametrize("io", [0, 1])
@pytest.mark.parametrize("depth,tw,th", [(16, 0, 0), (1, 4, 8), (7, 3, 5), (32, 8, 64),
                                         (32, 64, 128), (25, 16, 100), (32, 16, 128),
                                         (32, 30, 64), (9, 30, 17), (0, 0, 0),
                                         (32, 0, 64), (32, 0, 192), (32, 0, 300), (32, 0, 400),
                                         (5, 0, 0), (31, 0, 100)])
def test_life_temporal_blocking_tiles(om_lib, oracle, depth, tw, th, io):
    size = (1024, 640)
    init = oracle.life_bernoulli(size[0], size[1], 11, 0.3)
    cells, pops, pop, gen, launches = run_gpu(om_lib, size, init, 70, depth=depth,
                                              tile_x=tw, tile_y=th, life_io=io)
    rc, rp = oracle.life_run(init, 70, cyclic=True)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)
    assert launches >= 2


@pytest.mark.parametrize("kernel", list(range(1, 17)))
@pytest.mark.parametrize("depth", [32, 13])
def test_life_warp_specialised(om_lib, oracle, kernel, depth):
    size = (2048, 1500)   # several tiles per CTA on a small grid, partial tiles
    init = oracle.life_bernoulli(size[0], size[1], 17, 0.3)
    # four CTAs: each walks several tiles, so the producer, consumer and
    # store warps all run their pipelined stages
    cells, pops, pop, gen, launches = run_gpu(om_lib, size, init, 45, depth=depth,
                                              life_kernel=kernel, grid_limit=4)
    rc, rp = oracle.life_run(init, 45, cyclic=True)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)


@pytest.mark.parametrize("size", [(128, 128), (1024, 1), (512, 2), (256, 4), (64, 16), (32, 32),
                                  (1024, 32), (512, 64)])
def test_life_small_grid_in_registers(om_lib, oracle, size):
    # grids of at most 1024 packed words with rows of 1, 2, 4, 8, 16 or 32
    # words run in one CTA, one word per thread (life_smallreg_kernel)
    pg = om_lib
    init = oracle.life_bernoulli(size[0], size[1], 23, 0.35)
    life = pg.Life(size)
    life.write("cell", init)
    life.profile(True)
    life.proceed(300)
    assert life.profile_query("life_smallreg_kernel")[0] == 1
    rc, rp = oracle.life_run(init, 300, cyclic=True)
    assert np.array_equal(life.read("cell"), rc)
    assert np.array_equal(life.population_history(300), rp)
    life.close()


def test_life_automatic_kernel_choice(om_lib):
    # with no kernel or tile shape given, a grid of at least 1.5 warp-
    # specialised tiles per SM runs on that kernel (WANT_WS: its TMA variant
    # where rows hold at least 1024 cells) and a smaller one on the
    # register-resident blocks; both equal the register-resident blocks
    # forced by a tile height (pinned to the oracle above) bit for bit
    pg = om_lib
    for size, want in [((8192, 8192), WANT_WS), ((2048, 1024), "life_reg_kernel")]:
        init = None
        out = []
        for cfg in ({}, {"tile_y": 320}):
            life = pg.Life(size, **cfg)
            if init is None:
                life.fill_random(5, 0.3)
                init = life.read("cell")
            else:
                life.write("cell", init)
            life.profile(True)
            life.proceed(70)
            if not cfg:
                assert life.profile_query(want)[0] >= 2
            out.append((life.read("cell"), life.population_history(70)))
            life.close()
        assert np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[0][1], out[1][1])


def test_life_nonbinary_first_step(om_lib, oracle):
    init = oracle.life_bernoulli(256, 96, 2, 0.3)
    init[10, 10] = 3
    init[20, 30] = -1
    init[50, 200] = 7
    cells, pops, *_ = run_gpu(om_lib, (256, 96), init, 30)
    rc, rp = oracle.life_run(init, 30, cyclic=True)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)


def test_life_host_write_checks_cell_values(om_lib, oracle):
    # a host write of 0/1 cells keeps every generation on the packed kernels;
    # any other value costs exactly one generation of the general kernel
    init = oracle.life_bernoulli(256, 96, 3, 0.3)
    rc, rp = oracle.life_run(init, 30, cyclic=True)
    cells, pops, _, _, packed_launches = run_gpu(om_lib, (256, 96), init, 30)
    assert np.array_equal(cells, rc) and np.array_equal(pops, rp)
    init[5, 7] = 2
    rc, rp = oracle.life_run(init, 30, cyclic=True)
    cells, pops, _, _, launches = run_gpu(om_lib, (256, 96), init, 30)
    assert np.array_equal(cells, rc) and np.array_equal(pops, rp)
    assert launches == packed_launches + 1


def test_life_host_mirror_and_graph_replay(om_lib, oracle):
    pg = om_lib
    life = pg.Life((512, 256))
    life.init()
    assert life.population == 0 and life.generation == 0
    m = life.array("cell")          # writable mirror: marks the host newer
    glider = ((1, 0), (2, 1), (0, 2), (1, 2), (2, 2))
    for x, y in glider:
        m[y + 100, x + 100] = 1
    ref = m.copy()
    for rep in range(3):            # graph captured once, replayed twice
        life.proceed(8)
        ref, rp = oracle.life_run(ref, 8, cyclic=True)
        assert np.array_equal(life.read("cell"), ref)
        assert life.population == 5
    assert life.generation == 24
    # const reads do not disturb the device copy
    life.proceed(1)
    ref, _ = oracle.life_run(ref, 1, cyclic=True)
    assert np.array_equal(life.read("cell"), ref)
    life.close()


def test_life_full_size_properties(om_lib, oracle):
    # 16384x16384, Bernoulli(0.3): 20 generations against the oracle, and
    # the temporally blocked path against the general integer path over 100
    pg = om_lib
    n = 16384
    life = pg.Life((n, n))
    life.fill_random(1, 0.3)
    init = life.read("cell")
    life.proceed(20)
    rc, rp = oracle.life_run(init, 20, cyclic=True)
    assert np.array_equal(life.population_history(20), rp)
    assert np.array_equal(life.read("cell"), rc)
    del rc
    life.proceed(80)
    tb_pops = life.population_history(80)
    tb_cells = life.read("cell")
    life.close()
    # the same 100 generations on the integer one-cell-per-thread kernel
    gen = pg.Life((n, n), variant=1)
    gen.write("cell", init)
    gen.proceed(100)
    assert gen.last_launch_count() >= 100
    assert np.array_equal(gen.population_history(100)[20:], tb_pops)
    assert np.array_equal(gen.read("cell"), tb_cells)
    gen.close()


@pytest.mark.parametrize("kernel", [5, 8, 11, 14, 15, 16])
@pytest.mark.parametrize("size", [(1024, 700), (3072, 333), (1984, 1111)])
def test_life_tma_rows_edge_tiles(om_lib, oracle, kernel, size):
    """The TMA variants on grids whose first and last tile columns wrap (the
    wrapped halo word comes in as a one-word box), whose last tile column is
    narrow (1984 = 62 words: 30 + 30 + 2) and whose rows are not a multiple
    of the tile height; three CTAs, so each walks several tiles."""
    init = oracle.life_bernoulli(size[0], size[1], 29, 0.3)
    cells, pops, pop, gen, launches = run_gpu(om_lib, size, init, 70, life_kernel=kernel,
                                              grid_limit=3)
    rc, rp = oracle.life_run(init, 70, cyclic=True)
    assert np.array_equal(cells, rc)
    assert np.array_equal(pops, rp)
