"""Generates the golden fixtures in this directory by running the
reference's own pre-generated code (oracle/_ref/, compiled from
examples-old/Life-exampled/dist/Life.cpp and
examples-old/Hydro-exampled/dist/Hydro.cpp of the reference tree).

Run from the repository root after `make -C oracle` with the reference
tree present:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def hashed_field(seed: int, shape, lo: float, hi: float) -> np.ndarray:
    """Uniform [lo, hi) float32 field from the oracle's counter hash."""
    return O.hash_uniform_f32(seed, shape, lo, hi)


def main() -> None:
    assert O.ref_available(), "build oracle/_ref first (make -C oracle with the reference tree)"
    # Life: the generated init (R-pentomino at the centre, open boundary), 1000 generations
    cells, pops = O.ref_life_run(None, 1000)
    np.savez_compressed(os.path.join(OUT, "life_ref_rpentomino.npz"), populations=pops,
                        cells=cells.astype(np.int8), cells_sha256=sha(cells))
    # Life: Bernoulli(0.3) seed 7 on the 128x128 interior, 200 generations
    init = O.life_bernoulli(128, 128, 7, 0.3, cyclic=False)
    cells, pops = O.ref_life_run(init, 200)
    np.savez_compressed(os.path.join(OUT, "life_ref_bernoulli.npz"), seed=7, p=0.3,
                        init=init.astype(np.int8), populations=pops,
                        cells=cells.astype(np.int8), cells_sha256=sha(cells))
    # Hydro: the generated init (jet, gamma 5/3, float, open), 2 steps, cfl 0.5
    st, times = O.ref_hydro_run(None, 2, cfl=0.5)
    rows = np.arange(0, 1030, 257)
    np.savez_compressed(os.path.join(OUT, "hydro_ref_jet.npz"), times=times, cfl=0.5,
                        sha256=np.array([sha(a) for a in st]),
                        sample_rows=rows, samples=np.stack([a[rows] for a in st]))
    # Hydro: hashed random supersonic state, 1 step, cfl 0.4
    shape = (1030, 1030)
    ini = (hashed_field(11, shape, 0.2, 3.0), hashed_field(12, shape, -4.0, 4.0),
           hashed_field(13, shape, -4.0, 4.0), hashed_field(14, shape, 0.05, 3.0))
    st, times = O.ref_hydro_run(ini, 1, cfl=0.4)
    np.savez_compressed(os.path.join(OUT, "hydro_ref_random.npz"), times=times, cfl=0.4,
                        seeds=np.array([11, 12, 13, 14]),
                        ranges=np.array([[0.2, 3.0], [-4.0, 4.0], [-4.0, 4.0], [0.05, 3.0]]),
                        input_sha256=np.array([sha(a) for a in ini]),
                        sha256=np.array([sha(a) for a in st]),
                        sample_rows=rows, samples=np.stack([a[rows] for a in st]))
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
