"""Writes the golden fixtures of this directory (run from the repository root:
`python tests/golden/make_golden.py`).

The reference (Julia) cannot run here, so the fixtures are:
  * philox_kat.json: the published known-answer vectors of Philox4x32-10 (Random123,
    Salmon et al., SC'11), the generator both the oracle and the GPU path use;
  * the oracle's outputs on three small seeded cases, the same inputs the GPU parity tests
    draw: an integer-TI iqsim with hard and soft data (every distance is an exact integer, so
    the GPU realizations must equal these bit for bit), a continuous graph cut and integer
    distance maps with a disabled window. tests/test_oracle.py checks that the oracle still
    reproduces them; tests/test_gpu_parity.py checks the CUDA path against them.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import iqsim_oracle as O  # noqa: E402

PHILOX_KAT = [  # (counter, key, output), hexadecimal words
    (["00000000"] * 4, ["00000000"] * 2, ["6627e8d5", "e169c58d", "bc57ac4c", "9b00dbd8"]),
    (["ffffffff"] * 4, ["ffffffff"] * 2, ["408f276d", "41c83b0e", "a20bc7c6", "6d5451fd"]),
    (["243f6a88", "85a308d3", "13198a2e", "03707344"], ["a4093822", "299f31d0"],
     ["d16cfe09", "94fdcceb", "5001e420", "24126ea1"]),
]


def iqsim_case():
    rng = np.random.default_rng(34)
    ti = rng.integers(0, 4, (30, 28, 14)).astype(np.float32)
    simsize = (40, 36, 14)
    hard = {(int(rng.integers(0, 40)), int(rng.integers(0, 36)), int(rng.integers(0, 14))):
            float(rng.integers(0, 4)) for _ in range(10)}
    aux = rng.integers(0, 5, simsize).astype(np.float32)
    auxti = rng.integers(0, 5, ti.shape).astype(np.float32)
    reals = O.iqsim(ti, (9, 8, 6), simsize, overlap=(0.25, 0.25, 0.25), path="raster", nreal=3,
                    seed=99, hard=hard, soft=[(aux, auxti)])
    return dict(ti=ti, tilesize=np.array((9, 8, 6)), simsize=np.array(simsize),
                overlap=np.array((0.25, 0.25, 0.25)), seed=np.array(99), nreal=np.array(3),
                hard_coords=np.array(list(hard.keys()), np.int64),
                hard_values=np.array(list(hard.values()), np.float64),
                aux=aux, auxti=auxti, reals=np.stack([np.asarray(r, np.float32) for r in reals]))


def graphcut_case():
    rng = np.random.default_rng(15)
    A = np.exp(rng.normal(size=(6, 24, 12))).astype(np.float32)
    B = np.exp(rng.normal(size=(6, 24, 12))).astype(np.float32)
    return dict(A=A, B=B, dim=np.array(0), mask=O.graphcut(A, B, 0))


def fastdistance_case():
    rng = np.random.default_rng(32)
    ti = rng.integers(0, 6, (40, 30, 8)).astype(np.float32)
    ti[3, 4, 2] = np.nan
    tm = rng.integers(-2, 5, (300, 9, 7, 3)).astype(np.float32)[:4]
    w = np.ones((9, 7, 3), bool)
    w[tuple(slice(max(1, t // 4), t) for t in (9, 7, 3))] = False
    dis = O.finddisabled(ti, (9, 7, 3))
    maps = []
    for t in tm:
        ref = O.fastdistance(np.nan_to_num(ti), t, w, "direct")
        ref[dis] = np.inf
        maps.append(ref.astype(np.float32))
    return dict(ti=ti, tmpl=tm, weights=w, maps=np.stack(maps))


def main():
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump([{"counter": c, "key": k, "output": o} for c, k, o in PHILOX_KAT], f, indent=1)
    for name, fn in (("iqsim_int3d", iqsim_case), ("graphcut_cont3d", graphcut_case),
                     ("fastdistance_int3d", fastdistance_case)):
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **fn())


if __name__ == "__main__":
    main()
