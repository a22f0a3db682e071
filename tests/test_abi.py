"""The C ABI without a GPU: the library loads, exports every declared entry point, and its
host-side parts (path generation, argument checks) match the oracle."""
import os
import re

import numpy as np
import pytest

from oracle import iqsim_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(iq_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(iq):
    lib = iq.load()
    declared = _declared()
    assert {"iq_simulate", "iq_fastdistance", "iq_pick", "iq_graphcut"} <= declared
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert lib.iq_version() >= 100


def test_binding_covers_header(iq):
    from importlib import import_module
    lib_mod = import_module("iqgpu._lib")
    assert _declared() <= set(lib_mod.SIGNATURES)


@pytest.mark.parametrize("kind", ["raster", "random", "dilation"])
@pytest.mark.parametrize("extent", [(10, 10, 10), (7, 5), (12,), (22, 22, 11)])
def test_genpath_matches_oracle(iq, kind, extent):
    for seed in (0, 123, 2 ** 63 + 5):
        assert iq.genpath(seed, extent, kind) == O.genpath(seed, extent, kind, [])


def test_genpath_data_first(iq):
    for seed in (1, 2, 3):
        di = [0, 999, 500, 17]
        g = iq.genpath(seed, (10, 10, 10), "raster", di)
        assert g == O.genpath(seed, (10, 10, 10), "raster", di)
        assert sorted(g[:4]) == sorted(di) and sorted(g) == list(range(1000))


def test_assertions_match_reference(iq):
    TI = np.ones((20, 20))
    cases = [((TI, (30, 10)), {}, "invalid tile size"),
             ((TI, (10, 10), (5, 5)), {}, "invalid grid size"),
             ((TI, (10, 10)), {"overlap": (0, 0.5)}, "overlaps must be in range"),
             ((TI, (10, 10)), {"tol": 1.5}, "tolerance must be in range"),
             ((TI, (10, 10)), {"path": "spiral"}, "invalid simulation path"),
             ((TI, (10, 10)), {"nreal": 0}, "invalid number of realizations"),
             ((TI, (10, 10)), {"hard": {(20, 0): 1.0}}, "hard data coordinates outside"),
             ((TI, (10, 10)), {"soft": [(np.ones((5, 5)), TI)]}, "soft data size"),
             ((TI, (10, 10)), {"soft": [(TI, np.ones((5, 5)))]}, "auxiliary TI")]
    for args, kw, msg in cases:
        with pytest.raises(AssertionError, match=msg):
            iq.iqsim(*args, **kw)
        with pytest.raises(AssertionError, match=msg):
            O.iqsim(*args, **kw)
