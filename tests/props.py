"""Size-independent properties of an iqsim result, for sizes the oracle cannot check in full.

Every voxel of a realization was pasted from some training-image window (the first tile of a
region is pasted whole, later tiles keep the existing voxels inside their cut), and the hard
data are written last (src/iqsim.jl:252-307). So every value is a TI value or a hard datum,
every hard datum sits at its coordinate, and the seeded draws make two identical calls agree.
"""
import numpy as np


def check_realizations(reals, ti, hard):
    allowed = np.unique(np.concatenate([np.asarray(ti, np.float32).ravel(),
                                        np.array(list(hard.values()), np.float32)]))
    for r in reals:
        r = np.asarray(r, np.float32)
        assert np.all(np.isin(r, allowed)), "a voxel is neither a TI value nor a hard datum"
        for c, v in hard.items():
            assert r[c] == np.float32(v), ("hard datum not honoured", c)
    if len(reals) > 1:
        assert not all(np.array_equal(reals[0], r) for r in reals[1:]), "realizations identical"
