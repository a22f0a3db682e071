"""Philox4x32-10 counter-based generator (oracle side).

TEST INFRASTRUCTURE ONLY: used by the CPU oracle, the tests and the CPU baseline of bench.py.

Published method: J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw, "Parallel random
numbers: as easy as 1, 2, 3", SC'11 (Philox4x32 with 10 rounds). The same generator is
implemented in CUDA/C++ in the library (csrc/iq_rng.h); both are checked against the
published known-answer vectors of the method.

The reference draws from Julia's `Random.default_rng()` / `Xoshiro` (src/iqsim.jl:62,243,
src/utils.jl:169,174,188). That stream cannot be reproduced without Julia, so the project
defines its own streams, keyed by a 64-bit seed:

  * the weighted draw of realization r at tile t   : counter (t, r, 1, 0)
  * the i-th integer drawn while building the path : counter (i, 0, 2, 0)

A counter yields four 32-bit words x0..x3; the 64-bit value used is (x1 << 32) | x0.
"""

M0 = 0xD2511F53
M1 = 0xCD9E8D57
W0 = 0x9E3779B9
W1 = 0xBB67AE85
MASK32 = 0xFFFFFFFF

PURPOSE_DRAW = 1
PURPOSE_PATH = 2


def philox4x32_10(ctr, key):
    """One Philox4x32-10 block: ctr is 4 uint32, key is 2 uint32; returns 4 uint32."""
    x0, x1, x2, x3 = (c & MASK32 for c in ctr)
    k0, k1 = key[0] & MASK32, key[1] & MASK32
    for rnd in range(10):
        if rnd:
            k0 = (k0 + W0) & MASK32
            k1 = (k1 + W1) & MASK32
        p0 = M0 * x0
        p1 = M1 * x2
        hi0, lo0 = p0 >> 32, p0 & MASK32
        hi1, lo1 = p1 >> 32, p1 & MASK32
        x0, x1, x2, x3 = (hi1 ^ x1 ^ k0), lo1, (hi0 ^ x3 ^ k1), lo0
    return x0, x1, x2, x3


def seed_key(seed):
    seed &= (1 << 64) - 1
    return (seed & MASK32, seed >> 32)


def u64(seed, c0, c1, c2, c3=0):
    """64-bit value of the block at counter (c0, c1, c2, c3) under `seed`."""
    x0, x1, _, _ = philox4x32_10((c0, c1, c2, c3), seed_key(seed))
    return (x1 << 32) | x0


def uniform01(seed, c0, c1, c2, c3=0):
    """Double in [0, 1): the top 53 bits of the 64-bit value times 2^-53 (exact)."""
    return (u64(seed, c0, c1, c2, c3) >> 11) * (1.0 / 9007199254740992.0)


def draw_uniform(seed, tile, real):
    """u in [0,1) for the weighted draw of realization `real` at tile `tile` (0-based)."""
    return uniform01(seed, tile, real, PURPOSE_DRAW)


class PathStream:
    """Sequential integer stream used by path generation (random/dilation/data-first)."""

    def __init__(self, seed):
        self.seed = seed
        self.i = 0

    def below(self, m):
        """Integer in [0, m): high 64 bits of the 128-bit product value*m."""
        v = u64(self.seed, self.i, 0, PURPOSE_PATH)
        self.i += 1
        return (v * m) >> 64

    def shuffle(self, a):
        """Fisher-Yates from the back: for i = n-1..1 swap a[i] with a[j], j = below(i+1)."""
        for i in range(len(a) - 1, 0, -1):
            j = self.below(i + 1)
            a[i], a[j] = a[j], a[i]
        return a

    def randperm(self, n):
        """Permutation of 0..n-1: shuffle of the identity."""
        return self.shuffle(list(range(n)))
