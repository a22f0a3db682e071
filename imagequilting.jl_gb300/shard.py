"""Realization sharding of one iqsim call across devices or ranks.

Realizations are independent (src/iqsim.jl:163-312: each one restarts from an empty grid and
shares only the training image, the tile path and the data with the others). The library keys
the draw of realization r at tile t by the Philox counter (t, real0 + r), so a call with
`real0` simulates exactly the realizations [real0, real0 + nreal) of the whole call with the
same seed. Sharding is therefore a contiguous split of the realization range, one block per
rank, with no exchange on the data path; the only collective is the final gather of the
realizations to one host, done here with `torch.distributed.all_gather_object` (gloo or NCCL).
"""


def shard_range(nreal, rank, world):
    """(real0, count) of `rank`'s block of `nreal` realizations over `world` ranks.

    Blocks are contiguous and in rank order; the first nreal % world ranks hold one more."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %r outside a world of %r" % (rank, world))
    if nreal < 0:
        raise ValueError("negative realization count")
    base, extra = divmod(int(nreal), int(world))
    count = base + (1 if rank < extra else 0)
    real0 = rank * base + min(rank, extra)
    return real0, count


def iqsim_shard(iqsim, trainimg, tilesize, simsize=None, *, nreal=1, rank=0, world=1, **kwargs):
    """This rank's block of an iqsim call of `nreal` realizations: (real0, realizations).

    `iqsim` is the simulation function to shard (the library's api.iqsim); kwargs are passed
    through, so every rank must use the same seed (`rng`)."""
    real0, count = shard_range(nreal, rank, world)
    if count == 0:
        return real0, []
    out = iqsim(trainimg, tilesize, simsize, nreal=count, real0=real0, **kwargs)
    return real0, list(out)


def gather_realizations(dist, real0, local):
    """Every rank's (real0, realizations) gathered and ordered by real0: the whole call's list.

    `dist` is torch.distributed with an initialized process group, or None for one rank."""
    if dist is None:
        return list(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (int(real0), list(local)))
    out = []
    for _, reals in sorted(parts, key=lambda x: x[0]):
        out.extend(reals)
    return out
