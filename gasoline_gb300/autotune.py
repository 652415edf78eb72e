"""Launch-shape autotuner of the gravity path.

The walk's bucket size (the reference's nBucket, 8/16/32 particles handled
by one warp), the resident walk blocks per SM, the tree builder's task
size (the largest node one CTA builds whole) and the walk mode are chosen
by timing real gravity evaluations of the caller's own particles on the
device:

    best, table = tune_gravity(ctx, grav_params(...))

The walk modes, as (walkGroup, walkLists) pairs: walk groups of 128
particles (0, 0); the two-pass walk, a list pass and then the evaluation
pass (-1, 1); one fused pass per bucket (-1, -1).

Only nBucket changes the tree and the interaction lists (it is a physics
parameter of the reference: a different bucket size is a different tree).
The block count, the task size and the two-pass walk are result-neutral,
which the tests check bit for bit; groups change only the order in which
each particle's terms are summed.  Groups pay off on clustered systems
(fewer opening tests per bucket), the two-pass walk where the tree walk's
latency dominates, which is why the mode is tuned.  The context is left
with the best knobs set.

The bucket size runs to 32 (TSPH_MAX_BUCKET): one warp walks one bucket
with a lane per (particle, entry slot), 32/nBucket slots per particle, so
the warp is the bucket's unit of work and "warps per bucket" is one by
construction.  The list-tile lengths (128 particle-particle entries, 64
cells) are compile-time constants that set the walk's shared memory and
so its resident blocks; a 48-cell variant with six blocks per SM measured
slower on both a periodic box and a Plummer sphere, and the walk-block
count is the knob that trades the same resources at run time.
"""
import itertools

from . import GravParams


def _time_grav(ctx, gp, reps):
    ctx.grav_all(gp)                       # warm: allocations, constants
    best = float("inf")
    for _ in range(reps):
        ctx.grav_all(gp)
        best = min(best, ctx.timings()["total"])
    return best


def tune_gravity(ctx, gp, nbuckets=(8, 16, 32), walk_blocks=(4, 5), task_sizes=(0, 65536),
                 walk_modes=((0, 0), (-1, 1), (-1, -1)), reps=2):
    """Time every (nBucket, walkBlocksPerSM, taskSize, walk mode) on the
    context's current particles; returns (best, table) where best holds the
    winning knobs and its time in ms, and table every measurement."""
    table = []
    for nb, wb, ts, (wg, wl) in itertools.product(nbuckets, walk_blocks, task_sizes, walk_modes):
        ctx.set_tuning(taskSize=ts, walkBlocksPerSM=wb, walkGroup=wg, walkLists=wl)
        g = GravParams.from_buffer_copy(gp)
        g.nBucket = nb
        ms = _time_grav(ctx, g, reps)
        table.append({"nBucket": nb, "walkBlocksPerSM": wb, "taskSize": ts, "walkGroup": wg,
                      "walkLists": wl, "ms": ms})
    best = min(table, key=lambda r: r["ms"])
    ctx.set_tuning(taskSize=best["taskSize"], walkBlocksPerSM=best["walkBlocksPerSM"],
                   walkGroup=best["walkGroup"], walkLists=best["walkLists"])
    return dict(best), table
