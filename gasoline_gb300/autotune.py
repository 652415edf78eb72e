"""Launch-shape autotuner of the gravity path.

The walk's bucket size (the reference's nBucket, 8/16/32 particles handled
by one warp), the resident walk blocks per SM and the tree builder's task
size (the largest node one CTA builds whole) are chosen by timing real
gravity evaluations of the caller's own particles on the device:

    best, table = tune_gravity(ctx, grav_params(...))

Only nBucket changes results (it is a physics parameter of the reference:
a different bucket size is a different tree); the other two knobs are
result-neutral, which the tests check bit for bit.  The context is left
with the best knobs set.
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


def tune_gravity(ctx, gp, nbuckets=(8, 16, 32), walk_blocks=(2, 4, 6), task_sizes=(0, 65536),
                 reps=2):
    """Time every (nBucket, walkBlocksPerSM, taskSize) on the context's
    current particles; returns (best, table) where best holds the winning
    knobs and its time in ms, and table every measurement."""
    table = []
    for nb, wb, ts in itertools.product(nbuckets, walk_blocks, task_sizes):
        ctx.set_tuning(taskSize=ts, walkBlocksPerSM=wb)
        g = GravParams.from_buffer_copy(gp)
        g.nBucket = nb
        ms = _time_grav(ctx, g, reps)
        table.append({"nBucket": nb, "walkBlocksPerSM": wb, "taskSize": ts, "ms": ms})
    best = min(table, key=lambda r: r["ms"])
    ctx.set_tuning(taskSize=best["taskSize"], walkBlocksPerSM=best["walkBlocksPerSM"])
    return dict(best), table
