"""Group-tile autotuner for the FP32 sweep (host face of umt103_autotune).

The sweep assigns one team of `lanes_per_zone` lanes to each (direction,
zone) pair and gives every lane `groups_per_lane` consecutive groups
(lanes_per_zone * groups_per_lane = G).  More groups per lane amortise the
zone program's decode and widen every load, but raise register use and lower
the number of resident teams; the best point depends on G, the direction
count and the mesh, so the library times every legal tile on the loaded
problem, keeps the fastest and caches it per problem shape
(umt_gb300/csrc/capi.cu, umt103_autotune / umt103_autotune_contexts).
"""
from __future__ import annotations

from . import capi


def autotune(lib: capi.Library, reps: int = 2, verbose: bool = False):
    """Tune the current context.  Returns (best_tile, {tile: ms})."""
    best, times = lib.autotune(reps)
    if verbose:
        for (gt, gpl), ms in sorted(times.items()):
            print(f"tile lanes_per_zone={gt:2d} groups_per_lane={gpl}: {ms:.3f} ms")
    return best, times


def autotune_batch(lib: capi.Library, ids, reps: int = 2):
    """Tune each distinct problem shape of a batch of contexts once; every
    context then sweeps with its shape's tile (umt103_batch_sweep applies
    them)."""
    lib.autotune_contexts(ids, reps)
