"""Group-tile autotuner for the FP32 sweep.

The production kernel assigns one team of `lanes_per_zone` lanes to each
(direction, zone) pair and gives every lane `groups_per_lane` consecutive
groups (lanes_per_zone * groups_per_lane = G).  More groups per lane amortise
the zone's structure decode and widen every load to 64 or 128 bits, but raise
register use (about 96 / 124 / 200 registers per thread for 1 / 2 / 4 groups
per lane) and lower the number of resident teams.  The best point depends on G,
the direction count and the mesh, so it is measured: every legal tile is timed
on the problem already loaded in the library, and the fastest is kept.
"""
from __future__ import annotations

from . import capi

LANES = (1, 2, 4, 8, 16, 32)
GROUPS_PER_LANE = (1, 2, 4)


def candidates(G: int):
    return [(G // gpl, gpl) for gpl in GROUPS_PER_LANE if G % gpl == 0 and (G // gpl) in LANES]


def autotune(lib: capi.Library, reps: int = 3, verbose: bool = False):
    """Time every legal tile with device-resident sweeps; keep the fastest.

    Returns (best_tile, {tile: stage-kernel ms})."""
    results = {}
    for tile in candidates(lib.G):
        lib.set_group_tile(*tile)
        lib.sweep_resident(False, capi.UMT_FP32)          # capture + warm
        best = float("inf")
        for _ in range(reps):
            lib.sweep_resident(False, capi.UMT_FP32)
            best = min(best, lib.timing()[1])
        results[tile] = best
        if verbose:
            print(f"tile lanes_per_zone={tile[0]:2d} groups_per_lane={tile[1]}: {best:.3f} ms")
    if not results:
        return None, results
    best_tile = min(results, key=results.get)
    lib.set_group_tile(*best_tile)
    return best_tile, results
