"""The execution forms of the level-scheduled sweeps, forced through the
library's tuning knobs so every form is checked on small systems:

* small   -- one CTA, vector in global memory
* cta     -- one CTA, vector in shared memory (the default for small levels)
* cluster -- a 16-CTA cluster, vector in distributed shared memory
* cluster_global -- a 16-CTA cluster, vector in global memory (L2)
* cluster_pre -- the default split: DIC/DILU sweeps in a 16-CTA cluster's
             shared memory, Gauss-Seidel sweeps on the persistent grid
* grid    -- the persistent grid, wavefront: each 32-slot group waits for the
             groups it reads (vector in global memory)
* levels  -- the persistent grid with whole-level counters
* tile    -- the tile form (the default for vectors larger than one CTA's
             shared memory), here with 2 KB of shared memory per CTA so that
             small meshes run as many tiles over many bands, each publishing
             its progress every level
* tile_pub3 -- the same with 4 KB tiles publishing every third level
"""
import contextlib

from openfoam_dev_gb300 import ldu

FORMS = {
    "small": {ldu.TUNE_SMALL_SWEEP: 1 << 30, ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_TILE: 0},
    "cta": {},
    "cluster": {ldu.TUNE_CLUSTER_SIZE: 16, ldu.TUNE_SMEM_BYTES: 8192, ldu.TUNE_TILE: 0},
    "cluster_global": {ldu.TUNE_CLUSTER_SIZE: 16, ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_CLUSTER_GLOBAL: 1 << 30,
                       ldu.TUNE_TILE: 0},
    # DIC/DILU sweeps on a 16-CTA cluster, Gauss-Seidel on the grid
    "cluster_pre": {ldu.TUNE_SMEM_BYTES: 8192, ldu.TUNE_CLUSTER_PRE: 16, ldu.TUNE_TILE: 0},
    "grid": {ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_GRID_WAVE: 1, ldu.TUNE_TILE: 0},
    "levels": {ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_GRID_WAVE: 0, ldu.TUNE_TILE: 0},
    "tile": {ldu.TUNE_SMEM_BYTES: 2048, ldu.TUNE_TILE: 1, ldu.TUNE_TILE_PUBLISH: 1},
    "tile_pub3": {ldu.TUNE_SMEM_BYTES: 4096, ldu.TUNE_TILE: 1, ldu.TUNE_TILE_PUBLISH: 3},
}
KNOBS = (ldu.TUNE_SMALL_SWEEP, ldu.TUNE_CLUSTER_GLOBAL, ldu.TUNE_CLUSTER_SIZE, ldu.TUNE_SMEM_BYTES,
         ldu.TUNE_GRID_WAVE, ldu.TUNE_CLUSTER_PRE, ldu.TUNE_TILE, ldu.TUNE_TILE_PUBLISH)


@contextlib.contextmanager
def sweep_form(name):
    old = {k: ldu.tune_get(k) for k in KNOBS}
    try:
        for k, v in FORMS[name].items():
            ldu.tune_set(k, v)
        yield name
    finally:
        for k in KNOBS:
            ldu.tune_set(k, old[k])
