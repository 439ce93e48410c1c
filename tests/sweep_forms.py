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
* flow    -- the dataflow form (each slot waits for exactly the values it
             reads, the value being its own ready flag), here for every mesh
             larger than 256 FP64 cells and every schedule (by default it
             runs the schedules of at most 8 entries per slot)
* level_launch -- one ordinary launch per DAG level (schedules of at most
             128 levels; the default for the multicolour schedules)
* auto    -- the default choice on the same meshes: a launch per level for
             schedules of at most 96 levels (unless the vector fits one CTA
             and the levels are narrow), else the dataflow form for
             schedules of at most 8 entries per slot, the level counters for
             the others
"""
import contextlib

from openfoam_dev_gb300 import ldu

_NL = {ldu.TUNE_LEVEL_LAUNCH: 0}  # keeps the forced form from giving way to a launch per level
FORMS = {
    "small": {ldu.TUNE_SMALL_SWEEP: 1 << 30, ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_FLOW: 0, **_NL},
    "cta": {**_NL},
    "cluster": {ldu.TUNE_CLUSTER_SIZE: 16, ldu.TUNE_SMEM_BYTES: 8192, ldu.TUNE_FLOW: 0, **_NL},
    "cluster_global": {ldu.TUNE_CLUSTER_SIZE: 16, ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_CLUSTER_GLOBAL: 1 << 30,
                       ldu.TUNE_FLOW: 0, **_NL},
    # DIC/DILU sweeps on a 16-CTA cluster, Gauss-Seidel on the grid
    "cluster_pre": {ldu.TUNE_SMEM_BYTES: 8192, ldu.TUNE_CLUSTER_PRE: 16, ldu.TUNE_FLOW: 0, **_NL},
    "grid": {ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_GRID_WAVE: 1, ldu.TUNE_FLOW: 0, **_NL},
    "levels": {ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_GRID_WAVE: 0, ldu.TUNE_FLOW: 0, **_NL},
    "flow": {ldu.TUNE_SMEM_BYTES: 2048, ldu.TUNE_FLOW: 1, **_NL},
    "level_launch": {ldu.TUNE_SMEM_BYTES: 0, ldu.TUNE_LEVEL_LAUNCH: 128},
    "auto": {ldu.TUNE_SMEM_BYTES: 2048, ldu.TUNE_FLOW: 2},
}
KNOBS = (ldu.TUNE_SMALL_SWEEP, ldu.TUNE_CLUSTER_GLOBAL, ldu.TUNE_CLUSTER_SIZE, ldu.TUNE_SMEM_BYTES,
         ldu.TUNE_GRID_WAVE, ldu.TUNE_CLUSTER_PRE, ldu.TUNE_FLOW, ldu.TUNE_LEVEL_LAUNCH)


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
