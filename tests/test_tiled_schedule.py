"""The tiled form of the sweep schedules, checked on the CPU (no GPU).

The tiled form cuts the levels of a sweep's dependency DAG into bands and
each band, in (sweep, cell) order, into tiles; a tile runs on one CTA with
the values it produces in shared memory, and waits for the published
progress of the tiles it reads from.  cfx_sched_tiled_check builds it and
checks it against the sequential sweep of the reference: every (sweep, cell)
once, every cell's terms in the reference's order, every value read either
produced earlier in the same tile (and still the version the sweep reads)
or waited for, and every wait on a lower tile, so that with all CTAs
resident no wait can deadlock.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from openfoam_dev_gb300 import cases, ldu


def _meshes():
    out = {"cube16": cases.pcg_cube(16, seed=1), "jcube14": cases.gamg_cube(14, jitter=0.2, seed=5),
           "cd12_cm": cases.bicgstab_cube(12, seed=2)}
    s = out["jcube14"]
    agg = orc.Agglomeration(s, n_coarsest=10)
    for i in range(min(agg.n_levels, 3)):
        _, _, _, nc, ncf, cl, cu = agg.level(i)
        out[f"jcube14_level{i + 1}"] = {"diag": np.zeros(nc), "l": cl, "u": cu}
    return out


MESHES = _meshes()
KINDS = [("forward", 1), ("backward", 1), ("GaussSeidel", 1), ("GaussSeidel", 2), ("GaussSeidel", 4),
         ("symGaussSeidelBackward", 1)]


@pytest.mark.parametrize("kind,sweeps", KINDS)
@pytest.mark.parametrize("mesh", sorted(MESHES))
@pytest.mark.parametrize("tile,ctas,pub", [(64, 152, 1), (256, 8, 2), (1000, 3, 4), (4096, 152, 2)])
def test_tiled_schedule_is_a_valid_sweep(mesh, kind, sweeps, tile, ctas, pub):
    s = MESHES[mesh]
    st = ldu.sched_tiled_check(s["diag"].size, s["l"], s["u"], kind, sweeps, tile, ctas, pub)
    assert st["slots"] >= s["diag"].size * (sweeps if kind == "GaussSeidel" else 1)
    assert st["maxTileCells"] <= tile
    assert st["ctas"] <= ctas


def test_too_narrow_a_grid_is_refused():
    s = MESHES["cube16"]
    with pytest.raises(ldu.CfxError) as e:
        ldu.sched_tiled_check(s["diag"].size, s["l"], s["u"], "GaussSeidel", 2, 32, 1, 1)
    assert e.value.status == -8
