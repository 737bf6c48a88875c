"""Tuning parameters: validation on the host; on the GPU, every setting gives
the same results and the autotuner returns a valid, applied setting."""
import numpy as np
import pytest

from distance3d_gb300 import _lib
from distance3d_gb300.tune import autotune, get_tuning, set_tuning


def test_tuning_validation():
    start = get_tuning()
    try:
        assert set_tuning(gjk_block=256, epa_warps=2)["gjk_block"] == 256
        assert get_tuning()["epa_warps"] == 2
        for bad in (dict(gjk_block=96), dict(epa_warps=3), dict(sort_min=-1), dict(gjk_warps_per_sm=-2)):
            with pytest.raises(_lib.D3DError):
                set_tuning(**bad)
        with pytest.raises(ValueError):
            set_tuning(threads=1)
    finally:
        set_tuning(**start)


@pytest.mark.gpu
def test_every_tuning_same_results():
    from distance3d_gb300 import workloads
    from distance3d_gb300.serve import CollisionBatch
    from distance3d_gb300.store import ColliderStore
    cs, i1, i2 = workloads.pairs_mixed_six(12000, seed=51, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    start = get_tuning()
    try:
        ref = None
        for t in (dict(gjk_block=128, gjk_warps_per_sm=0, epa_warps=4, sort_min=4096),
                  dict(gjk_block=64, gjk_warps_per_sm=16, epa_warps=2, sort_min=2 ** 31 - 1),
                  dict(gjk_block=256, gjk_warps_per_sm=0, epa_warps=8, sort_min=0)):
            set_tuning(**t)
            for precision in ("mixed", "fp64"):
                r = CollisionBatch(st, 12000, precision=precision, graphs=False,
                                   epa_kw=dict(max_faces=256, max_loose_edges=128)).run(i1, i2)
                if ref is None:
                    ref = {}
                if precision not in ref:
                    ref[precision] = r
                    continue
                for k in r:
                    assert np.array_equal(r[k], ref[precision][k], equal_nan=True), (t, precision, k)
        best = autotune(st, i1[:8192], i2[:8192], epa_kw=dict(max_faces=256, max_loose_edges=128))
        assert best == get_tuning()
        assert best["gjk_block"] in (64, 128, 256) and best["epa_warps"] in (2, 4, 8)
    finally:
        set_tuning(**start)
