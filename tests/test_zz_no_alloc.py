"""d3d_epa_noalloc: EPA for callers that may not allocate device memory while
they run (a control loop on a fixed memory budget, a plugin whose host
application owns every GPU allocation).  It must give the same results as
d3d_epa, which takes a caller buffer and temporaries from the library's pool,
and as the oracle.

Two option sets cover its two paths: the defaults, whose polytopes the
one-warp-per-pair kernel keeps in shared memory (the static array then holds
only the work counter), and 252 iterations, one more than that kernel takes,
whose polytopes live in the static array's slots (2,184 slots of 64 faces and
32 loose edges; the grid is capped at 17 blocks of 128 threads, so the first
call below has more pairs than the array has slots in use at a time).

Calls the C ABI directly.  Kept in a file of its own, collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from distance3d_gb300 import _lib, workloads
from distance3d_gb300.epa import epa_batch
from distance3d_gb300.gjk import gjk_distance_batch
from distance3d_gb300.store import ColliderStore, _ptr
from oracle import oracle

pytestmark = pytest.mark.gpu

# the EPA tests compare FP64 results bit for bit; so does this one
WARP_KW = dict(max_iter=64, max_loose_edges=32, max_faces=64, epsilon=1e-8)
SLOT_KW = dict(max_iter=252, max_loose_edges=32, max_faces=64, epsilon=1e-8)
SLOT_THREADS = 17 * 128  # (16 MiB - 256 B) // (8 * (12 * 64 + 6 * 32)) = 2,184 slots -> 17 blocks of 128


def noalloc(store, i1, i2, simplex, kw):
    opts = _lib.EpaOptions(kw["max_iter"], kw["max_loose_edges"], kw["max_faces"], 0, kw["epsilon"])
    dev = store.device
    n = len(i1)
    a = torch.as_tensor(i1, dtype=torch.int32, device=dev)
    b = torch.as_tensor(i2, dtype=torch.int32, device=dev)
    s = torch.as_tensor(simplex, dtype=torch.float64, device=dev).contiguous()
    mtv = torch.full((n, 3), -7.0, dtype=torch.float64, device=dev)
    status = torch.full((n,), -1, dtype=torch.int8, device=dev)
    nf = torch.full((n,), -1, dtype=torch.int32, device=dev)
    faces = torch.zeros((n, opts.max_faces, 4, 3), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        rc = _lib.load().d3d_epa_noalloc(store.view, _ptr(a), _ptr(b), n, _ptr(s), ctypes.byref(opts), _ptr(mtv),
                                         _ptr(status), _ptr(nf), _ptr(faces), store.stream())
    _lib.check(rc)
    torch.cuda.synchronize(dev)
    return dict(mtv=mtv.cpu().numpy(), status=status.cpu().numpy(), n_faces=nf.cpu().numpy(),
                faces=faces.cpu().numpy())


def intersecting(seed, n):
    cs, i1, i2 = workloads.pairs_mixed_six(n, seed=seed, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    st = ColliderStore(cs)
    g = {k: v.cpu().numpy() for k, v in gjk_distance_batch(st, i1, i2).items()}
    hit = np.flatnonzero((g["dist"] == 0.0) & (g["n_simplex"] == 4))
    return cs, st, i1[hit], i2[hit], g["simplex"][hit]


def same(got, want):
    assert np.array_equal(got["status"], want["status"])
    assert np.array_equal(got["n_faces"], want["n_faces"])
    assert np.array_equal(got["mtv"], want["mtv"], equal_nan=True)
    for k in range(len(got["status"])):
        nf = want["n_faces"][k]
        assert np.array_equal(got["faces"][k, :nf], want["faces"][k, :nf])


@pytest.mark.parametrize("kw", [WARP_KW, SLOT_KW], ids=["warp_kernel", "static_slots"])
def test_noalloc_matches_epa_and_oracle_on_two_calls_in_a_row(kw):
    # first more EPA pairs than the slot path runs at a time, then fewer
    for seed, n in ((41, 12000), (42, 3000)):
        cs, st, i1, i2, simplex = intersecting(seed, n)
        assert len(i1) > 500
        if seed == 41:
            assert len(i1) > SLOT_THREADS
        got = noalloc(st, i1, i2, simplex, kw)
        want = {k: v.cpu().numpy() for k, v in epa_batch(st, i1, i2, simplex, return_faces=True, **kw).items()}
        same(got, want)
        same(got, oracle.epa(cs, i1, i2, simplex, want_faces=True, **kw))
    # with 64 faces some polytopes outgrow the face buffer, so that status ran too
    assert (got["status"] == _lib.STATUS_EPA_FACE_OVERFLOW).any()


def test_noalloc_rejects_oversized_polytopes():
    _, st, i1, i2, simplex = intersecting(43, 200)
    # 16,384 faces: beyond a block's shared memory (32 B per face) and, at
    # 12 * 16384 + 6 * 4096 doubles per pair, room for 9 pairs in the array
    big = _lib.EpaOptions(64, 4096, 16384, 0, 1e-8)
    a = torch.as_tensor(i1, dtype=torch.int32, device=st.device)
    rc = _lib.load().d3d_epa_noalloc(st.view, _ptr(a), _ptr(a), len(i1), None, ctypes.byref(big), None, None,
                                     None, None, st.stream())
    assert rc == _lib.D3D_ERR_CAPACITY
    assert b"static scratch" in _lib.load().d3d_last_error()
