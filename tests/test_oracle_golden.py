"""The C oracle against golden vectors produced by the distance3d reference.

The oracle restates the reference's rounding sequence (NumPy/OpenBLAS fused
multiply-add orders), so every comparison here is bit-exact.
"""
import numpy as np
import pytest

from oracle import oracle


@pytest.mark.parametrize("name", ["gjk_mixed6", "gjk_scb", "gjk_all9", "gjk_mesh10"])
def test_gjk_distance_bit_exact(golden, name):
    g, cs = golden(name)
    r = oracle.gjk_distance(cs, g["i1"], g["i2"])
    assert np.array_equal(r["dist"], g["dist"])
    assert np.array_equal(r["n_simplex"], g["n_simplex"])
    assert np.array_equal(r["iterations"], g["iterations"])
    assert np.array_equal(r["cp1"], g["cp1"], equal_nan=True)
    assert np.array_equal(r["cp2"], g["cp2"], equal_nan=True)
    written = ~np.isnan(g["simplex"])
    assert np.array_equal(r["simplex"][written], g["simplex"][written])
    assert np.all(r["status"] == 0)


@pytest.mark.parametrize("name", ["gjk_mixed6", "gjk_scb", "gjk_all9", "gjk_mesh10"])
def test_gjk_intersection_and_aabbs(golden, name):
    g, cs = golden(name)
    h = oracle.gjk_intersection(cs, g["i1"], g["i2"])
    assert np.array_equal(h["hit"], g["intersect"])
    assert np.array_equal(g["intersect"], g["dist"] == 0.0)
    assert np.array_equal(oracle.aabbs(cs), g["aabbs"])


@pytest.mark.parametrize("name", ["gjk_all9", "gjk_mesh10"])
def test_supports_bit_exact(golden, name):
    """Every type's support function, Margin wrappers included, along random
    directions, +/- the local z axis and the zero vector."""
    g, cs = golden(name)
    n = len(cs)
    idx = np.repeat(np.arange(n), 6)
    got = oracle.support_batch(cs, idx, g["support_dirs"].reshape(-1, 3)).reshape(n, 6, 3)
    assert np.array_equal(got, g["supports"])
    assert np.unique(cs.base_types).size >= 9 and cs.wrapped.any()


# the EPA limit settings of the fixtures (tests/golden/make_golden.py): the
# reference's defaults, the bench's polytope, and limits under which the face
# buffer (tight), the iteration bound (short) and the loose-edge list (edges)
# run out on some pairs
EPA_SETTINGS = [("default", {}), ("large", dict(max_faces=256, max_loose_edges=128)),
                ("tight", dict(max_iter=20, max_faces=24, max_loose_edges=6)),
                ("short", dict(max_iter=6, max_faces=256, max_loose_edges=128)),
                ("edges", dict(max_faces=256, max_loose_edges=4)),
                ("eps", dict(max_faces=256, max_loose_edges=128, epsilon=1e-4))]


@pytest.mark.parametrize("fixture", ["mixed6", "all9", "mesh10"])
@pytest.mark.parametrize("tag,kw", EPA_SETTINGS)
def test_epa_bit_exact(golden, fixture, tag, kw):
    g, cs = golden("gjk_" + fixture)
    e, _ = golden("epa_" + fixture)
    p = e["pair"]
    r = oracle.epa(cs, g["i1"][p], g["i2"][p], g["simplex"][p], **kw)
    st = e[f"status_{tag}"]
    assert np.array_equal(r["status"], st)
    # converged, and stopped at the iteration bound (epa.py:76-78 returns the
    # closest face's MTV unconverged)
    ok = (st == 0) | (st == 4)
    assert ok.sum() >= 20
    if tag == "tight":
        assert (st == 5).sum() > 100  # face buffer full (epa.py:128)
    if tag == "short":
        assert (st == 4).sum() > 100  # iteration bound
    assert np.array_equal(r["mtv"][ok], e[f"mtv_{tag}"][ok])
    assert np.array_equal(r["n_faces"][ok], e[f"n_faces_{tag}"][ok])


def test_tree_pairs_equal_brute_force(golden):
    t, cs = golden("aabb_tree")
    assert np.array_equal(oracle.aabbs(cs), t["aabbs"])
    assert np.array_equal(oracle.self_pairs(t["aabbs"]), t["tree_pairs"])
    n = int(t["bvh_n"])
    sub = oracle.self_pairs(t["aabbs"][:n])
    both = np.sort(np.concatenate([sub, sub[:, ::-1]]).view("i4,i4"), axis=0).view(np.int32).reshape(-1, 2)
    assert np.array_equal(both, t["bvh_pairs"])


def test_queries_match_tree(golden):
    t, _ = golden("aabb_tree")
    for q in range(len(t["queries"])):
        want = t["query_idx"][t["query_ptr"][q]:t["query_ptr"][q + 1]]
        got = oracle.cross_pairs(t["queries"][q:q + 1], t["aabbs"])[:, 1]
        assert np.array_equal(np.sort(got), want)


@pytest.mark.parametrize("fixture", ["all9", "mesh10"])
def test_mpr_bit_exact(golden, fixture):
    """mpr_penetration and mpr_intersection on the nine- and ten-type pairs."""
    g, cs = golden("gjk_" + fixture)
    m, _ = golden("mpr_" + fixture)
    r = oracle.mpr(cs, m["i1"], m["i2"])
    assert np.all(r["status"] == 0)
    assert np.array_equal(r["hit"], m["hit"])
    assert m["hit"].sum() > 200
    assert np.array_equal(r["depth"], m["depth"], equal_nan=True)
    assert np.array_equal(r["dir"], m["dir"], equal_nan=True)
    assert np.array_equal(r["pos"], m["pos"], equal_nan=True)
    ri = oracle.mpr(cs, m["i1"], m["i2"], penetration=False)
    assert np.array_equal(ri["hit"], m["hit_intersection"])


@pytest.mark.parametrize("fixture", ["scb", "mixed6", "all9", "mesh10"])
@pytest.mark.parametrize("tag,kw", [("clip", dict(max_distance_squared=0.01)), ("coarse", dict(tolerance=1e-3))])
def test_gjk_options_bit_exact(golden, fixture, tag, kw):
    """gjk_distance_jolt with a clipping distance many pairs exceed
    (MAX_FLOAT, no points, _gjk_jolt.py:209-210) and with a coarse tolerance
    under which the reference's sanity assertion fails on some pairs
    (_gjk_jolt.py:216, status 2 here; on the sphere/capsule/box set it fails
    on none)."""
    g, cs = golden("gjk_" + fixture)
    r = oracle.gjk_distance(cs, g["i1"], g["i2"], **kw)
    st = g[f"status_{tag}"]
    assert np.array_equal(r["status"], st)
    if not (fixture == "scb" and tag == "coarse"):
        assert (st == (1 if tag == "clip" else 2)).sum() > 10
    ok = st != 2
    assert np.array_equal(r["dist"][ok], g[f"dist_{tag}"][ok])
    assert np.array_equal(r["cp1"][ok], g[f"cp1_{tag}"][ok], equal_nan=True)


@pytest.mark.parametrize("fixture", ["all9", "mesh10"])
@pytest.mark.parametrize("tag,kw", [("coarse", dict(tolerance=1e-2)), ("short", dict(max_iterations=3))])
def test_mpr_options_bit_exact(golden, fixture, tag, kw):
    """mpr_penetration with a coarse tolerance and with an iteration bound the
    search runs into (tests/golden/make_golden.py MPR_SETTINGS)."""
    g, cs = golden("gjk_" + fixture)
    m, _ = golden("mpr_" + fixture)
    r = oracle.mpr(cs, m["i1"], m["i2"], **kw)
    assert np.array_equal(r["hit"], m[f"hit_{tag}"])
    assert np.array_equal(r["depth"], m[f"depth_{tag}"], equal_nan=True)


def test_edge_colliders_bit_exact(golden):
    """Degenerate and boundary colliders (zero sizes, tied and zero disk
    normals, flat and point hulls, tied mesh vertices, margins of 0):
    supports, AABBs (NaN where the reference's are), GJK, EPA and MPR."""
    g, cs = golden("edge")
    n = len(cs)
    k = len(g["support_dirs"])
    got = oracle.support_batch(cs, np.repeat(np.arange(n), k), np.tile(g["support_dirs"], (n, 1))).reshape(n, k, 3)
    assert np.array_equal(got, g["supports"], equal_nan=True)
    assert np.array_equal(oracle.aabbs(cs), g["aabbs"], equal_nan=True)
    r = oracle.gjk_distance(cs, g["i1"], g["i2"])
    ok = ~g["sanity"]
    assert np.array_equal(r["status"][~ok], np.full((~ok).sum(), 2))
    for key in ("dist", "n_simplex", "iterations"):
        assert np.array_equal(r[key][ok], g[key][ok]), key
    assert np.array_equal(r["cp1"][ok], g["cp1"][ok], equal_nan=True)
    written = ~np.isnan(g["simplex"])
    assert np.array_equal(r["simplex"][written], g["simplex"][written])
    assert np.array_equal(oracle.gjk_intersection(cs, g["i1"], g["i2"])["hit"], g["intersect"])
    m = oracle.mpr(cs, g["i1"], g["i2"])
    assert np.array_equal(m["hit"], g["mpr_hit"])
    for key in ("depth", "dir", "pos"):
        assert np.array_equal(m[key], g["mpr_" + key], equal_nan=True), key
    assert np.array_equal(oracle.mpr(cs, g["i1"], g["i2"], penetration=False)["hit"], g["mpr_hit_intersection"])
    p = g["epa_pair"]
    for tag, kw in (("default", {}), ("large", dict(max_faces=256, max_loose_edges=128))):
        e = oracle.epa(cs, g["i1"][p], g["i2"][p], g["simplex"][p], **kw)
        st = g[f"epa_status_{tag}"]
        assert np.array_equal(e["status"], st)
        assert np.array_equal(e["mtv"][st == 0], g[f"epa_mtv_{tag}"][st == 0])


def test_mesh_cache_bit_exact(golden):
    """The stock reference MeshGraph's vertex caching (mesh.py:30, 82-85):
    each pair's climbs start from the caches the previous calls left, and
    the oracle, given those caches, reproduces the outputs and the caches
    after the call."""
    g, cs = golden("gjk_mesh_cached")
    cache = g["cache_before"].copy()
    r = oracle.gjk_distance_cached(cs, g["i1"], g["i2"], cache)
    assert np.array_equal(cache, g["cache_after"])
    assert np.array_equal(r["dist"], g["dist"])
    assert np.array_equal(r["n_simplex"], g["n_simplex"])
    assert np.array_equal(r["iterations"], g["iterations"])
    assert np.array_equal(r["cp1"], g["cp1"], equal_nan=True)
    assert np.array_equal(r["cp2"], g["cp2"], equal_nan=True)
    written = ~np.isnan(g["simplex"])
    assert np.array_equal(r["simplex"][written], g["simplex"][written])


def test_mesh_cache_chained(golden):
    """One cache per collider object carried from call to call in the
    fixture's order, one pair per call: the caches each call sees and leaves
    are the recorded ones."""
    g, cs = golden("gjk_mesh_cached")
    state = {}
    for k in range(len(g["i1"])):
        for side, idx in enumerate((g["i1"][k], g["i2"][k])):
            state.setdefault(int(idx), int(g["cache_before"][k, side]))
    for k in range(len(g["i1"])):
        a, b = int(g["i1"][k]), int(g["i2"][k])
        cache = np.array([[state[a], state[b]]], np.int32)
        assert np.array_equal(cache[0], g["cache_before"][k])
        r = oracle.gjk_distance_cached(cs, g["i1"][k:k + 1], g["i2"][k:k + 1], cache)
        assert r["dist"][0] == g["dist"][k]
        assert np.array_equal(cache[0], g["cache_after"][k])
        state[a], state[b] = int(cache[0, 0]), int(cache[0, 1])


def test_mesh_cache_changes_answers(golden):
    """The fixture exercises the cache: climbs from the start vertex stop at
    other tied vertices on many pairs (same distance to rounding, other
    closest points)."""
    g, cs = golden("gjk_mesh_cached")
    r = oracle.gjk_distance(cs, g["i1"], g["i2"])
    written = ~np.isnan(g["cp1"][:, 0])
    differ = written & np.any(r["cp1"] != g["cp1"], axis=1)
    assert differ.sum() > 50
    np.testing.assert_allclose(r["dist"], g["dist"], rtol=0, atol=1e-12)
    assert np.any(g["cache_before"] != g["cache_after"])
