"""Cell facet tables (madi_facets_build): every Voronoi facet is listed, and the
facet margins alone reproduce the SI Eq. S2 label of the all-seed rule."""

import numpy as np
import pytest

from custom_madi_gb300.ensemble import build_facets


def _images(pts, L):
    off = np.array([(x, y, z) for x in (-1, 0, 1) for y in (-1, 0, 1) for z in (-1, 0, 1)], np.float64)
    P = (pts[None, :, :] + L * off[:, None, :]).reshape(-1, 3)
    ids = np.tile(np.arange(len(pts)), len(off))
    return P, ids, 13 * len(pts)      # offset (0, 0, 0) is the 14th block


def _table(beg, pl, nbr, c):
    rows, nb = pl[beg[c]:beg[c + 1]], nbr[beg[c]:beg[c + 1]]
    return rows, nb


@pytest.mark.parametrize("n", [27, 64, 300])
def test_periodic_facets_are_the_delaunay_neighbours(n):
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(n)
    L = 10.0
    pts = rng.uniform(0.0, L, (n, 3))
    beg, pl, nbr, h_max, reach = build_facets(np.c_[pts, np.full(n, 0.2)], True, L)
    assert np.all(np.diff(beg.astype(np.int64)) % 4 == 0)
    P, ids, centre = _images(pts, L)
    tri = spatial.Delaunay(P)
    ptr, ind = tri.vertex_neighbor_vertices
    for c in range(n):
        v = centre + c
        want = {(int(ids[j]), tuple(np.round(P[j] - P[v], 6))) for j in ind[ptr[v]:ptr[v + 1]]}
        rows, nb = _table(beg, pl, nbr, c)
        real = nb >= 0
        assert np.all(rows[~real, 3] > 1e37)                       # padding never binds
        u = 2.0 * rows[real, 3:4].astype(np.float64) * rows[real, :3].astype(np.float64)
        # match each listed facet to a Delaunay edge by neighbour id and direction
        got = set()
        for j, uu in zip(nb[real], u):
            cand = [w for w in want if w[0] == j and np.linalg.norm(np.array(w[1]) - uu) < 1e-4 * L]
            assert len(cand) == 1, (c, j, uu)
            got.add(cand[0])
        assert got == want, c
    assert 0.0 < h_max <= reach


def test_periodic_facet_margins_give_the_all_seed_label():
    rng = np.random.default_rng(3)
    n, L = 40, 8.0
    pts = rng.uniform(0.0, L, (n, 3))
    alpha = rng.uniform(0.05, 0.4, n)
    beg, pl, nbr, _, _ = build_facets(np.c_[pts, alpha], True, L)
    P, ids, _ = _images(pts, L)
    q = rng.uniform(0.0, L, (3000, 3))
    d2 = ((q[:, None, :] - P[None]) ** 2).sum(-1)
    i1 = d2.argmin(1)
    c1 = P[i1]
    u = P[None] - c1[:, None, :]
    un = np.linalg.norm(u, axis=-1)
    m = (d2 - d2[np.arange(len(q)), i1][:, None]) / (2.0 * np.where(un > 0, un, 1.0))
    m[np.arange(len(q)), i1] = np.inf
    m_all = m.min(1)
    for k in range(len(q)):
        c = int(ids[i1[k]])
        rows, nb = _table(beg, pl, nbr, c)
        w = q[k] - pts[c]
        w -= L * np.round(w / L)
        mf = (rows[:, 3].astype(np.float64) - rows[:, :3].astype(np.float64) @ w).min()
        assert abs(mf - m_all[k]) < 1e-5, (k, mf, m_all[k])
        assert (mf >= alpha[c]) == (m_all[k] >= alpha[c]) or abs(m_all[k] - alpha[c]) < 1e-5


def test_outer_cells_of_a_finite_population_are_flagged():
    rng = np.random.default_rng(5)
    pts = rng.uniform(0.0, 10.0, (300, 3))
    beg, pl, nbr, _, _ = build_facets(np.c_[pts, np.full(300, 0.2)], False, 10.0)
    first = pl[beg[:-1].astype(np.int64), 3]
    open_ = first < -1e37
    assert 0 < open_.sum() < 300
    # every unbounded cell (seed on the convex hull) is flagged; the others
    # flagged are bounded cells reaching beyond the search radius, all in the
    # outer shell of the population, never interior ones
    spatial = pytest.importorskip("scipy.spatial")
    hull = set(spatial.ConvexHull(pts).vertices.tolist())
    flagged = set(np.flatnonzero(open_).tolist())
    assert hull <= flagged
    depth = np.minimum(pts, 10.0 - pts).min(1)
    assert depth[sorted(flagged - hull)].max(initial=0.0) < 1.5


def test_coincident_seeds_are_rejected():
    pts = np.array([[1.0, 1.0, 1.0, 0.1], [1.0, 1.0, 1.0, 0.1], [3.0, 2.0, 1.0, 0.1], [2.0, 4.0, 3.0, 0.1]])
    with pytest.raises(Exception):
        build_facets(pts, True, 5.0)


def test_fixed_stride_packing_keeps_every_facet_in_its_cell_block():
    from custom_madi_gb300.ensemble import pack_facets
    rng = np.random.default_rng(11)
    pts = rng.uniform(0.0, 9.0, (70, 3))
    beg, pl, nbr, _, _ = build_facets(np.c_[pts, np.full(70, 0.2)], True, 9.0)
    stride, fpl, fnb = pack_facets(beg, pl, nbr)
    assert stride % 32 == 0 and stride >= int(np.diff(beg.astype(np.int64)).max())
    assert fpl.shape == (70, stride, 4) and fnb.shape == (70, stride)
    for c in range(70):
        k = int(beg[c + 1] - beg[c])
        np.testing.assert_array_equal(fpl[c, :k], pl[beg[c]:beg[c + 1]])
        np.testing.assert_array_equal(fnb[c, :k], nbr[beg[c]:beg[c + 1]])
        assert np.all(fpl[c, k:, 3] == np.float32(3.0e38)) and np.all(fpl[c, k:, :3] == 0.0)
        assert np.all(fnb[c, k:] == -1)


def test_packing_declines_cells_with_more_than_64_slots():
    from custom_madi_gb300.ensemble import pack_facets
    beg = np.array([0, 4, 72], np.uint32)
    stride, fpl, fnb = pack_facets(beg, np.zeros((72, 4), np.float32), np.zeros(72, np.int32))
    assert stride == 0 and len(fpl) == 0 and len(fnb) == 0


def test_builder_rejects_bad_arguments_and_reports_capacity():
    import ctypes as C
    from custom_madi_gb300 import _native as N
    pts = np.ascontiguousarray(np.c_[np.random.default_rng(2).uniform(0, 5.0, (20, 3)), np.full(20, 0.1)])
    begin = np.zeros(21, np.uint32)
    total = C.c_int64(0)
    lib = N.lib()
    # one seed, or a periodic box without an edge, is rejected
    assert lib.madi_facets_build(pts.ctypes.data, 1, 1, 5.0, begin.ctypes.data, None, None, 0, C.byref(total), None) == N.MADI_ERR_INVALID
    assert lib.madi_facets_build(pts.ctypes.data, 20, 1, 0.0, begin.ctypes.data, None, None, 0, C.byref(total), None) == N.MADI_ERR_INVALID
    # too small an output: MADI_ERR_CAPACITY with the size needed
    planes = np.zeros((4, 4), np.float32)
    nbr = np.zeros(4, np.int32)
    st = lib.madi_facets_build(pts.ctypes.data, 20, 1, 5.0, begin.ctypes.data, planes.ctypes.data, nbr.ctypes.data, 4,
                               C.byref(total), None)
    assert st == N.MADI_ERR_CAPACITY and total.value > 4
    assert "capacity" in lib.madi_last_error_string().decode()
