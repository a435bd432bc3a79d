"""EDGE raster mode of the oracle: the inside test the reference's mask
encodes (main.h:1440: all three biased edge functions > 0) applied, where the
reference itself (REF mode) writes every pixel of a face's rectangle."""
import numpy as np

from oracle import pyoracle as po

CAM = po.camera()


def _tri(rng, size):
    c = rng.uniform([60, 60], [580, 420])
    v = np.zeros((3, 3), np.float32)
    v[:, :2] = c + rng.normal(0, size, (3, 2))
    v[:, 2] = rng.uniform(300, 1500, 3)
    return v


def _img(zb):
    return zb[po.GUARD:po.GUARD + CAM.height, po.GUARD:po.GUARD + CAM.width]


def test_edge_writes_are_a_subset_of_ref_with_equal_depths():
    rng = np.random.default_rng(3)
    covered = 0
    for _ in range(200):
        v = _tri(rng, rng.choice([1.0, 4.0, 15.0]))
        zr, ze = po.zbuf_new(CAM), po.zbuf_new(CAM)
        nr, br = po.raster_face(v[0], v[1], v[2], CAM, zr)
        ne, be = po.raster_face(v[0], v[1], v[2], CAM, ze, mode=po.RASTER_EDGE)
        assert list(br) == list(be)  # the render AABB takes every face rectangle either way
        written = ze < po.DEPTH_BG
        assert ne <= nr
        np.testing.assert_array_equal(ze[written], zr[written])
        covered += int(written.sum())
    assert covered > 1000


def _edge_inside_exact(v):
    """Covered pixels recomputed from the definition with exact integers:
    28.4 snapping of the vertices, sample point (x, y) at integer pixel
    coordinates, edge function E_ij(p) = DX_ij (16 y) - DY_ij (16 x) + C_ij
    with C_ij = DY_ij X_i - DX_ij Y_i plus the top-left bias, inside when all
    three are > 0."""
    X = [int(np.rint(np.float32(16.0) * np.float32(p[0]))) for p in v]
    Y = [int(np.rint(np.float32(16.0) * np.float32(p[1]))) for p in v]
    if (X[0] - X[1]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[0] - Y[1]) <= 0:
        return set()
    minx, maxx = (min(X) + 15) >> 4, (max(X) + 15) >> 4
    miny, maxy = (min(Y) + 15) >> 4, (max(Y) + 15) >> 4
    out = set()
    edges = [(0, 1), (1, 2), (2, 0)]
    for y in range(miny, maxy):
        for x in range(minx, maxx):
            ok = True
            for i, j in edges:
                dx, dy = X[i] - X[j], Y[i] - Y[j]
                c = dy * X[i] - dx * Y[i] + (1 if (dy < 0 or (dy == 0 and dx > 0)) else 0)
                if dx * (16 * y) - dy * (16 * x) + c <= 0:
                    ok = False
                    break
            if ok:
                out.add((y, x))
    return out


def test_edge_coverage_matches_exact_definition():
    rng = np.random.default_rng(4)
    for _ in range(150):
        v = _tri(rng, rng.choice([0.8, 3.0, 10.0]))
        ze = po.zbuf_new(CAM)
        po.raster_face(v[0], v[1], v[2], CAM, ze, mode=po.RASTER_EDGE)
        got = {(int(y), int(x)) for y, x in zip(*np.nonzero(_img(ze) < po.DEPTH_BG))}
        assert got == _edge_inside_exact(v)


def test_edge_fan_is_watertight():
    """Triangles sharing edges (a fan around a centre) cover every pixel
    sample at most once (top-left fill convention) and the covered count is
    the polygon's area to within its perimeter."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        c = rng.uniform([200, 150], [440, 330])
        n = int(rng.integers(5, 9))
        # a star-shaped polygon: angular gaps below pi keep the fan a partition
        ang = 2 * np.pi * (np.arange(n) + rng.uniform(-0.3, 0.3, n)) / n
        rad = rng.uniform(20, 60, n)
        ring = np.stack([c[0] + rad * np.cos(ang), c[1] + rad * np.sin(ang)], 1)
        ring = np.round(ring * 16) / 16  # shared vertices snap identically
        cc = np.round(c * 16) / 16
        zb = po.zbuf_new(CAM)
        writes = 0
        area = 0.0
        for i in range(n):
            a, b = ring[i], ring[(i + 1) % n]
            tri = np.array([[cc[0], cc[1], 900.0], [b[0], b[1], 900.0], [a[0], a[1], 900.0]], np.float32)
            if (tri[0, 0] - tri[1, 0]) * (tri[2, 1] - tri[0, 1]) - (tri[2, 0] - tri[0, 0]) * (tri[0, 1] - tri[1, 1]) <= 0:
                tri = tri[[0, 2, 1]]
            k, _ = po.raster_face(tri[0], tri[1], tri[2], CAM, zb, mode=po.RASTER_EDGE)
            writes += k
            area += 0.5 * abs((a[0] - cc[0]) * (b[1] - cc[1]) - (b[0] - cc[0]) * (a[1] - cc[1]))
        distinct = int((_img(zb) < po.DEPTH_BG).sum())
        assert writes == distinct  # no pixel written twice
        perim = sum(np.hypot(*(ring[(i + 1) % n] - ring[i])) for i in range(n))
        assert abs(distinct - area) <= perim


def test_edge_mode_solve_runs_and_differs_from_ref():
    import scene
    from tests.helpers import oracle_obs, oracle_params

    w = scene.workload_c1()
    s = dict(w["solves"][0], particles=16, iterations=4)
    soa, F = w["meshes"][0]
    ref = po.solve(soa, F, oracle_obs(w, s), CAM, oracle_params(s), trace=True)
    edge = po.solve(soa, F, oracle_obs(w, s), CAM, oracle_params(s, raster_mode=po.RASTER_EDGE), trace=True)
    assert not np.array_equal(ref["trace_gbest"], edge["trace_gbest"])
    assert np.isfinite(edge["fit"])
