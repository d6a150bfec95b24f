"""Ray-query parity (closest hit and any hit) of the CUDA traversal against the CPU oracle.

Workload shapes follow the ray-query microbenchmark: incoherent rays (origins uniform in the scene box,
directions uniform on the sphere) and secondary-like rays (origins on random surface points, cosine
hemisphere directions), tmax ~ U[0.1, scene diagonal]. Primitive and instance IDs must match bit-exactly;
hit distances within 1e-5 relative (the arithmetic is identical, so they are expected to be equal)."""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cornell(core_lib, oracle_lib):
    from lighthouse2_gb300.core import RenderCore
    sc = S.cornell_sphere(subdiv=6)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return sc, core, o


@pytest.fixture(scope="module")
def spheres(core_lib, oracle_lib):
    from lighthouse2_gb300.core import RenderCore
    sc = S.spheres_2m(n_spheres=8, slices=40, stacks=26, tex_size=64)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return sc, core, o


def _compare_closest(g, c):
    assert np.array_equal(g["prim"], c["prim"]), f"prim mismatch on {np.count_nonzero(g['prim'] != c['prim'])} rays"
    hit = c["prim"] >= 0
    assert np.array_equal(g["inst"][hit], c["inst"][hit])
    rel = np.abs(g["t"][hit] - c["t"][hit]) / np.maximum(np.abs(c["t"][hit]), 1e-30)
    assert rel.max(initial=0) <= 1e-5
    assert np.array_equal(g["bary"][hit], c["bary"][hit])


@pytest.mark.parametrize("kind", ["incoherent", "secondary"])
@pytest.mark.parametrize("scene", ["cornell", "spheres"])
def test_closest_and_any(kind, scene, request):
    sc, core, o = request.getfixturevalue(scene)
    rays = S.random_rays(sc, 200_000, seed=11 if kind == "incoherent" else 12, kind=kind)
    g = core.trace_host(rays, mode=0)
    c = o.trace(rays, mode=0)
    _compare_closest(g, c)
    if scene == "cornell":
        assert (c["prim"] >= 0).mean() > 0.2   # closed room: most rays hit
    assert (c["prim"] >= 0).sum() > 100
    ga = core.trace_host(rays, mode=1)
    ca = o.trace(rays, mode=1)
    assert np.array_equal(ga, ca)


def test_empty_and_degenerate_rays(cornell):
    sc, core, o = cornell
    rays = np.zeros(64, S.RAY_DTYPE)
    rays["o"] = (0.0, 1.0, 0.0)
    rays["d"][:, 2] = -1.0
    rays["tmax"] = np.linspace(0.0, 5.0, 64)           # tmax 0 -> miss
    rays["d"][5] = (0.0, 0.0, 0.0)                      # zero direction
    rays["tmin"][6] = 10.0                               # tmin > tmax
    rays["d"][7] = (1e-30, 0.0, 0.0)
    g = core.trace_host(rays, 0)
    c = o.trace(rays, 0)
    _compare_closest(g, c)
    assert np.array_equal(core.trace_host(rays, 1), o.trace(rays, 1))
    assert len(core.trace_host(rays[:0], 0)) == 0


@pytest.mark.parametrize("scene", ["cornell", "spheres"])
def test_negative_tmin(scene, request):
    """Rays with tmin < 0 find hits behind their origins: the closest hit is the smallest t above tmin, which may be
    negative. Once such a hit is found, pending boxes the ray entered before its origin must still be visited."""
    sc, core, o = request.getfixturevalue(scene)
    rays = S.random_rays(sc, 100_000, seed=21, kind="incoherent")
    span = float(np.linalg.norm(np.asarray(sc.bounds[1]) - np.asarray(sc.bounds[0])))
    rng = np.random.default_rng(5)
    rays["tmin"] = -rng.uniform(0.0, 0.5, len(rays)) * span
    rays["tmin"][:1000] = -1e30
    g = core.trace_host(rays, mode=0)
    c = o.trace(rays, mode=0)
    _compare_closest(g, c)
    behind = (c["prim"] >= 0) & (c["t"] < 0)
    assert behind.sum() > 1000
    assert np.array_equal(core.trace_host(rays, mode=1), o.trace(rays, mode=1))


@pytest.mark.parametrize("scene", ["cornell", "spheres"])
def test_nan_rays(scene, request):
    """A NaN in a ray's origin, direction, tmin or tmax makes it a miss (and never occluded), as in the oracle, without
    a traversal that the box tests' NaN handling would otherwise widen to every box along the ray's other axes."""
    sc, core, o = request.getfixturevalue(scene)
    rays = S.random_rays(sc, 20_000, seed=31, kind="incoherent")
    nan = np.float32(np.nan)
    rays["o"][0:500, 0] = nan
    rays["o"][500:1000, 1:] = nan
    rays["d"][1000:1500] = nan                       # the whole direction
    rays["d"][1500:2000, 2] = nan
    rays["tmin"][2000:2500] = nan
    rays["tmax"][2500:3000] = nan
    g = core.trace_host(rays, mode=0)
    c = o.trace(rays, mode=0)
    _compare_closest(g, c)
    assert (g["prim"][:3000] < 0).all() and (g["prim"][3000:] >= 0).sum() > 1000
    ga = core.trace_host(rays, mode=1)
    assert np.array_equal(ga, o.trace(rays, mode=1)) and not ga[:3000].any()
