"""The serving loop (lh2g_server_*) on the GPU.

Jobs of two resident scenes with different resolutions, sample counts and depths, submitted all at once so that
they share the wavefront queues, must each produce exactly the image the plain core renders for the same job
alone (lh2g_render_ex, accumulator after one frame), and the same image when the job runs alone through the
server, whether the jobs go through the shared queues, run as express jobs (each path traced whole within a tick)
or both. A capacity smaller than the sum of the jobs makes them wait for path memory and still complete exactly;
a job larger than the capacity is refused at submission. Ray queries run beside the render jobs and return what
lh2g_trace_host returns. One job is checked against the CPU oracle as well.
"""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, CoreError, make_params, camera_r0, RP_NEE, RP_DEPTH_W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_scenes(core_lib):
    a = S.cornell_sphere(subdiv=4)
    b = S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=128)
    ca, cb = RenderCore(), RenderCore()
    ca.set_scene(a)
    cb.set_scene(b)
    return (a, ca), (b, cb)


JOBS = [  # (scene, W, H, spp, depth, rr, frame)
    (0, 64, 48, 1, 4, 2, 0), (1, 80, 48, 2, 8, 4, 0), (0, 32, 32, 4, 6, 1, 1), (1, 120, 72, 1, 5, 3, 2),
    (0, 96, 64, 2, 3, 1, 3), (1, 40, 40, 3, 7, 2, 4), (0, 128, 96, 1, 8, 4, 5), (1, 64, 64, 1, 4, 1, 6),
]


def job_inputs(sc_idx, W, H, spp, depth, rr, frame):
    view = S.cornell_view(W, H) if sc_idx == 0 else S.spheres_view(W, H, frame=frame)
    p = make_params(W, H, spp, max_depth=depth, rr_start=rr, samples_taken=frame % 3, camera_r0=camera_r0(frame),
                    flags=RP_NEE | RP_DEPTH_W)
    return view, p


def plain_core_image(core, view, p):
    core.SetTarget(int(p["width"]), int(p["height"]), int(p["spp"]))
    core.render_ex(view, p, accumulate=False, counters=False)
    return core.read_accumulator()


@pytest.mark.parametrize("express_max,device_loop", [(None, 1), (None, 0), (5000, 1), (5000, 0), (1 << 20, 1)])
def test_jobs_in_the_mix_equal_plain_core_and_alone(two_scenes, express_max, device_loop):
    """express_max: all jobs through the queues (default), mixed, all express; device_loop: ticks in the device-side
    graph loop (default) or launched by the host one by one"""
    from lighthouse2_gb300.server import RenderServer
    (sa, ca), (sb, cb) = two_scenes
    cores = [ca, cb]
    expect = []
    for j in JOBS:
        view, p = job_inputs(*j)
        expect.append(plain_core_image(cores[j[0]], view, p))
    opts = {"deviceLoop": device_loop}
    if express_max is not None:
        opts["expressMaxPaths"] = express_max
    srv = RenderServer(path_capacity=1 << 20, **opts)
    sid = [srv.add_scene(ca), srv.add_scene(cb)]
    # all at once: the jobs share ticks
    ids = []
    for j in JOBS:
        view, p = job_inputs(*j)
        ids.append(srv.submit_render(sid[j[0]], view, p))
    for k, jid in enumerate(ids):
        srv.wait(jid)
        got = srv.result(jid)
        assert np.array_equal(got.view(np.uint32), expect[k].view(np.uint32)), f"job {k} in the mix differs from the plain core"
        assert got[:, :3].sum() > 0
    # alone, one after the other
    for k, j in enumerate(JOBS):
        view, p = job_inputs(*j)
        jid = srv.submit_render(sid[j[0]], view, p)
        srv.wait(jid)
        assert np.array_equal(srv.result(jid).view(np.uint32), expect[k].view(np.uint32)), f"job {k} alone differs"
        srv.release(jid)
    st = srv.stats()
    assert st["jobsDone"] == 2 * len(JOBS) and st["deviceStatus"] == 0 and st["pathsInFlight"] == 0
    assert (st["loopLaunches"] > 0) == bool(device_loop)
    srv.close()


def test_admission_by_path_memory_and_queries(two_scenes, oracle_lib):
    from lighthouse2_gb300.server import RenderServer
    (sa, ca), (sb, cb) = two_scenes
    cap = 20000                                  # smaller than the sum of the jobs below: they queue for memory
    srv = RenderServer(path_capacity=cap, expressMaxPaths=0)   # (express jobs would not use queue memory)
    sid = [srv.add_scene(ca), srv.add_scene(cb)]
    jobs = [(0, 96, 96, 2, 5, 2, 0), (1, 100, 100, 1, 6, 3, 1), (0, 64, 64, 4, 4, 1, 2), (1, 128, 64, 2, 5, 2, 3)]
    assert all(j[1] * j[2] * j[3] <= cap for j in jobs) and sum(j[1] * j[2] * j[3] for j in jobs) > cap
    rays = S.random_rays(sb, 20000, seed=3)
    q0 = srv.submit_trace(sid[1], rays, mode=0)
    ids = []
    for j in jobs:
        view, p = job_inputs(*j)
        ids.append(srv.submit_render(sid[j[0]], view, p))
    q1 = srv.submit_trace(sid[1], rays, mode=1)
    for k, jid in enumerate(ids):
        t = srv.wait(jid)
        assert t[0] <= t[1] <= t[2]
        view, p = job_inputs(*jobs[k])
        exp = plain_core_image([ca, cb][jobs[k][0]], view, p)
        assert np.array_equal(srv.result(jid).view(np.uint32), exp.view(np.uint32)), f"job {k} under admission limits differs"
    # admission counts the live paths of the jobs in flight: the queue never had to drop new paths
    assert srv.stats()["deviceStatus"] == 0
    srv.wait(q0), srv.wait(q1)
    assert np.array_equal(srv.result(q0), cb.trace_host(rays, 0))
    assert np.array_equal(srv.result(q1), cb.trace_host(rays, 1))
    # a job larger than the capacity is refused
    view, p = job_inputs(0, 200, 200, 1, 3, 1, 0)
    with pytest.raises(CoreError):
        srv.submit_render(sid[0], view, p)
    # one job against the CPU oracle
    o = oracle_lib.Oracle()
    o.set_scene(sa)
    view, p = job_inputs(0, 48, 40, 2, 5, 2, 1)
    jid = srv.submit_render(sid[0], view, p)
    srv.wait(jid)
    ref = o.render(view, p)["accum"]
    rel = np.abs(srv.result(jid) - ref) / np.maximum(np.abs(ref), 1e-6)
    assert rel.max() <= 1e-4
    srv.close()


def test_large_job_lane(two_scenes):
    """Jobs of at least "largeJobPaths" paths run as plain frames on the server's own stream beside the ticks (and
    need no queue memory: one is larger than the queue capacity); every image equals the plain core's, in the mix
    and alone."""
    from lighthouse2_gb300.server import RenderServer
    (sa, ca), (sb, cb) = two_scenes
    cores = [ca, cb]
    jobs = JOBS + [(1, 320, 240, 1, 6, 3, 7), (0, 256, 256, 2, 5, 2, 2)]   # 76,800 and 131,072 paths
    expect = []
    for j in jobs:
        view, p = job_inputs(*j)
        expect.append(plain_core_image(cores[j[0]], view, p))
    srv = RenderServer(path_capacity=1 << 16, largeJobPaths=6000)
    sid = [srv.add_scene(ca), srv.add_scene(cb)]
    ids = []
    for j in jobs:
        view, p = job_inputs(*j)
        ids.append(srv.submit_render(sid[j[0]], view, p))
    for k, jid in enumerate(ids):
        srv.wait(jid)
        assert np.array_equal(srv.result(jid).view(np.uint32), expect[k].view(np.uint32)), f"job {k} differs from the plain core"
        srv.release(jid)
    view, p = job_inputs(*jobs[-1])
    jid = srv.submit_render(sid[jobs[-1][0]], view, p)
    srv.wait(jid)
    assert np.array_equal(srv.result(jid).view(np.uint32), expect[-1].view(np.uint32))
    st = srv.stats()
    assert st["deviceStatus"] == 0 and st["pathsInFlight"] == 0 and st["raysTraced"] > 0
    srv.close()


@pytest.mark.parametrize("tick_budget", [0, 3000])
def test_device_loop(two_scenes, tick_budget):
    """"deviceLoop": ticks run on the device inside one graph launch (a conditional WHILE node) until a job finishes
    or one is submitted; with a small tick budget the device admits the further ranges of the jobs in flight. Every
    image equals the plain core's, in the mix and with jobs submitted while a loop runs; a launch runs several ticks."""
    from lighthouse2_gb300.server import RenderServer
    (sa, ca), (sb, cb) = two_scenes
    cores = [ca, cb]
    expect = []
    for j in JOBS:
        view, p = job_inputs(*j)
        expect.append(plain_core_image(cores[j[0]], view, p))
    opts = {"deviceLoop": 1}
    if tick_budget:
        opts["tickBudget"] = tick_budget
    srv = RenderServer(path_capacity=1 << 16, **opts)
    sid = [srv.add_scene(ca), srv.add_scene(cb)]
    for rnd in range(2):
        ids = []
        for k, j in enumerate(JOBS):
            view, p = job_inputs(*j)
            ids.append(srv.submit_render(sid[j[0]], view, p))
            if rnd == 1 and k == 1:
                srv.wait(ids[0])            # later jobs arrive while earlier ones run
        for k, jid in enumerate(ids):
            srv.wait(jid)
            assert np.array_equal(srv.result(jid).view(np.uint32), expect[k].view(np.uint32)), f"job {k} differs (round {rnd})"
            srv.release(jid)
    st = srv.stats()
    assert st["deviceStatus"] == 0 and st["pathsInFlight"] == 0 and st["jobsDone"] == 2 * len(JOBS)
    assert 0 < st["loopLaunches"] < st["ticks"], st   # launches ran more than one tick each on average
    srv.close()


@pytest.mark.parametrize("express_max", [None, 1 << 20])
def test_deepest_paths_served(two_scenes, express_max):
    """maxDepth 64 without Russian roulette in the closed room: served paths carry their depth up to 64 in their flag
    word (through the queues, or whole as express jobs), beside a shallow job; images equal the plain core's."""
    from lighthouse2_gb300.server import RenderServer
    (sa, ca), (sb, cb) = two_scenes
    kw = {} if express_max is None else {"expressMaxPaths": express_max}
    srv = RenderServer(path_capacity=1 << 16, **kw)
    sid = [srv.add_scene(ca), srv.add_scene(cb)]
    jobs = [(0, 32, 24, 2, 64, 64, 1), (1, 40, 32, 1, 4, 2, 2), (0, 24, 24, 1, 64, 30, 3)]
    ids = []
    for j in jobs:
        view, p = job_inputs(*j)
        ids.append(srv.submit_render(sid[j[0]], view, p))
    for k, jid in enumerate(ids):
        srv.wait(jid)
        view, p = job_inputs(*jobs[k])
        exp = plain_core_image([ca, cb][jobs[k][0]], view, p)
        assert np.array_equal(srv.result(jid).view(np.uint32), exp.view(np.uint32)), f"job {k} differs"
    assert srv.stats()["deviceStatus"] == 0
    srv.close()
