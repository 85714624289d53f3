"""Serving loop (drgb_server_*): admission by memory budget and slots,
continuous batching, and the same result for a job alone and in the mix."""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D

pytestmark = pytest.mark.gpu


def job(kind, seed):
    """(scene, init scene, cams, targets, settings, params) of a small job."""
    if kind == "ico":
        true = D.make_icosphere(3, seed=seed)
        init = D.perturb_vertices(true, 0.02, seed=seed + 1, radial=True)
        cams = D.ring_cameras(2, 3.0, 48, 48)
        st = D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4)
        lr = 0.005
    elif kind == "cube":
        true = D.make_cube(seed=seed)
        init = D.perturb_vertices(true, 0.1, seed=seed + 1)
        cams = [D.CamInfo(origin=(0, 0, 3), width=64, height=64)]
        st = D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 16)
        lr = 0.01
    else:  # a larger displaced sphere
        true = D.displace_radially(D.make_uv_sphere(24, 48, seed=seed), seed=seed + 7, n_waves=8, amplitude=0.05)
        init = D.perturb_vertices(true, 0.02, seed=seed + 1, radial=True)
        cams = D.ring_cameras(3, 3.0, 96, 96)
        st = D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 8)
        lr = 0.005
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    r = D.MakeDifferentialRenderer(st)
    r.commit(ts)
    tgt = r.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=lr)
    p.base_lr = lr
    return isc, cams, tgt, st, p


def run_alone_plain_and_mix(deterministic, steps=12):
    a = job("ico", 4)
    srv = D.OptimizationServer(deterministic=deterministic)
    ta = srv.submit(a[0], a[1], a[2], a[3], a[4], steps)
    srv.wait(ta, timeout=120)
    assert srv.info(ta)["state"] == "done"
    alone = (srv.losses(ta), srv.result_scene(ta))
    srv.close()
    # the plain one-job optimiser
    r = D.MakeDifferentialRenderer(a[3])
    if deterministic:
        r.set_option(D.native.OPT_DETERMINISTIC, 1)
    opt = D.CreateSimpleOptimizer()
    opt.Init(a[0], r, a[1], a[2], a[4])
    opt.Run(steps)
    plain = (np.array(opt.losses), opt.current_scene())
    # in a mix with jobs of other models and sizes that finish at other steps
    mix = D.OptimizationServer(deterministic=deterministic)
    others = [job("cube", 1), job("sphere", 11), job("cube", 21)]
    t1 = mix.submit(*others[0][:5], 30)
    t2 = mix.submit(*others[1][:5], 5)
    tm = mix.submit(a[0], a[1], a[2], a[3], a[4], steps)
    t3 = mix.submit(*others[2][:5], 8)
    mix.wait(0, timeout=300)
    for t in (t1, t2, tm, t3):
        assert mix.info(t)["state"] == "done"
        assert mix.info(t)["steps_done"] == mix.info(t)["steps"]
    ms, jobs = mix.step_times()
    assert jobs.max() >= 3                          # the jobs really overlapped
    mixed = (mix.losses(tm), mix.result_scene(tm))
    mix.close()
    return a, alone, plain, mixed


def test_server_job_same_alone_and_in_mix():
    """Deterministic reduction: the same bits alone, in the plain optimiser
    and in the mix."""
    a, alone, plain, mixed = run_alone_plain_and_mix(True)
    assert np.array_equal(alone[0], mixed[0]) and np.array_equal(alone[0], plain[0])
    for s in (plain[1], mixed[1]):
        assert np.array_equal(s.meshes[0].vertices, alone[1].meshes[0].vertices)
        assert np.array_equal(s.meshes[0].colors, alone[1].meshes[0].colors)


def test_server_job_alone_and_in_mix_atomic_mode():
    """Float atomics: the first forward pass is identical; afterwards the
    summation order can flip the sign of near-zero gradient components, whose
    step the reference's normalised update makes a full learning-rate step,
    and the trajectories drift apart at a rate that varies from run to run.
    Measured relative loss deviation from the job alone over 12 steps: the
    first three at most 1e-6; the last ones 3e-3 to 5e-3 in one run and up
    to 4.9e-2 in another.  Bounds: 1e-4 for the first three steps, 0.1 for
    all (the deterministic mode, above, gives the same bits)."""
    a, alone, plain, mixed = run_alone_plain_and_mix(False)
    assert alone[0][0] == mixed[0][0] == plain[0][0]
    assert alone[0].size == mixed[0].size == plain[0].size == 12
    for name, other in (("mix", mixed[0]), ("plain", plain[0])):
        print(name, "relative loss deviation per step", np.round(np.abs(other / alone[0] - 1), 6).tolist())
        np.testing.assert_allclose(other[:3], alone[0][:3], rtol=1e-4)
        np.testing.assert_allclose(other, alone[0], rtol=0.1)


def test_server_budget_and_slots():
    jobs = [job("cube", 100 + k) for k in range(5)]
    est = D.estimate_job_bytes(jobs[0][0], jobs[0][1], mode=int(D.SHADING_MODEL.VERTEX_COLOR), spp=16)
    # measured device bytes of one such job
    probe = D.OptimizationServer(worker=False)
    t = probe.submit(*jobs[4][:5], 1)
    probe.step()
    measured = probe.info(t)["device_bytes"]
    assert 0 < measured <= est                      # the estimate is an upper bound
    probe.close()
    # admission charges residents at their measured size and a candidate at its
    # estimate: this budget holds exactly two of these jobs at a time
    budget = 2 * measured + est - 1
    srv = D.OptimizationServer(hbm_budget_bytes=budget)
    tickets = [srv.submit(*j[:5], 6) for j in jobs[:4]]
    srv.wait(0, timeout=300)
    st = srv.stats()
    assert st["done"] == 4 and st["failed"] == 0
    assert st["bytes_peak"] <= budget and st["bytes_in_use"] == 0
    ms, resident = srv.step_times()
    assert resident.max() == 2 and resident.min() >= 1
    assert st["job_iterations"] == 4 * 6 == int(resident.sum())
    for t in tickets:
        i = srv.info(t)
        assert 0 <= i["t_submit"] <= i["t_admit"] <= i["t_done"]
        assert i["device_bytes"] == measured
    srv.close()
    # a job larger than the whole budget is refused at submission
    small = D.OptimizationServer(hbm_budget_bytes=est // 2)
    with pytest.raises(D.native.DrgbError) as e:
        small.submit(*jobs[0][:5], 3)
    assert e.value.code == -3
    small.close()
    # one slot: one job at a time
    one = D.OptimizationServer(max_jobs=1)
    for j in jobs[:3]:
        one.submit(*j[:5], 4)
    one.wait(0, timeout=300)
    ms, resident = one.step_times()
    assert (resident == 1).all() and ms.size == 12
    one.close()


def test_server_manual_steps_and_failed_job():
    srv = D.OptimizationServer(worker=False)
    good = job("cube", 5)
    bad = list(job("cube", 6))
    bad[4] = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.01, diff_mesh_ids=(3,))  # no mesh 3
    tg = srv.submit(*good[:5], 5)
    tb = srv.submit(*bad[:5], 5)
    n = 0
    while srv.stats()["done"] + srv.stats()["failed"] < 2:
        srv.step()
        n += 1
        assert n < 50
    assert srv.info(tg)["state"] == "done" and srv.info(tg)["steps_done"] == 5
    assert srv.info(tb)["state"] == "failed" and srv.info(tb)["error"] != 0
    assert np.isfinite(srv.losses(tg)).all()
    srv.release(tg)
    with pytest.raises(D.native.DrgbError):
        srv.info(tg)
    srv.close()


def test_server_estimate_covers_large_job():
    true = D.displace_radially(D.make_uv_sphere(80, 160, seed=3), seed=4, n_waves=8, amplitude=0.05)
    s = D.Scene()
    s.add_mesh(true)
    cams = D.ring_cameras(4, 3.0, 256, 256)
    est = D.estimate_job_bytes(s, cams, mode=int(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR), spp=4)
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4))
    r.commit(s)
    tgt = r.render(s, cams)
    srv = D.OptimizationServer(worker=False)
    t = srv.submit(s, cams, tgt, D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4),
                   D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.001), 2)
    srv.step()
    measured = srv.info(t)["device_bytes"]
    assert measured <= est <= 3 * measured
    while srv.stats()["done"] < 1:
        srv.step()
    srv.close()
