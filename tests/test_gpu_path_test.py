"""PATH_TEST (the reference's path tracer, src/shade_path_test.cpp:183-289)
on the GPU.

The reference draws its random numbers from the shared rand(); the GPU and
the oracle draw them from the same counter-based generator (sample key,
bounce, job seed), with the same sin/cos polynomial for the concentric disk
map, so:

  * against the oracle with the same seed (brute-force traversal, the
    oracle's caster): images within 1e-4 max abs per value; loss of
    d_render_and_compare to 1e-5 relative, gradients within 1e-3 (interior:
    the texture term of shade_grad<TEXTURE_COLOR>, shade_path_test.cpp:284-289)
    and 1e-2 (edge) relative L2;
  * against the reference itself (fixture `render_path_test`: its mean image
    over 16 renders at 64 spp, and the per-value variance), 16 GPU renders
    with the hierarchy, seeds 1000..1015: the statistics of the oracle's own
    test (tests/test_oracle_path_test.py): mean z^2 < 1.3, |z| < 5.5, mean
    level within 2e-3, values without variance equal;
  * 20 steps of the reference's optimiser on the sphere's texture follow
    the oracle's losses within 2 % relative.
"""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O
from fixtures import cams_from, load, rel_l2, scene_from

pytestmark = pytest.mark.gpu

REPEATS, SPP = 16, 64
INTERIOR_TOL, EDGE_TOL, IMAGE_TOL = 1e-3, 1e-2, 1e-4


def renderer(spp, seed, bruteforce=False):
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.PATH_TEST, spp))
    r.set_model_params(D.ModelParams(seed=seed))
    r.set_option(N.OPT_TRACE_BRUTEFORCE, int(bruteforce))
    return r


@pytest.fixture(scope="module")
def scene():
    d = load("render_path_test")
    return d, scene_from(d), cams_from(d)


def test_path_test_render_vs_oracle(scene):
    _, sc, cams = scene
    r = renderer(SPP, 7, bruteforce=True)
    r.commit(sc)
    got = r.render(sc, cams).reshape(-1)
    ref = O.render(sc, cams, O.PATH_TEST, SPP, mp=O.model_params(seed=7))
    diff = np.abs(got - ref)
    print(f"PATH_TEST vs oracle: max abs {diff.max():.3g}, {int((diff > 0).sum())} of {diff.size} values differ")
    assert diff.max() <= IMAGE_TOL


def test_path_test_mean_image_vs_reference(scene):
    d, sc, cams = scene
    imgs = []
    for k in range(REPEATS):
        r = renderer(SPP, 1000 + k)
        r.commit(sc)
        imgs.append(r.render(sc, cams).reshape(-1))
    imgs = np.stack(imgs)
    got, got_var = imgs.mean(0), imgs.var(0, ddof=1)
    ref, ref_var = d["out.images"], d["out.images_var"]
    noisy = (ref_var + got_var) > 0
    z = (got - ref)[noisy] / np.sqrt((got_var + ref_var)[noisy] / REPEATS)
    print(f"GPU vs reference: mean z^2 {np.mean(z * z):.3f}, max |z| {np.abs(z).max():.2f} over {z.size} values")
    assert np.mean(z * z) < 1.3
    assert np.abs(z).max() < 5.5
    assert abs(got.mean() - ref.mean()) < 2e-3 * ref.mean()
    assert np.array_equal(got[~noisy], ref[~noisy])


def perturbed(sc):
    init = sc.copy()
    m = init.meshes[0]
    m.textures[0].data[:] = np.float32(0.5)
    m.vertices = D.perturb_vertices(m, 0.01, seed=3).vertices
    return init


def test_path_test_d_render_and_compare_vs_oracle(scene):
    _, sc, cams = scene
    spp, samples = 16, 32 * 32
    tgt = O.render(sc, cams, O.PATH_TEST, spp, mp=O.model_params(seed=5))
    init = perturbed(sc)
    r = renderer(spp, 9, bruteforce=True)
    r.commit(init)
    ds = D.DScene(r, [0])
    imgs = np.zeros(tgt.size, np.float32)
    loss = r.d_render_and_compare(init, cams, tgt, samples, ds, out_images=imgs)
    oloss, ods, oimgs = O.d_render_and_compare(init, cams, O.PATH_TEST, spp, tgt, samples, mp=O.model_params(seed=9))
    assert np.abs(imgs - oimgs).max() <= IMAGE_TOL
    assert loss == pytest.approx(oloss, rel=1e-5)
    nv, _, p, c, t = (int(x) for x in ds.layout[0][:5])
    assert c < 0 and t >= 0  # texture and positions, no vertex colours (dmesh.h:41-44)
    ntex = sc.meshes[0].textures[0].data.size
    gp, rp = ds.data[p:p + 3 * nv], ods[p:p + 3 * nv]
    gt, rt = ds.data[t:t + ntex], ods[t:t + ntex]
    assert np.abs(rt).max() > 0 and np.abs(rp).max() > 0
    assert rel_l2(gt, rt) <= INTERIOR_TOL, rel_l2(gt, rt)
    assert rel_l2(gp, rp) <= EDGE_TOL, rel_l2(gp, rp)


def test_path_test_optimizer_follows_the_oracle(scene):
    """20 "Adam" steps of the sphere's texture alone (the reference's
    optimiser, graph-replayed): the losses follow the oracle's trajectory
    and fall by more than 10x."""
    _, sc, cams = scene
    spp = 16
    tgt = O.render(sc, cams, O.PATH_TEST, spp, mp=O.model_params(seed=11))
    init = sc.copy()
    init.meshes[0].textures[0].data[:] = np.float32(0.5)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.0, tex_lr=0.05)
    p.flags = D.OptimizerParameters._OPT_TEX
    opt = D.CreateSimpleOptimizer()
    opt.Init(init, renderer(spp, 11), cams, tgt, p)
    opt.Run(20)
    orc = O.optimize(init, cams, O.PATH_TEST, spp, tgt, O.opt_params(position_lr=0.0, textures_lr=0.05, flags=p.flags),
                     20, mp=O.model_params(seed=11))
    got, ref = np.asarray(opt.losses, np.float64), orc["losses"].astype(np.float64)
    print("losses", got[[0, 5, 10, 19]], "oracle", ref[[0, 5, 10, 19]])
    assert np.allclose(got, ref, rtol=2e-2), np.abs(got / ref - 1).max()
    assert got[-1] < 0.1 * got[0]


def test_path_test_in_a_batch_gives_the_plain_bits(scene):
    """Deterministic mode: a PATH_TEST job alone and batched beside a
    vertex-colour job (the batch's flattening writes its tangents, its
    group runs the PATH_TEST pixel kernel and the generic edge shader)
    gives the same losses and texture, bit for bit."""
    _, sc, cams = scene
    spp, iters = 16, 3
    tgt = O.render(sc, cams, O.PATH_TEST, spp, mp=O.model_params(seed=11))
    init = sc.copy()
    init.meshes[0].textures[0].data[:] = np.float32(0.5)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.001, tex_lr=0.05)
    st = D.DiffRenderSettings(D.SHADING_MODEL.PATH_TEST, spp)
    mp = D.ModelParams(seed=11)
    r = renderer(spp, 11)
    r.set_option(N.OPT_DETERMINISTIC, 1)
    opt = D.CreateSimpleOptimizer()
    opt.Init(init, r, cams, tgt, p)
    opt.Run(iters)
    cube = D.make_cube(seed=1)
    cs = D.Scene()
    cs.add_mesh(cube)
    vc = D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 4)
    rc = D.MakeDifferentialRenderer(vc)
    rc.commit(cs)
    ctgt = rc.render(cs, cams)
    b = D.BatchOptimizer()
    b.set_option(N.OPT_DETERMINISTIC, 1)
    b.add_job(cs, cams, ctgt, vc, D.OptimizerParameters(D.OptimizerParameters.GD_Adam))
    jid = b.add_job(init, cams, tgt, st, p, model_params=mp)
    b.run(iters)
    assert np.array_equal(b.losses(jid), np.asarray(opt.losses, np.float32))
    got = b.job_scene(jid).meshes[0]
    ref = opt.current_scene().meshes[0]
    assert np.array_equal(got.textures[0].data, ref.textures[0].data)
    assert np.array_equal(got.vertices, ref.vertices)
