"""300-iteration optimisations against the reference's own, in the shape of
its TESTS 2.1, 2.2 and 2.4 (src/tests.cpp:144-260): the triangle and pyramid
of src/scenes.cpp restated and turned apart between start and target, three
cameras around at distance 5 (create_cameras_around), 256x256, 16 spp,
"Adam" with the tests' learning rates.  The fixtures hold the reference
optimiser's final error and last mesh (tests/golden/make_golden.py
convergence).  On these scenes the reference itself stays below its own
PSNR bar of 35 (6.1, 10.5 and 16.5 dB: the start is turned 70-90 degrees from
the target and the silhouette gradient leads to a local minimum), so the
test asks for the same end point rather than for the bar: the final error
within 5 % of the reference's and the last mesh close to it.  The
gradients are summed in a fixed order (deterministic mode), so the result
is the same on every run; what remains is the reference's different
summation order carried through 300 normalised steps (with float atomics
the final error varies by about 2 % from run to run)."""
import math

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
from fixtures import cams_from, load, scene_from

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["converge_triangle_sil", "converge_pyramid_sil", "converge_pyramid_vc"])
def test_300_iterations_end_where_the_reference_ends(name):
    d = load(name)
    sc, cams = scene_from(d), cams_from(d)
    iters = int(d["iters"][0])
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(int(d["mode"][0])), int(d["spp"][0])))
    r.set_option(N.OPT_DETERMINISTIC, 1)  # the same end point on every run
    opt = D.CreateSimpleOptimizer()
    opt.Init(sc, r, cams, d["targets"], D.OptimizerParameters(D.OptimizerParameters.GD_Adam,
                                                              pos_lr=float(d["opt_pos_lr"][0]),
                                                              tex_lr=float(d["opt_tex_lr"][0])))
    cur, err = opt.Run(iters)
    ref = float(d["out.final_error"][0])
    print(f"{name}: final error {err:.6g} (reference {ref:.6g}), PSNR {-10 * math.log10(err):.2f} dB "
          f"(reference {-10 * math.log10(ref):.2f})")
    assert opt.losses[-1] < opt.losses[0] or name != "converge_triangle_sil"
    assert err == pytest.approx(ref, rel=5e-2)
    dv = np.abs(cur.meshes[0].vertices.reshape(-1) - d[f"out.it{iters - 1}.m0.vertices"].reshape(-1)).max()
    print(f"  last mesh: max vertex difference {dv:.3g}")
    assert dv < 5e-2, dv
