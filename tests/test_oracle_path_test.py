"""The oracle's PATH_TEST model against the reference's own renders.

shade<PATH_TEST> (src/shade_path_test.cpp:183-289) draws from the C
library's shared rand(), in whatever order the OpenMP threads call it, so no
two runs of the reference give the same image and parity can only be
statistical.  The fixture `render_path_test` holds the reference's mean image
over 16 renders at 64 spp and the per-value variance across those renders
(tests/golden/make_golden.py path_test).  The oracle restates the model with
a counter-based generator; 16 renders with seeds 1000..1015 give its mean and
variance.  Per value, z = (mean_oracle - mean_ref) / sqrt((var_oracle +
var_ref) / 16) is close to a Student t with ~30 degrees of freedom when both
estimate the same expectation:

  * mean of z^2 below 1.3 (measured 1.10; a t with 30 degrees of freedom has
    E[t^2] = 1.07),
  * every |z| below 5.5 (measured 3.7 over 2,028 values),
  * the mean image level within 2e-3 relative (measured 6e-5),
  * values without variance (background, ambient 0.5) equal.

A model error the size of the one this test caught while it was written (the
light colour used without PointLight's normalisation, scene.h:77-82) gave a
mean z^2 of 325.
"""
import numpy as np

import pyoracle as O
from fixtures import cams_from, load, scene_from

REPEATS, SPP = 16, 64


def oracle_stats(sc, cams):
    imgs = np.stack([O.render(sc, cams, O.PATH_TEST, SPP, mp=O.model_params(seed=1000 + k)) for k in range(REPEATS)])
    return imgs.mean(0), imgs.var(0, ddof=1)


def test_path_test_oracle_matches_reference_in_expectation():
    d = load("render_path_test")
    assert int(d["repeats"][0]) == REPEATS and int(d["spp"][0]) == SPP and int(d["mode"][0]) == O.PATH_TEST
    sc, cams = scene_from(d), cams_from(d)
    ref, ref_var = d["out.images"], d["out.images_var"]
    got, got_var = oracle_stats(sc, cams)
    noisy = (ref_var + got_var) > 0
    assert noisy.sum() > 1000  # most of the image is sphere and floor
    z = (got - ref)[noisy] / np.sqrt((got_var + ref_var)[noisy] / REPEATS)
    print(f"mean z^2 {np.mean(z * z):.3f}, max |z| {np.abs(z).max():.2f} over {z.size} values")
    assert np.mean(z * z) < 1.3
    assert np.abs(z).max() < 5.5
    assert abs(got.mean() - ref.mean()) < 2e-3 * ref.mean()
    assert np.array_equal(got[~noisy], ref[~noisy])
