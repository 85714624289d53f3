"""The reference's derivative tests 1.1-1.5 (src/tests.cpp:31-107) on the GPU
renderer, with the reference's own protocol and coordinates
(tests/reference_fd.py): forward differences (h = 2/W for positions, 0.1
for colours and texels) against d_render with W*H edge samples, error
sum|g - fd| / sum(|g| + |fd|), pass below 0.5 (positions, colours) and 0.01
(texture).

  * default renderer (hierarchy): every test passes the reference's bars;
  * with the reference's triangle loop (DRGB_OPT_TRACE_BRUTEFORCE) the
    renders are the reference's bit for bit and the edge samples replay its
    random streams, so the errors are the ones the reference's test binary
    prints: 1.1 = 0.012, 1.2 = 0.013, 1.3 = 0.400, 1.4 = 0.072 (colours;
    the oracle, tests/test_oracle_reference_fd.py, gives the same for 1.1,
    1.2 and 1.4).  The binary did not finish 1.5 within 25 minutes on the
    host (its brute-force caster).
  * 1.5 as written tests nothing: the sphere's texture coordinates
    (CreateSphere, src/scenes.cpp:484-485: v = (1 - i) / (n - 1), zero or
    negative below the pole) clamp to the texture's first row, none of the
    250 drawn texels lies there, and gradient and differences are all zero
    (error 0).  The first row's 256 texels, which the sphere does show, are
    checked against the same bar with central differences.
"""
import pytest

import reference_fd as F

pytestmark = pytest.mark.gpu

PRINTED = {1: ("pos", 0.012), 2: ("pos", 0.013), 3: ("pos", 0.400), 4: ("color", 0.072)}


@pytest.mark.parametrize("case", [1, 2, 3, 4, 5])
def test_reference_derivative_tests_on_the_gpu(case):
    err = F.run(F.GpuBackend(F.CASES[case][0]), case)
    print(case, err)
    tested = {k: v for k, v in err.items() if v is not None and k != "nonzero"}
    assert tested
    for k, v in tested.items():
        assert v < F.PASS[k], (k, v)


@pytest.mark.parametrize("case", [1, 2, 3, 4])
def test_reference_derivative_tests_print_the_reference_errors(case):
    err = F.run(F.GpuBackend(F.CASES[case][0], bruteforce=True), case)
    key, printed = PRINTED[case]
    print(case, err)
    assert err[key] == pytest.approx(printed, abs=5e-4), err


def test_texture_derivatives_on_the_visible_texels():
    import numpy as np
    fwd = F.run(F.GpuBackend(F.TEXTURE_COLOR), 5, texels=np.arange(256))
    cen = F.run(F.GpuBackend(F.TEXTURE_COLOR), 5, texels=np.arange(256), central=True)
    print("forward", fwd, "central", cen)
    assert fwd["nonzero"] > 300  # of 768 channel coordinates
    # the image is linear in a texel, the loss quadratic: a forward
    # difference carries h * w^2 / 2(I - T) of second-order term beside the
    # derivative (measured 0.027), a central one none (0.0029)
    assert fwd["texture"] < 0.05, fwd
    assert cen["texture"] < F.PASS["texture"], cen
