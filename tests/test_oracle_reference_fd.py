"""The reference's derivative tests 1.1, 1.2 and 1.4 (src/tests.cpp:31-107)
run on the oracle with the reference's own protocol (tests/reference_fd.py).

These three test every vertex of their meshes, so nothing is left to the
reference's rand(): the oracle, bit-exact with the reference's CPU renderer
on these models, must give the errors the reference's own test binary
prints for them (1.1 = 0.012, 1.2 = 0.013, 1.4 = 0.072 for the colours), and
pass its bar of 0.5.
"""
import pytest

import reference_fd as F


@pytest.mark.parametrize("case,key,printed", [(1, "pos", 0.012), (2, "pos", 0.013), (4, "color", 0.072)])
def test_reference_derivative_tests_on_the_oracle(case, key, printed):
    err = F.run(F.OracleBackend(F.CASES[case][0]), case)
    print(case, err)
    assert err[key] == pytest.approx(printed, abs=5e-4)
    assert all(v is None or v < F.PASS[k] for k, v in err.items() if k != "nonzero")
