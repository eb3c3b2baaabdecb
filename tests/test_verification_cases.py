"""The remaining verification cases of the reference's 3D suite run through
the oracle on the CPU (tests/verification_cases.py): each meets the
reference's pass rule and reproduces the values the reference recorded for
it in tests/verification_report.md."""
import numpy as np
import pytest

pytest.importorskip("scipy")
import verification_cases as V
from mpf3d import inputs


def oracle_runner(phi0, temp_value, quats, phys, steps, aniso, torque, sample_every=None, observer=None):
    """The reference harness's step sequence (run_3d_simulation,
    tests/verification_3d.py:830-904) on the oracle."""
    import oracle as O
    N, nx, ny, nz = phi0.shape
    wij, aij, mij = inputs.matrices_for(phys, N)
    n111 = inputs.rotated_n111(quats)
    sc = O.make_scalars(list(phys.kernel_scalars(f32=False)), True)
    rate = phys.derived()["cooling_rate"]
    phi = np.ascontiguousarray(phi0, np.float32)
    temp = np.full((nx, ny, nz), np.float32(temp_value), np.float32)
    samples, done = [], 0
    chunk = sample_every or steps
    while done < steps:
        k = min(chunk, steps - done)
        phi, temp, _, _ = O.run(phi, temp, wij, aij, mij, n111, sc, k, cooling_rate=rate, rate_f32=True,
                                cooling=rate != 0.0, checked=True, switchable=True, aniso=aniso, torque=torque)
        done += k
        if observer is not None:
            samples.append(observer(phi, done))
    return phi, samples


@pytest.fixture(scope="module")
def scan_cache():
    return {}


@pytest.mark.parametrize("name", list(V.CASES))
def test_case_passes_and_matches_recorded_values(name, scan_cache):
    vals, passed = V.run_case(name, oracle_runner, cache=scan_cache)
    assert passed, vals
    assert V.compare_recorded(name, vals) == []
