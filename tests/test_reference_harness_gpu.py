"""The reference's own verification harness, ``tests/verification_3d.py`` of
the reference repository, run unmodified on this library's drop-in kernels
(all 20 cases, each judged by the harness's own pass rules).

The harness file, the reference's host helpers and its ``config_3d.yaml``
come from a checkout of the reference named by MPF3D_REFERENCE_ROOT; without
one the test is skipped.  numba, PyYAML and matplotlib are replaced by the
test-only stand-ins of ``tests/harness`` where they are not installed.  The
run is a subprocess, so the assembled ``src`` package and the stand-ins never
reach this test process.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_reference_harness_passes_all_cases(tmp_path):
    ref = os.environ.get("MPF3D_REFERENCE_ROOT")
    if not ref or not os.path.exists(os.path.join(ref, "tests", "verification_3d.py")):
        pytest.skip("needs a checkout of the reference repository (MPF3D_REFERENCE_ROOT)")
    r = subprocess.run([sys.executable, os.path.join(HERE, "harness", "run_reference_verification.py"),
                        "--reference", ref, "--out", str(tmp_path)], capture_output=True, text=True, timeout=3600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["kernel_modules"]["src.gpu_kernels_3d"].startswith(os.path.dirname(HERE))
    names = [c["name"] for c in res["cases"]]
    assert len(names) == 20, names
    failed = [(c["name"], c["failure_reason"] or c["summary"]) for c in res["cases"] if not c["passed"]]
    assert not failed, failed
    assert res["exit_status"] == 0
