"""Runs the reference's own verification harness, ``tests/verification_3d.py``
of daikihatanaka0327/multiphasefield-solidification-v2, unmodified, on this
library's drop-in kernels (``src/gpu_kernels_3d.py`` and ``src/gpu_kernels.py``
of this repository).

Test infrastructure only.  The harness imports ``src.gpu_kernels_3d``,
``src.gpu_kernels`` and the reference's host helpers (``src.orientation_utils``,
``src.seed_modes*``, ``src.plot_utils*``) from one package ``src``; here that
package is assembled from two directories, this repository's ``src`` first,
so the two kernel modules resolve to the drop-ins and every other module to
the reference's own file.  Where numba, PyYAML or matplotlib is not installed,
the stand-ins next to this file take its place (device arrays on torch, a
block-style YAML reader, figures not drawn).  The harness runs in a scratch
directory holding a copy of the reference's ``config_3d.yaml``, as it would
from the reference's root.

    python tests/harness/run_reference_verification.py --reference <checkout> [--out DIR] [CASE ...]

Prints one JSON line: every case's verdict and summary, from the harness's
own CSV, and the harness's exit status.
"""

from __future__ import annotations

import argparse
import csv
import importlib
import importlib.util
import json
import os
import shutil
import sys
import tempfile
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "multiphasefield-solidification-v2_gb300")


def _stand_in(name: str) -> str:
    """Import `name`, or load the stand-in next to this file in its place."""
    try:
        importlib.import_module(name)
        return "installed"
    except ImportError:
        pass
    pkg_dir = os.path.join(HERE, name)
    if os.path.isdir(pkg_dir):
        spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                      submodule_search_locations=[pkg_dir])
    else:
        spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return "stand-in"


def run(reference: str, out_dir: str, cases=None) -> dict:
    reference = os.path.abspath(reference)
    harness = os.path.join(reference, "tests", "verification_3d.py")
    if not os.path.exists(harness):
        raise FileNotFoundError(harness)
    # run as a script, this file's directory is first on sys.path and would
    # let the stand-ins shadow installed packages: take it out, then load a
    # stand-in only where the real package is missing
    sys.path[:] = [p for p in sys.path if os.path.abspath(p or os.curdir) != HERE]
    used = {m: _stand_in(m) for m in ("numba", "yaml", "matplotlib")}
    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    src = types.ModuleType("src")
    src.__path__ = [os.path.join(PKG, "src"), os.path.join(reference, "src")]
    sys.modules["src"] = src
    os.makedirs(out_dir, exist_ok=True)
    work = tempfile.mkdtemp(prefix="refverif_", dir=out_dir)
    shutil.copy(os.path.join(reference, "config_3d.yaml"), os.path.join(work, "config_3d.yaml"))
    cwd = os.getcwd()
    os.chdir(work)
    try:
        spec = importlib.util.spec_from_file_location("verification_3d", harness)
        vmod = importlib.util.module_from_spec(spec)
        sys.modules["verification_3d"] = vmod
        spec.loader.exec_module(vmod)
        argv = ["verification_3d.py", "--out-dir", "out", "--report-path", "verification_report.md"]
        if cases:
            argv += ["--cases", *cases]
        sys.argv = argv
        rc = vmod.main()
        rows = list(csv.DictReader(open(os.path.join("out", "verification_results.csv"), encoding="utf-8")))
    finally:
        os.chdir(cwd)
    kernels = {m: getattr(sys.modules.get(m), "__file__", None) for m in ("src.gpu_kernels_3d", "src.gpu_kernels")}
    return {"exit_status": rc, "modules": used, "kernel_modules": kernels, "work_dir": work,
            "cases": [{"name": r.get("name"), "passed": r.get("passed") == "1", "summary": r.get("summary"),
                       "failure_reason": r.get("failure_reason")} for r in rows],
            "rows": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="checkout of the reference repository")
    ap.add_argument("--out", default=tempfile.gettempdir())
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    print(json.dumps(run(a.reference, a.out, a.cases or None), default=str))


if __name__ == "__main__":
    main()
