"""Host-side helpers of bench.py that need no GPU."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_committed_traffic_is_read_from_the_step_profile():
    """bench.py's roofline `traffic` comes from the committed ncu summary of
    the step kernels; the summary must keep the line it parses, with the
    per-step DRAM bytes of the three kernels (a few bytes per cell-step)."""
    import bench
    t = bench.committed_traffic()
    assert t is not None
    cells = 256 ** 3
    assert 1.0 < t / cells < 20.0
