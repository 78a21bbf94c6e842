"""CPU: the benchmark's readers of the committed ncu summaries, and the reusable
result buffers of the Python binding."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from parafrost_gb300.sigma import ResultBuffers  # noqa: E402


def test_profiled_lines_for_the_hot_kernels():
    for kernel in ("mis_rounds", "bve_decide"):
        t = bench.profiled_traffic(kernel, "aig-2.2m")
        assert t and t > 0
        u = bench.profiled_utilisation(kernel, "aig-2.2m")
        assert u and 0 < u["sm_throughput_pct"] <= 100 and 0 < u["dram_throughput_pct"] <= 100
    assert bench.profiled_traffic("mis_rounds", "no-such-workload") is None


def test_profiled_line_for_the_default_workload():
    # the default workload's election traffic, measured at full size, rides along in the
    # benchmark line beside the algorithmic bytes it is compared with
    t = bench.profiled_traffic("mis_rounds", "community-20m")
    assert t and t > 1e9
    u = bench.profiled_utilisation("mis_rounds", "community-20m")
    assert u and 0 < u["dram_throughput_pct"] <= 100 and u["launch"] == "round_average"


def test_result_buffers_grow_and_reuse():
    sizes = []
    buf = ResultBuffers(lambda n: sizes.append(n) or np.empty(n, dtype=np.uint8))
    a = buf.take("lits", 10, np.uint32)
    assert a.shape == (10,) and a.dtype == np.uint32 and sizes == [40]
    b = buf.take("lits", 8, np.uint32)  # fits: same memory, no allocation
    assert sizes == [40] and np.shares_memory(a, b)
    c = buf.take("lits", 11, np.uint32)  # grows
    assert sizes == [40, 44] and c.shape == (11,)
    assert buf.take("units", 0, np.uint32).shape == (0,)
