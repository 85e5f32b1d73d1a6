"""CPU tests of the benchmark configurations' host-side construction (no device work)."""
from __future__ import annotations

import numpy as np


def test_config_shapes():
    from speo_gb300 import workloads as w

    s1, i1 = w.config1_specs()
    assert len(s1) == 64 and {s.pop_size for s in s1} == {100} and {s.dim for s in s1} == {30}
    assert [s.ring_next for s in s1][:3] == [1, 2, 3] and s1[-1].ring_next == 0
    s2, i2 = w.config2_specs(16)
    assert {s.dim for s in s2} == {100} and len(i2) == 16
    assert {s.func_id for s in s2} <= {w.SPHERE, w.RASTRIGIN}
    s3, i3 = w.config3_specs(64)
    assert {s.dim for s in s3} <= {10, 30, 50, 100} and all(50 <= s.pop_size <= 200 for s in s3)
    s4, _ = w.config4_specs()
    assert len(s4) == 128 and {s.pop_size for s in s4} == {256} and {s.dim for s in s4} == {50}


def test_mixed_table_layout_cpu():
    """A batched-uneven table built on the CPU: rows contiguous per run, one stride, balanced tiles."""
    from speo_gb300 import workloads as w

    specs, inst = w.config3_specs(32)
    tab = w.table(specs, inst, device="cpu")
    assert tab.rows == sum(s.pop_size for s in specs)
    assert tab.ld == max((s.dim + 3) // 4 * 4 for s in specs)
    rows = np.zeros(tab.rows, dtype=int)
    for it in tab.host_items:
        seg = tab.host_segs[it.segment]
        rows[seg.row0 + it.first: seg.row0 + it.first + it.count] += 1
        assert it.count <= 64
    assert np.all(rows == 1)
