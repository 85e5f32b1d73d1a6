"""The allocation-free ring migration, against the one that takes caller scratch.

speo_ring_migrate_noalloc exists for callers that cannot allocate device memory (a plugin
whose host process owns all device memory, a loop that must not allocate once running): its
staging is a fixed array inside the library. This file runs last in the suite so that a failure
here leaves every other test already run; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ring(cuda, n_islands=16, P=100, D=30):
    from speo_gb300.device import SegmentSpec, SegmentTable
    from speo_gb300.instances import make_instance

    inst = [make_instance(77, D)]
    specs = [SegmentSpec(pop_size=P, dim=D, func_id=9, instance=0, seed=500 + i, ring_next=(i + 1) % n_islands)
             for i in range(n_islands)]
    return SegmentTable(specs, inst, device=str(cuda))


def test_noalloc_migration_matches_caller_staging(lib, cuda):
    import torch
    from speo_gb300 import _lib

    bits = ctypes.c_uint32(0)
    assert lib.speo_device_error_bits(ctypes.byref(bits)) == 0    # reads and clears earlier flags
    a, b = _ring(cuda), _ring(cuda)
    a.init_population()
    b.init_population()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):                           # two calls in a row, on fresh data each time
        a.generation()
        b.generation()
        torch.cuda.synchronize()
        assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
        a.migrate(5)
        _lib.check(lib.speo_ring_migrate_noalloc(b.d_segs.data_ptr(), len(b.specs), 5, b.pop[b.cur].data_ptr(),
                                                 b.fit[b.cur].data_ptr(), b.max_ld, stream),
                   "speo_ring_migrate_noalloc")
        torch.cuda.synchronize()
        # migration moves rows bit for bit: the two versions must agree exactly
        assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy()), f"call {call}"
        assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy()), f"call {call}"
    assert lib.speo_device_error_bits(ctypes.byref(bits)) == 0 and bits.value == 0


def test_noalloc_migration_rejects_oversize(lib, cuda):
    from speo_gb300 import _lib

    tab = _ring(cuda, n_islands=4)
    too_big_ld = _lib.NOALLOC_STAGING_FLOATS // (4 * 32)     # 4 segments x 32 migrants x (ld + 1) > limit
    st = lib.speo_ring_migrate_noalloc(tab.d_segs.data_ptr(), 4, 32, tab.pop[0].data_ptr(), tab.fit[0].data_ptr(),
                                       too_big_ld, None)
    assert st == _lib.SPEO_ERR_INVALID_ARG
    assert b"exceed the fixed" in lib.speo_last_error()


def test_noalloc_migration_at_the_exact_staging_limit(lib, cuda):
    """One segment migrating into itself with max_ld = 2^20 - 1 needs exactly the fixed array
    (1 x 1 x 2^20 floats): accepted, and equal to the caller-staged version; one float more is
    rejected before any device work."""
    import torch
    from speo_gb300 import _lib

    a, b = _ring(cuda, n_islands=1), _ring(cuda, n_islands=1)
    a.init_population()
    b.init_population()
    a.generation()
    b.generation()
    lim = _lib.NOALLOC_STAGING_FLOATS
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    staging = torch.zeros(lim, device=cuda)
    _lib.check(lib.speo_ring_migrate(a.d_segs.data_ptr(), 1, 1, a.pop[a.cur].data_ptr(), a.fit[a.cur].data_ptr(),
                                     staging.data_ptr(), lim - 1, stream), "speo_ring_migrate")
    _lib.check(lib.speo_ring_migrate_noalloc(b.d_segs.data_ptr(), 1, 1, b.pop[b.cur].data_ptr(),
                                             b.fit[b.cur].data_ptr(), lim - 1, stream), "speo_ring_migrate_noalloc")
    torch.cuda.synchronize()
    assert np.array_equal(a.pop[a.cur].cpu().numpy(), b.pop[b.cur].cpu().numpy())
    assert np.array_equal(a.fit[a.cur].cpu().numpy(), b.fit[b.cur].cpu().numpy())
    st = lib.speo_ring_migrate_noalloc(b.d_segs.data_ptr(), 1, 1, b.pop[b.cur].data_ptr(), b.fit[b.cur].data_ptr(),
                                       lim, stream)
    assert st == _lib.SPEO_ERR_INVALID_ARG
