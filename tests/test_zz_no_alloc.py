"""gapgpu_neighbours_static against gapgpu_neighbours, through the C ABI, on the GPU.

gapgpu_neighbours_static is for host codes that cannot allocate device memory: codes
whose HBM all belongs to their own pool allocator, and time-step loops that must not
call cudaMalloc/cudaFree because those synchronise the device.  It keeps its scratch in
one fixed device array inside the library, so it must give the allocating entry
point's list exactly, call after call, whatever the previous call left in that array.
The lists are integers, so the tolerance is zero: offsets, neighbour indices and
shifts must be identical, element by element, in the same order.

This file is named to be collected last, so that a run stopping at the first failure
has already run every other test.
"""
import ctypes
import os

import numpy as np
import pytest

from quip_gb300 import _lib, models

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUTOFF = 5.0


def _static_list(at, cutoff):
    """Two-phase use as a caller without an allocator would do it: count, then fill
    into caller-owned device buffers (torch allocates them here, outside the call)."""
    import torch
    L = _lib.load()
    n = len(at)
    stream = torch.cuda.current_stream()
    d_pos = torch.tensor(np.ascontiguousarray(at.positions, dtype=np.float64), device="cuda")
    lat = np.asfortranarray(at.lattice, dtype=np.float64).ravel(order="F").copy()
    pbc = np.asarray(at.pbc, dtype=np.int32).reshape(3).copy()
    d_off = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    tot = ctypes.c_int64(-1)
    _lib.check(L.gapgpu_neighbours_static(n, d_pos.data_ptr(), _lib.ptr(lat), _lib.ptr(pbc), cutoff, d_off.data_ptr(),
                                          None, None, 0, ctypes.byref(tot), ctypes.c_void_p(stream.cuda_stream)))
    cap = tot.value
    d_j = torch.full((max(cap, 1),), -7, dtype=torch.int32, device="cuda")
    d_sh = torch.full((max(cap, 1), 3), -7, dtype=torch.int32, device="cuda")
    tot2 = ctypes.c_int64(-1)
    _lib.check(L.gapgpu_neighbours_static(n, d_pos.data_ptr(), _lib.ptr(lat), _lib.ptr(pbc), cutoff, d_off.data_ptr(),
                                          d_j.data_ptr(), d_sh.data_ptr(), cap, ctypes.byref(tot2),
                                          ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    assert tot2.value == cap
    return d_off.cpu().numpy(), d_j.cpu().numpy()[:cap], d_sh.cpu().numpy()[:cap]


def _cases():
    rng = np.random.default_rng(17)
    big = models.si_diamond(4, rattle=0.08, seed=5)            # 512 atoms, periodic
    small = models.random_triclinic(9, rng=rng)                 # small cell: many periodic images
    cluster = models.si_diamond(2, rattle=0.05, seed=6)
    cluster.pbc = np.array([False, False, False])               # calc_lat_eff path
    mixed = models.si_diamond(2, rattle=0.05, seed=7)
    mixed.pbc = np.array([True, False, True])
    return [("si512", big), ("triclinic9", small), ("cluster64", cluster), ("mixed_pbc64", mixed),
            ("si512_again", big)]


def test_static_neighbours_match_allocating_entry_point():
    from quip_gb300.potential import Potential
    pot = Potential(param_filename=os.path.join(ROOT, "tests", "golden", "gap_water", "GAP.xml"))
    for name, at in _cases():
        ref_off, ref_j, ref_sh = pot.neighbours(at, CUTOFF)
        # two calls in a row on the same structure, each after a different predecessor
        for _ in range(2):
            off, j, sh = _static_list(at, CUTOFF)
            np.testing.assert_array_equal(off, ref_off, err_msg=name)
            np.testing.assert_array_equal(j, ref_j, err_msg=name)
            np.testing.assert_array_equal(sh, ref_sh, err_msg=name)
        assert len(ref_j) > 0, name


def test_static_neighbours_reject_sizes_above_the_limit():
    import torch
    L = _lib.load()
    n = 65536 + 1  # GAPGPU_STATIC_MAX_ATOMS + 1: rejected before any device access
    d_pos = torch.zeros(3, dtype=torch.float64, device="cuda")
    d_off = torch.zeros(1, dtype=torch.int32, device="cuda")
    lat = np.eye(3).ravel(order="F") * 100.0
    pbc = np.ones(3, np.int32)
    tot = ctypes.c_int64(-1)
    rc = L.gapgpu_neighbours_static(n, d_pos.data_ptr(), _lib.ptr(lat), _lib.ptr(pbc), CUTOFF, d_off.data_ptr(), None,
                                    None, 0, ctypes.byref(tot), None)
    assert rc == _lib.ERR_ARG
    assert b"static limit" in L.gapgpu_last_error()
    assert tot.value == -1
