"""fsr_spatial_hash_noalloc: spatial hashing for callers that cannot allocate.

Callers that run inside their own memory pool, or in a step where
cudaMalloc is not allowed, use this entry point; its scratch is a static
device array.  The test calls it through the C ABI and checks its sorted
particles, cell ranges and permutation against those of the existing
allocating entry point (fsr_reconstruct with intermediates kept) for the
same particles, on two calls in a row with different inputs (a larger then a
smaller set, so stale scratch contents from the first call would show), then
repeats the first.  Sorting and ranges are integer results and must match
bit for bit; sorted coordinates are copies and must match exactly.

This file sorts last on purpose (pytest collects it after the other test
files).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind():
    from fluidsurfacereconstructiongpu_gb300 import _native as N
    f = N.lib.fsr_spatial_hash_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(N.FrameHeader), ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
    return N, f


def _frame(n_side, seed, origin):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    return synthetic.lattice_cube(n_side, 0.0125, seed=seed, origin=origin)


def _existing(fr):
    """Sorted order, ranges and sorted data from the allocating path."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    rec = api.Reconstructor("zb05", 0, keep_intermediates=True)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    out = rec.debug("perm"), rec.debug("ranges"), rec.debug("sorted_xyz")
    rec.close()
    return out


def _noalloc(N, f, fr, cell_capacity):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    n = fr.n
    xyz = torch.from_numpy(fr.pos).cuda()
    den = torch.from_numpy(fr.density).cuda()
    out_xyz = torch.full((n, 3), -1.0, device="cuda")
    out_den = torch.full((n,), -1.0, device="cuda")
    ranges = torch.zeros((cell_capacity, 2), dtype=torch.int32, device="cuda")
    perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    oog = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    ncells = ctypes.c_uint64(0)
    stream = torch.cuda.current_stream()
    st = f(ctypes.byref(api.header_of(fr)), ctypes.c_float(1.0), xyz.data_ptr(), den.data_ptr(), n,
           out_xyz.data_ptr(), out_den.data_ptr(), ranges.data_ptr(), cell_capacity, perm.data_ptr(),
           oog.data_ptr(), ctypes.byref(ncells), ctypes.c_void_p(stream.cuda_stream))
    assert st == N.FSR_OK, N.STATUS_NAMES.get(st, st)
    torch.cuda.synchronize()
    c = int(ncells.value)
    return (perm.cpu().numpy().view(np.uint32), ranges[:c].cpu().numpy().view(np.uint32),
            out_xyz.cpu().numpy(), out_den.cpu().numpy(), int(oog.item()))


def test_noalloc_matches_allocating_path_on_consecutive_calls():
    N, f = _bind()
    big = _frame(40, seed=3, origin=(0.2, 0.25, 0.3))     # 64,000 particles
    small = _frame(23, seed=9, origin=(0.4, 0.35, 0.3))   # 12,167 particles
    assert big.n <= 1 << 18
    cap = 64 ** 3
    for fr in (big, small, big):
        perm_e, ranges_e, xyz_e = _existing(fr)
        perm, ranges, xyz, den, oog = _noalloc(N, f, fr, cap)
        assert oog == 0
        assert np.array_equal(perm, perm_e)
        assert np.array_equal(ranges, ranges_e)
        assert np.array_equal(xyz, xyz_e)
        assert np.array_equal(den, fr.density[perm_e])


def test_noalloc_rejects_oversize_and_small_range_buffers():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    N, f = _bind()
    fr = _frame(8, seed=1, origin=(0.3, 0.3, 0.3))
    ncells = ctypes.c_uint64(0)
    hdr = api.header_of(fr)
    st = f(ctypes.byref(hdr), ctypes.c_float(1.0), None, None, (1 << 18) + 1, None, None, None, 0, None, None,
           ctypes.byref(ncells), None)
    assert st == 8  # FSR_ERR_TOO_LARGE
    x = torch.from_numpy(fr.pos).cuda()
    d = torch.from_numpy(fr.density).cuda()
    st = f(ctypes.byref(hdr), ctypes.c_float(1.0), x.data_ptr(), d.data_ptr(), fr.n, x.data_ptr(), d.data_ptr(),
           x.data_ptr(), 1, None, None, ctypes.byref(ncells), None)
    assert st == 7 and ncells.value > 1  # FSR_ERR_CAPACITY, nothing written


def _call(N, f, fr, pos, cap, with_optional=True):
    """One call on the given positions; returns status, n_cells, perm, ranges,
    sorted xyz and the out-of-grid count (None when not requested)."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    n = pos.shape[0]
    xyz = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    den = torch.full((n,), 1000.0, device="cuda")
    out_xyz = torch.full((max(n, 1), 3), -1.0, device="cuda")
    out_den = torch.full((max(n, 1),), -1.0, device="cuda")
    ranges = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    oog = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    ncells = ctypes.c_uint64(0)
    st = f(ctypes.byref(api.header_of(fr)), ctypes.c_float(1.0), xyz.data_ptr() if n else None,
           den.data_ptr() if n else None, n, out_xyz.data_ptr() if n else None, out_den.data_ptr() if n else None,
           ranges.data_ptr(), cap, perm.data_ptr() if with_optional else None,
           oog.data_ptr() if with_optional else None, ctypes.byref(ncells),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    c = int(ncells.value)
    return (st, c, perm[:n].cpu().numpy().view(np.uint32), ranges[:c].cpu().numpy().view(np.uint32),
            out_xyz[:n].cpu().numpy(), int(oog.item()) if with_optional else None)


def test_noalloc_edge_cases():
    """n = 0 and n = 1, a particle outside the grid (counted, no write out of
    bounds: it is hashed to cell 0) and null optional outputs."""
    N, f = _bind()
    fr = _frame(8, seed=1, origin=(0.3, 0.3, 0.3))
    cap = 64 ** 3
    st, c, _, ranges, _, oog = _call(N, f, fr, np.zeros((0, 3), np.float32), cap)
    assert st == N.FSR_OK and c > 0 and oog == 0
    assert np.all(ranges == 0xFFFFFFFF)
    one = fr.pos[5:6]
    st, c, perm, ranges, xyz, oog = _call(N, f, fr, one, cap)
    assert st == N.FSR_OK and oog == 0 and perm.tolist() == [0]
    assert np.array_equal(xyz, one)
    nonempty = np.flatnonzero(ranges[:, 0] != 0xFFFFFFFF)
    assert nonempty.size == 1 and ranges[nonempty[0]].tolist() == [0, 1]
    pos = fr.pos.copy()
    pos[3] = [5.0, 0.5, 0.5]
    st, _, perm, ranges, _, oog = _call(N, f, fr, pos, cap)
    assert st == N.FSR_OK and oog == 1
    assert sorted(perm.tolist()) == list(range(fr.n))
    # without the optional outputs the sorted particles and ranges are the same
    st1, _, _, r1, x1, _ = _call(N, f, fr, fr.pos, cap)
    st2, _, _, r2, x2, none = _call(N, f, fr, fr.pos, cap, with_optional=False)
    assert st1 == st2 == N.FSR_OK and none is None
    assert np.array_equal(r1, r2) and np.array_equal(x1, x2)
