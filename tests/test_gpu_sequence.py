"""Pipelined frame sequences (fsr_reconstruct_host_frames) against the
single-call host path.

The sequence overlaps each frame's upload and read-back with its
neighbours' kernels; every frame must still give exactly the results of
fsr_reconstruct_host on the same particles (the same kernels on the same
inputs): mesh positions and normals bit for bit, per-frame statuses, the
capacity-overflow re-run, and the handle holding the last frame afterwards.
The single-frame path itself is checked against the oracle in the parity
tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames(seed, sizes):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    return [synthetic.lattice_count(n, seed=seed + i) for i, n in enumerate(sizes)]


def _host(method, fr, **kw):
    from fluidsurfacereconstructiongpu_gb300 import api
    rec = api.Reconstructor(method, 0, **kw)
    m = rec.reconstruct_host(fr.pos, fr.density, api.header_of(fr))  # sized by the call itself
    rec.close()
    return m


@pytest.mark.parametrize("method", ["yu13", "zb05", "akinci12"])
def test_sequence_matches_single_calls(method):
    from fluidsurfacereconstructiongpu_gb300 import api
    frames = _frames(21, [3000, 17000, 6000, 30000, 9000])
    rec = api.Reconstructor(method, 0)
    meshes = rec.reconstruct_host_frames([(fr.pos, fr.density, api.header_of(fr)) for fr in frames])
    for i, fr in enumerate(frames):
        ref = _host(method, fr)
        assert meshes[i].positions.shape[0] > 0, i
        assert np.array_equal(meshes[i].positions, ref.positions), (method, i)
        assert np.array_equal(meshes[i].normals, ref.normals), (method, i)
    # the handle holds the last frame
    last = rec.mesh()
    assert rec.stats().n_particles == frames[-1].n
    assert np.array_equal(last.positions, meshes[-1].positions)
    # a second call on the same handle (its buffers and events are reused)
    again = rec.reconstruct_host_frames([(fr.pos, fr.density, api.header_of(fr)) for fr in frames[::-1]])
    for a, b in zip(again, meshes[::-1]):
        assert np.array_equal(a.positions, b.positions)
    rec.close()


def test_sequence_overflow_rerun_and_capacity_status():
    """A handle sized by a small first frame meets a much larger one: its band
    overflows, the frame is re-run inside the sequence, and the frames around
    it are unaffected.  One frame's output buffer is too small: that frame
    gets FSR_ERR_CAPACITY and the others still complete."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, _native as N
    frames = _frames(40, [2000, 2500, 260000, 4000, 3000])
    kw = dict(grid_ratio=10)  # the 260k frame's band (millions of vertices) overflows the first frame's sizing
    refs = [_host("yu13", fr, **kw) for fr in frames]
    rec = api.Reconstructor("yu13", 0, **kw)
    arr = (N.HostFrame * len(frames))()
    keep = []
    for k, fr in enumerate(frames):
        xyz = torch.from_numpy(fr.pos).pin_memory()
        den = torch.from_numpy(fr.density).pin_memory()
        cap = 16 if k == 3 else refs[k].positions.shape[0] + 16
        pos = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
        nrm = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
        keep.append((xyz, den, pos, nrm))
        arr[k].header = api.header_of(fr)
        arr[k].xyz, arr[k].density, arr[k].n = xyz.data_ptr(), den.data_ptr(), fr.n
        arr[k].out_pos, arr[k].out_nrm, arr[k].capacity = pos.data_ptr(), nrm.data_ptr(), cap
    st = N.lib.fsr_reconstruct_host_frames(rec._h, arr, len(frames), None)
    assert st == 7  # FSR_ERR_CAPACITY, from frame 3
    assert [arr[k].status for k in range(len(frames))] == [0, 0, 0, 7, 0]
    assert rec.stats().n_retries >= 1
    for k, fr in enumerate(frames):
        ref = refs[k]
        assert arr[k].n_vertices == ref.positions.shape[0], k
        if k == 3:
            continue
        nv = arr[k].n_vertices
        assert np.array_equal(keep[k][2][:nv].numpy(), ref.positions), k
        assert np.array_equal(keep[k][3][:nv].numpy(), ref.normals), k
    assert rec.stats().n_particles == frames[-1].n
    rec.close()


def test_sequence_edge_counts():
    from fluidsurfacereconstructiongpu_gb300 import api, _native as N
    rec = api.Reconstructor("zb05", 0)
    assert N.lib.fsr_reconstruct_host_frames(rec._h, None, 0, None) == 0
    assert N.lib.fsr_reconstruct_host_frames(rec._h, None, 2, None) == 1  # null frames
    arr = (N.HostFrame * 1)()
    arr[0].n = 10  # null particle arrays
    assert N.lib.fsr_reconstruct_host_frames(rec._h, arr, 1, None) == 1
    assert arr[0].status == 1
    fr = _frames(7, [5000])[0]
    one = rec.reconstruct_host_frames([(fr.pos, fr.density, api.header_of(fr))])
    ref = _host("zb05", fr)
    assert np.array_equal(one[0].positions, ref.positions)
    rec.close()
