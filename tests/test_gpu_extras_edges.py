"""Edge cases of the welding, density, .vis and file-loop additions: empty
frames, pool growth with welding on, and an error in the middle of a
pipelined file run."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _empty(method, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    fr = synthetic.lattice_cube(8, 0.0125, seed=1)
    rec = api.Reconstructor(method, 0, **kw)
    nv = rec.reconstruct(torch.zeros((0, 3), device="cuda"),
                         None if kw.get("compute_density") else torch.zeros(0, device="cuda"), api.header_of(fr))
    return rec, nv


def test_empty_frame_with_weld_density_and_vis(tmp_path):
    rec, nv = _empty("yu13", weld=True, compute_density=True)
    assert nv == 0
    im = rec.indexed_mesh()
    assert im.positions.shape == (0, 3) and im.triangles.shape == (0, 3)
    assert rec.debug("density").shape == (0,)
    rec.write_vis(str(tmp_path / "e.vis"), "e.obj")
    lines = (tmp_path / "e.vis").read_text().splitlines()
    assert lines[9] == "0" and lines[-2] == "e.obj"
    rec.close()


def test_weld_after_pool_growth():
    """With small pools the first attempt overflows the mesh pool and the
    frame re-runs; the welded mesh still numbers the final soup's edges."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic, _native as N
    fr = synthetic.dam_break(30000, r=0.004, seed=6)
    rec = api.Reconstructor("zb05", 0, weld=True)
    rec.params.flags |= N.FLAG_SMALL_POOLS
    N.check(N.lib.fsr_set_params(rec._h, rec.params), rec._h)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    st = rec.stats()
    assert st.n_retries > 0
    soup, im, keys = rec.mesh(), rec.indexed_mesh(), rec.debug("weld_keys")
    rec.close()
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    rank = np.empty(uniq.size, np.int64)
    rank[np.argsort(first)] = np.arange(uniq.size)
    assert np.array_equal(im.triangles.reshape(-1).astype(np.int64), rank[inv.reshape(-1)])
    assert np.array_equal(im.positions.view(np.uint32), soup.positions[np.sort(first)].view(np.uint32))


def test_file_loop_stops_at_a_missing_frame(tmp_path):
    """Frame 1 of 0..2 is missing: the run reports the I/O error after
    writing frame 0's mesh, and the read-ahead of frame 2 does not leak or
    hang."""
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic, _native
    for k in (0, 2):
        api.write_xyz(str(tmp_path / f"m_{k:03d}.xyz"), synthetic.lattice_cube(9, 0.0125, seed=k))
    r = api.ReconstructorGPUOursZB05(str(tmp_path) + "/", "m_%03d", 0, 3)
    r.setOutputMeshFile(True)
    r.setBinarySidecar(True)
    with pytest.raises(_native.FsrError) as e:
        r.reconstruct()
    assert e.value.status == 5 and "m_001.xyz" in str(e.value)
    assert (tmp_path / "m_000.obj").stat().st_size > 0
    assert not (tmp_path / "m_002.obj").exists()
    # the sidecar of frame 0 was written; frame 2's read-ahead may have made its own
    assert (tmp_path / "m_000.xyzb").exists()
    assert not any(f.endswith(".tmp") for f in os.listdir(tmp_path))
