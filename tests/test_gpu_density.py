"""Densities computed on the GPU (FSR_FLAG_COMPUTE_DENSITY) for frames
without a density column.  The reference has no such pass (its .xyz files
carry the simulator's densities); the checker is an FP64 all-pairs SPH sum
with the reference field kernel's normalisation (oracle.pipeline.sph_density).
FP32 tolerance: 1e-5 relative per particle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(method, fr, compute, dens=None, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    rec = api.Reconstructor(method, 0, compute_density=compute, **kw)
    d = None if dens is None else torch.from_numpy(np.ascontiguousarray(dens, np.float32)).cuda()
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), d, api.header_of(fr))
    out = dict(mesh=rec.mesh(), density=rec.debug("density"), perm=rec.debug("perm"),
               sorted=rec.debug("sorted_xyz"), rec=rec)
    return out


@pytest.mark.parametrize("method", ["zb05", "yu13", "akinci12"])
def test_density_matches_fp64(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    from oracle import pipeline as P
    fr = synthetic.dam_break(6000, r=0.01, seed=3)
    a = _run(method, fr, True)
    a["rec"].close()
    want = P.sph_density(a["sorted"], fr.h, fr.mass)
    got = a["density"].astype(np.float64)
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() <= 1e-5, rel.max()
    # the interior of the column is near the rest density the mass was set for
    assert 0.8 * 1000 < np.median(got) < 1.2 * 1000, np.median(got)


def test_frame_with_computed_densities_equals_frame_fed_them():
    """A frame that computes its densities gives the mesh of a frame given
    those densities as input (bit for bit)."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    kw = dict(smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0)
    fr = synthetic.dam_break(30000, r=0.004, seed=8)
    a = _run("yu13", fr, True, **kw)
    a["rec"].close()
    dens_in = np.empty(fr.n, np.float32)
    dens_in[a["perm"]] = a["density"]
    b = _run("yu13", fr, False, dens=dens_in, **kw)
    b["rec"].close()
    assert a["mesh"].positions.shape[0] > 0
    assert np.array_equal(a["mesh"].positions.view(np.uint32), b["mesh"].positions.view(np.uint32))
    assert np.array_equal(a["mesh"].normals.view(np.uint32), b["mesh"].normals.view(np.uint32))


def test_density_argument_rules():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic, _native
    fr = synthetic.lattice_cube(8, 0.0125, seed=1)
    rec = api.Reconstructor("zb05", 0)
    with pytest.raises(_native.FsrError) as e:
        rec.reconstruct(torch.from_numpy(fr.pos).cuda(), None, api.header_of(fr))
    assert e.value.status == 1
    rec.close()
    a = _run("zb05", fr, True)
    with pytest.raises(_native.FsrError) as e:
        a["rec"].backward(torch.zeros((a["mesh"].positions.shape[0], 3), device="cuda"))
    assert e.value.status == 1
    a["rec"].close()
