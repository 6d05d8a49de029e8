"""GPU pipeline vs CPU oracle, through the C ABI (libfsr_gb300.so).

Each case runs one frame on cuda:0 with intermediates kept, then compares
every stage with the FP32 oracle (integers bit-exact) and the FP64 oracle
(field, G, mesh vertices within tolerance); see tests/parity.py.
"""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


def _run(method, fr, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P
    from tests.parity import compare_frame

    params = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass,
                           iso=kw.get("iso"), ratio=kw.get("grid_ratio"), cell_scale=kw.get("cell_size_scale"),
                           lam=kw.get("smoothing_lambda", 0.5),
                           aniso_radius=(kw["aniso_radius_over_h"] * fr.h if "aniso_radius_over_h" in kw else None))
    rec = api.Reconstructor(method, 0, keep_intermediates=True, **kw)
    xyz = torch.from_numpy(np.ascontiguousarray(fr.pos)).cuda()
    den = torch.from_numpy(np.ascontiguousarray(fr.density)).cuda()
    rec.reconstruct(xyz, den, api.header_of(fr))
    o32 = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    o64 = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    rep = compare_frame(rec, o32, o64, method, fr.h)
    rec.close()
    return rep


def _lattice(n, seed=1, origin=(0.3, 0.3, 0.3), r=0.0125):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    return synthetic.lattice_cube(n, r, seed=seed, origin=origin)


@pytest.mark.parametrize("method", ["zb05", "tc01", "akinci", "yu13"])
def test_small_lattice_reference_defaults(method):
    rep = _run(method, _lattice(12))
    assert rep["triangles"] > 0


def test_zb05_plain_small_workload():
    """32^3 lattice, spacing r, h = 4r, grid spacing 0.5r (ratio 8), reference iso."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.lattice_cube(32, 0.0125, seed=1)
    rep = _run("zb05", fr, grid_ratio=8)
    assert rep["triangles"] > 1000


def test_yu13_medium():
    rep = _run("yu13", _lattice(20, seed=7, origin=(0.25, 0.3, 0.2)))
    assert rep["triangles"] > 0


def test_yu13_dam_break_workload_parameters():
    """Small dam-break frame with the anisotropic workload's settings:
    lambda 0.9, neighbour radius 4r (= h), cell 1.25h, grid spacing 0.5r."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.dam_break(n_total=20000, r=0.012, seed=5)
    rep = _run("yu13", fr, smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10)
    assert rep["triangles"] > 0


@pytest.mark.parametrize("method", ["zb05", "yu13", "akinci"])
def test_format_example(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    _run(method, synthetic.format_example())


def test_single_cell_crowd():
    """Every particle in one spatial cell: stresses the stable radix sort."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    rng = np.random.default_rng(11)
    fr = _lattice(4)
    fr.pos = (0.5 + rng.uniform(0, 0.04, size=(5000, 3))).astype(np.float32)
    fr.density = np.full(5000, 1000.0, np.float32)
    _run("zb05", fr)


def test_empty_frame():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    fr = _lattice(4)
    rec = api.Reconstructor("zb05", 0)
    nv = rec.reconstruct(torch.zeros((0, 3), device="cuda"), torch.zeros(0, device="cuda"), api.header_of(fr))
    assert nv == 0
    rec.close()


def test_particle_outside_grid_is_an_error():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, _native
    fr = _lattice(6)
    pos = fr.pos.copy()
    pos[3] = [5.0, 0.5, 0.5]
    rec = api.Reconstructor("zb05", 0)
    with pytest.raises(_native.FsrError) as ei:
        rec.reconstruct(torch.from_numpy(pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    assert ei.value.status == 2
    # the handle stays usable
    nv = rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    assert nv > 0
    rec.close()


def test_host_path_matches_device_path():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    fr = _lattice(10)
    rec = api.Reconstructor("zb05", 0)
    m1 = rec.reconstruct_host(fr.pos, fr.density, api.header_of(fr))
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    m2 = rec.mesh()
    assert np.array_equal(m1.positions, m2.positions) and np.array_equal(m1.normals, m2.normals)
    rec.close()


def test_zb05_plain_small_workload_baseline_iso():
    """The same 32^3 lattice with the iso value 0.5 that the benchmark's
    configuration names.  ZB05's field is a distance minus the particle
    radius, which on the narrow band (within 1.5h of the surface particles)
    never reaches 0.5, so the frame has no valid cube and no triangle; every
    stage still matches the oracle."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.lattice_cube(32, 0.0125, seed=1)
    rep = _run("zb05", fr, grid_ratio=8, iso=0.5)
    assert rep["triangles"] == 0



def _translated(fr, offset):
    o = np.float32(offset)
    fr.pos = (fr.pos + o).astype(np.float32)
    fr.bbox_min = (fr.bbox_min + o).astype(np.float32)
    fr.bbox_max = (fr.bbox_max + o).astype(np.float32)
    return fr


def _run_exact(method, fr, **kw):
    """One frame against the FP32 oracle on the stages that are bit-exact by
    construction: sort order, cell ranges, sorted positions, surface flags,
    involved counts and FP32 means (Yu13), band vertices.  (The FP64 checks of
    compare_frame use absolute tolerances scaled for coordinates of order 1.)
    Returns the number of band vertices."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P

    params = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass,
                           iso=kw.get("iso"), ratio=kw.get("grid_ratio"), cell_scale=kw.get("cell_size_scale"),
                           lam=kw.get("smoothing_lambda", 0.5),
                           aniso_radius=(kw["aniso_radius_over_h"] * fr.h if "aniso_radius_over_h" in kw else None))
    rec = api.Reconstructor(method, 0, keep_intermediates=True, **kw)
    rec.reconstruct(torch.from_numpy(np.ascontiguousarray(fr.pos)).cuda(),
                    torch.from_numpy(np.ascontiguousarray(fr.density)).cuda(), api.header_of(fr))
    o32 = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    assert np.array_equal(rec.debug("perm"), o32.perm), "stable sort order differs"
    assert np.array_equal(rec.debug("ranges"), o32.ranges), "cell ranges differ"
    assert np.array_equal(rec.debug("sorted_xyz"), o32.pos), "sorted positions differ"
    assert np.array_equal(rec.debug("surface_flags"), o32.sflag), "surface particle flags differ"
    if method == "yu13":
        assert np.array_equal(rec.debug("involved_counts"), o32.ninv), "involved counts differ"
        assert np.array_equal(rec.debug("mean"), o32.mean32), "weighted means differ"
    sv = rec.debug("band")
    assert np.array_equal(sv, o32.sv), "band vertices differ"
    rec.close()
    return int(sv.size)


def test_yu13_frame_away_from_the_origin():
    """The dam-break settings of test_yu13_dam_break_workload_parameters with
    the frame moved by +10 on each axis (about 170 cells from the origin):
    the warp culls of the smoothing and covariance kernels, whose margins
    grow with the coordinates' magnitude, still keep every neighbour, so the
    FP32 means, counts and band equal the oracle's bit for bit."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = _translated(synthetic.dam_break(n_total=20000, r=0.012, seed=5), 10.0)
    nb = _run_exact("yu13", fr, smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10)
    assert nb > 0


def test_akinci_frame_away_from_the_origin():
    """A lattice moved by +10 on each axis through the colour field's warp
    culls: surface flags and band bit for bit."""
    assert _run_exact("akinci", _translated(_lattice(12), 10.0)) > 0
