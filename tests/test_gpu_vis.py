"""The .vis debug dump (fsr_write_vis) against the reference's layout filled
with the oracle's frame.

The expected file is written here the way saveMiddleDataToVisFile writes it
(ReconstructorGPUOursZB05.cpp:104-230, ReconstructorGPUOursYu13.cpp:285-420,
ReconstructorGPUAkinci12.cpp:290-420: std::ostream, %g floats, lists as
"count" then "i " per entry), from the FP32 oracle's arrays; the GPU's file
must match it byte for byte.  The one exception is the anisotropic path's
smoothed positions: the library forms them from a compensated mean (they
are within 1e-7 of FP64, the reference's FP32 ones are not), so that block
is written from the frame's own smoothed positions, which are checked
against the FP64 oracle within the parity bar (1e-6).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _g(x) -> str:
    return "%g" % float(np.float32(x))


def _expected(o, fr, mesh_name, smoothed=None):
    sp, sc = o.spatial, o.scalar
    out = []
    for g in (sp, sc):
        out.append(" ".join(_g(v) for v in g.minPos) + "\n")
        out.append(" ".join(_g(v) for v in g.maxPos) + "\n")
        out.append(" ".join("%d" % v for v in g.res) + "\n")
        out.append(_g(g.cellSize) + "\n")
    out.append(_g(fr.particle_radius) + "\n")
    n = o.pos.shape[0]
    out.append("%d\n" % n)
    out += ["%s %s %s\n" % (_g(p[0]), _g(p[1]), _g(p[2])) for p in o.pos]

    def lst(v, brk_if_empty=False):
        s = "%d\n" % len(v) + "".join("%d " % x for x in v)
        return s + ("\n" if len(v) or brk_if_empty else "")

    out.append(lst(np.flatnonzero(o.flag > 0), o.flag.size > 0))
    if o.method == "yu13":
        out.append("%d\n" % n)
        out += ["%s %s %s\n" % (_g(p[0]), _g(p[1]), _g(p[2])) for p in (o.smoothed if smoothed is None else smoothed)]
    else:
        out.append("0\n")
    out.append(lst(o.sv))
    out.append(lst(np.flatnonzero(o.sflag == 1)))
    if o.method == "yu13":
        inv_cells = o.ninv > 0
        keys = o.keys[o.perm]  # sorted cell ids
        out.append(lst(np.flatnonzero(inv_cells[keys])))
    else:
        out.append("0\n")
    out.append(lst(o.valid_idx))
    out.append(mesh_name + "\n")
    out.append(_g(fr.h) + "\n")
    return "".join(out).encode()


@pytest.mark.parametrize("method", ["zb05", "tc01", "yu13", "akinci12"])
def test_vis_matches_reference_layout(tmp_path, method):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    from oracle import pipeline as P
    fr = synthetic.lattice_cube(12, 0.0125, seed=3, origin=(0.3, 0.3, 0.3))
    rec = api.Reconstructor(method, 0, keep_intermediates=True)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    path = tmp_path / "frame_000.vis"
    rec.write_vis(str(path), "frame_000.obj")
    smoothed = rec.debug("smoothed") if method == "yu13" else None
    rec.close()
    p = api.default_params(method)
    params = P.FrameParams(method="akinci" if method == "akinci12" else method, h=fr.h,
                           particle_radius=fr.particle_radius, mass=fr.mass, iso=p.iso_value, ratio=p.grid_ratio, cell_scale=p.cell_size_scale,
                           lam=p.smoothing_lambda, aniso_radius=p.aniso_radius_over_h * fr.h,
                           min_neighbors=p.min_neighbors)
    o = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    if smoothed is not None:
        o64 = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
        assert np.abs(smoothed - o64.smoothed).max() <= 1e-6
    want = _expected(o, fr, "frame_000.obj", smoothed)
    got = path.read_bytes()
    if got != want:
        a, b = got.split(b"\n"), want.split(b"\n")
        k = next((i for i in range(min(len(a), len(b))) if a[i] != b[i]), min(len(a), len(b)))
        raise AssertionError((method, k, a[k][:120] if k < len(a) else None, b[k][:120] if k < len(b) else None))


def test_files_loop_writes_vis(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    fr = synthetic.lattice_cube(10, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    api.write_xyz(str(tmp_path / "s_004.xyz"), fr)
    r = api.ReconstructorGPUOursYu13(str(tmp_path) + "/", "s_%03d", 4, 5)
    r.setOutputVisualizeFile(True)
    r.reconstruct()
    lines = (tmp_path / "s_004.vis").read_text().splitlines()
    assert lines[-2] == "s_004.obj"
    assert lines[9] == "%d" % fr.n
