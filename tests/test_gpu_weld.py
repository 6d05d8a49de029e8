"""Vertex welding (FSR_FLAG_WELD): the triangle soup as an indexed mesh.

The soup is the reference's (generateTriangles, ReconstructionCUDA.cu:
383-463: three unshared vertices per triangle, each on a scalar-grid edge).
Checked here, per field method:
* every soup vertex's edge key names a grid edge that the vertex lies on (two
  coordinates are the FP32 grid coordinates of the edge's lower end point,
  the third lies between its end points);
* the indices equal the host's numbering of the keys by first use, exactly;
* welded vertices are the first copies, bit for bit, and every other copy is
  within a few ulps of it (the cubes sharing an edge interpolate it from
  opposite ends);
* welding leaves the soup unchanged and runs deterministically;
* the indexed .obj has one v/vn line per welded vertex and the soup's faces.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "zb05": dict(),
    "tc01": dict(),
    "akinci12": dict(),
    "yu13": dict(smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0),
}


def _run(method, fr, weld, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    rec = api.Reconstructor(method, 0, weld=weld, **kw)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    out = dict(soup=rec.mesh(), stats=rec.stats())
    if weld:
        out["im"] = rec.indexed_mesh()
        out["keys"] = rec.debug("weld_keys")
    rec.close()
    return out


def _scalar_grid(method, fr, kw):
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P
    p = api.default_params(method)
    scale = kw.get("cell_size_scale", p.cell_size_scale)
    ratio = kw.get("grid_ratio", p.grid_ratio)
    _, sc = P.grid_derive(fr.bbox_min, fr.bbox_max, fr.h, scale, ratio)
    return np.array(sc.minPos, np.float32), np.float32(sc.cellSize), np.array(sc.res, np.int64)


@pytest.mark.parametrize("method", sorted(CASES))
def test_weld_matches_edge_numbering(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    kw = CASES[method]
    fr = synthetic.lattice_cube(14, 0.0125, seed=7, origin=(0.3, 0.3, 0.3))
    a = _run(method, fr, True, **kw)
    soup, im, keys = a["soup"], a["im"], a["keys"]
    n = soup.positions.shape[0]
    assert n > 0 and keys.shape == (n,) and im.triangles.shape == (n // 3, 3)
    assert a["stats"].n_weld_vertices == im.positions.shape[0]

    # keys name edges the vertices lie on
    mn, cs, res = _scalar_grid(method, fr, kw)
    axis = (keys % 3).astype(np.int64)
    lin = (keys // 3).astype(np.int64)
    lo = np.stack([lin % res[0], (lin // res[0]) % res[1], lin // (res[0] * res[1])], axis=1)
    glo = (lo.astype(np.float32) * cs).astype(np.float32) + mn          # getVertexPos in FP32
    ghi = ((lo + 1).astype(np.float32) * cs).astype(np.float32) + mn
    p = soup.positions
    for ax in range(3):
        on = axis == ax
        off = ~on
        assert np.array_equal(p[off, ax], glo[off, ax]), method
        assert np.all((p[on, ax] >= glo[on, ax]) & (p[on, ax] <= ghi[on, ax])), method

    # numbering by first use
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    rank = np.empty(uniq.size, np.int64)
    rank[np.argsort(first)] = np.arange(uniq.size)
    want_idx = rank[inv.reshape(-1)]
    assert np.array_equal(im.triangles.reshape(-1).astype(np.int64), want_idx)
    order = np.sort(first)
    assert np.array_equal(im.positions.view(np.uint32), soup.positions[order].view(np.uint32))
    assert np.array_equal(im.normals.view(np.uint32), soup.normals[order].view(np.uint32))

    # other copies of a vertex differ from the first by a few ulps at most
    diff = np.abs(im.positions[want_idx] - p)
    assert np.all(diff <= 4 * np.spacing(np.maximum(np.abs(p), np.float32(1e-3)))), (method, diff.max())
    # a closed surface shares each vertex among several triangles
    assert im.positions.shape[0] < 0.35 * n, (method, im.positions.shape[0], n)


def test_weld_leaves_the_soup_alone_and_is_deterministic():
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.dam_break(40000, r=0.004, seed=5)
    kw = CASES["yu13"]
    a = _run("yu13", fr, True, **kw)
    b = _run("yu13", fr, True, **kw)
    c = _run("yu13", fr, False, **kw)
    # bitwise: normals next to the anisotropic fill value can be NaN
    assert np.array_equal(a["soup"].positions.view(np.uint32), c["soup"].positions.view(np.uint32))
    assert np.array_equal(a["soup"].normals.view(np.uint32), c["soup"].normals.view(np.uint32))
    assert np.array_equal(a["im"].triangles, b["im"].triangles)
    assert np.array_equal(a["im"].positions.view(np.uint32), b["im"].positions.view(np.uint32))
    assert np.array_equal(a["im"].normals.view(np.uint32), b["im"].normals.view(np.uint32))
    assert c["stats"].n_weld_vertices == 0


def test_indexed_obj(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    fr = synthetic.lattice_cube(12, 0.0125, seed=2, origin=(0.3, 0.3, 0.3))
    a = _run("zb05", fr, True)
    im = a["im"]
    path = tmp_path / "w.obj"
    api.write_obj(str(path), im)
    lines = path.read_text().splitlines()
    nv, nt = im.positions.shape[0], im.triangles.shape[0]
    assert len(lines) == 2 * nv + nt
    assert all(l.startswith("v ") for l in lines[:nv]) and all(l.startswith("vn ") for l in lines[nv:2 * nv])
    faces = np.array([[int(t.split("//")[0]) for t in l[2:].split()] for l in lines[2 * nv:]])
    assert np.array_equal(faces - 1, im.triangles.astype(np.int64))
    v = np.array([[float(x) for x in l.split()[1:]] for l in lines[:nv]])
    assert np.allclose(v, im.positions, rtol=1e-5, atol=1e-6)


def test_files_loop_writes_indexed_obj(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    fr = synthetic.lattice_cube(12, 0.0125, seed=2, origin=(0.3, 0.3, 0.3))
    api.write_xyz(str(tmp_path / "f_000.xyz"), fr)
    r = api.ReconstructorGPUOursZB05(str(tmp_path) + "/", "f_%03d", 0, 1)
    r.setOutputMeshFile(True)
    r.setIndexedMesh(True)
    r.reconstruct()
    got = (tmp_path / "f_000.obj").read_bytes()
    hdr, xyz, den = api.read_xyz(str(tmp_path / "f_000.xyz"))
    import torch
    rec = api.Reconstructor("zb05", 0, weld=True)
    rec.reconstruct(torch.from_numpy(xyz).cuda(), torch.from_numpy(den).cuda(), hdr)
    api.write_obj(str(tmp_path / "want.obj"), rec.indexed_mesh())
    rec.close()
    assert got == (tmp_path / "want.obj").read_bytes()
