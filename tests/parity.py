"""Shared GPU-vs-oracle comparison used by the parity tests and bench checks.

Integer results (sort order, cell ranges, surface flags, involved counts,
band vertices, MC cases, valid cubes, triangle counts) must equal the FP32
oracle's.  The only exemption: marching-cubes cubes with a corner whose FP64
field value lies within NEAR_ISO of the iso value, where a last-bit
difference in summation order may legitimately flip the case; such cubes are
counted and reported.  Field values, G matrices and mesh vertices are
compared with the FP64 oracle within the stated tolerances.
"""
from __future__ import annotations

import numpy as np

NEAR_ISO = 1e-6
# interpolated normals shorter than this before normalisation (the two
# corner normals nearly cancel) have ill-conditioned directions
NORMAL_MIN_LEN = 1e-2


def field_tolerance(method: str, h: float, phi64: np.ndarray) -> np.ndarray:
    """Absolute tolerance per band vertex: 1e-5 relative of the field's scale.
    ZB05 is a distance (scale h); TC01 and the anisotropic field are sums of
    O(1) kernel values (scale max(1, |phi|))."""
    if method in ("zb05", "akinci"):
        return 1e-5 * np.maximum(h, np.abs(phi64))  # a distance: relative to h
    return 1e-5 * np.maximum(1.0, np.abs(phi64))


def corner_ids(cubes: np.ndarray, res) -> np.ndarray:
    rx, ry = res[0], res[0] * res[1]
    off = np.array([0, rx * ry, rx * ry + rx, rx, 1, 1 + rx * ry, 1 + rx + rx * ry, 1 + rx], dtype=np.int64)
    # corner order of ReconstructionCUDA.cuh:441-452, (dx, dy, dz) per corner
    dx = np.array([0, 0, 0, 0, 1, 1, 1, 1])
    dy = np.array([0, 0, 1, 1, 0, 0, 1, 1])
    dz = np.array([0, 1, 1, 0, 0, 1, 1, 0])
    off = dx + dy * rx + dz * ry
    return cubes.astype(np.int64)[:, None] + off[None, :]


def compare_frame(rec, o32, o64, method: str, h: float) -> dict:
    """rec: api.Reconstructor after a frame with keep_intermediates=True."""
    rep = {}
    assert np.array_equal(rec.debug("perm"), o32.perm), "stable sort order differs"
    assert np.array_equal(rec.debug("ranges"), o32.ranges), "cell ranges differ"
    assert np.array_equal(rec.debug("sorted_xyz"), o32.pos), "sorted positions differ"
    assert np.array_equal(rec.debug("surface_flags"), o32.sflag), "surface particle flags differ"
    if method == "yu13":
        assert np.array_equal(rec.debug("involved_counts"), o32.ninv), "involved counts differ"
        assert np.array_equal(rec.debug("mean"), o32.mean32), "weighted means differ"
        sm = rec.debug("smoothed")
        assert np.allclose(sm, o64.smoothed, rtol=0, atol=1e-6), "smoothed positions"
        G = rec.debug("G")[o32.inv]
        G64 = o64.G
        rel = np.linalg.norm(G - G64, axis=1) / np.linalg.norm(G64, axis=1)
        rep["G_rel_max"] = float(rel.max()) if rel.size else 0.0
        assert rep["G_rel_max"] <= 1e-5, f"G relative error {rep['G_rel_max']:.3e}"
    sv = rec.debug("band")
    assert np.array_equal(sv, o32.sv), "band vertices differ"
    phi = rec.debug("field").astype(np.float64)
    phi64 = o64.phi[o64.sv]
    tol = field_tolerance(method, h, phi64)
    err = np.abs(phi - phi64)
    rep["field_abs_max"] = float(err.max()) if err.size else 0.0
    rep["field_viol"] = int((err > tol).sum())
    assert rep["field_viol"] == 0, f"{rep['field_viol']} field values beyond tolerance (max {err.max():.3e})"

    # marching cubes, end to end: integers equal the FP32 oracle's except in
    # cubes touching a near-iso corner
    info = rec.debug("mc_info")
    gcase, gnv, gvalid = info & 0xFF, (info >> 8) & 0xFF, (info >> 16) & 1
    ovalid = o32.valid.astype(np.uint32)
    res = o32.scalar.resolution
    V = o32.scalar.count
    x = sv % res[0]
    y = (sv // res[0]) % res[1]
    z = sv // (res[0] * res[1])
    inner = (x < res[0] - 1) & (y < res[1] - 1) & (z < res[2] - 1)
    near = np.zeros(sv.size, bool)
    if inner.any():
        corners = corner_ids(sv[inner], res)
        near[inner] = np.any(np.abs(o64.phi[np.clip(corners, 0, V - 1)] - o32.simparam.isoValue) < NEAR_ISO,
                             axis=1)
    rep["near_iso_cubes"] = int(near.sum())
    mism = (gvalid != ovalid) & ~near
    assert not mism.any(), f"{int(mism.sum())} valid-cube flags differ outside near-iso cubes"
    if method != "akinci":
        mism = (gnv != o32.nverts) & ~near
        assert not mism.any(), f"{int(mism.sum())} vertex counts differ outside near-iso cubes"
    from oracle import pipeline as P
    vq = np.flatnonzero(ovalid)
    ocase = np.zeros(sv.size, np.uint32)
    if vq.size:
        ocase[vq] = P.cube_cases("oracle32", o32, sv[vq])
    mism = (gcase != ocase) & (ovalid == 1) & ~near
    assert not mism.any(), f"{int(mism.sum())} MC case indices differ outside near-iso cubes"
    mesh = rec.mesh()
    rep["triangles"] = mesh.n_triangles
    rep["triangles_oracle"] = o32.n_triangles
    if rep["near_iso_cubes"] == 0:
        assert mesh.n_triangles == o32.n_triangles, "triangle count differs"

    # marching cubes as a stage: the FP64 oracle on the GPU's own field must
    # give the same cubes and cases bit for bit and the same vertices within
    # 1e-5 relative.  Normals are checked against the FP32 oracle: the
    # reference's normals are FP32 quantities whose squared length overflows
    # to infinity next to the Yu13 fill value (1.7e22), giving a zero corner
    # normal, where FP64 would not overflow.
    m64 = P.marching_cubes_on("oracle64", o32, phi.astype(np.float32))
    m32 = P.marching_cubes_on("oracle32", o32, phi.astype(np.float32))
    assert np.array_equal(gvalid, m64.valid.astype(np.uint32)), "MC valid flags on the GPU field"
    if method != "akinci":
        assert np.array_equal(gnv, m64.nverts), "MC vertex counts on the GPU field"
    assert mesh.positions.shape == m64.mesh_pos.shape, "mesh size on the GPU field"
    if mesh.positions.size:
        scale = np.maximum(np.abs(m64.mesh_pos), 1.0)
        perr = np.abs(mesh.positions - m64.mesh_pos) / scale
        rep["vertex_rel_max"] = float(perr.max())
        assert rep["vertex_rel_max"] <= 1e-5, f"mesh vertices off by {rep['vertex_rel_max']:.3e}"
        # normals: the direction of an interpolated normal whose length before
        # normalisation is tiny (two nearly opposite corner normals) is
        # ill-conditioned; those are counted, the rest must agree to 1e-4
        ln = m32.extra["normal_len"].astype(np.float64)
        fin = np.isfinite(m32.mesh_nrm).all(axis=1) & np.isfinite(ln)
        rep["normal_nonfinite"] = int((~fin).sum())
        assert np.array_equal(np.isfinite(mesh.normals).all(axis=1), np.isfinite(m32.mesh_nrm).all(axis=1)), \
            "non-finite normals differ"
        good = fin & (ln >= NORMAL_MIN_LEN)
        rep["normal_ill_conditioned"] = int((fin & ~good).sum())
        if good.any():
            rep["normal_abs_max"] = float(np.abs(mesh.normals[good] - m32.mesh_nrm[good]).max())
            assert rep["normal_abs_max"] <= 1e-4, f"normals off by {rep['normal_abs_max']:.3e}"
    return rep


def compare_frame_fullsize(rec, o32, o64, method: str, h: float, sample_seed: int = 0) -> dict:
    """See _compare_frame_fullsize; prints what was measured before a failed
    check is reported."""
    rep = {}
    try:
        return _compare_frame_fullsize(rec, o32, o64, method, h, rep)
    except AssertionError:
        import json
        print("PARTIAL_REPORT " + json.dumps({k: v for k, v in rep.items() if k != "field_worst"}), flush=True)
        raise


def _compare_frame_fullsize(rec, o32, o64, method: str, h: float, rep: dict) -> dict:
    """Parity of a large frame (the benchmark's sizes).

    Up to the band every integer equals the FP32 oracle's (the reference's
    arithmetic) bit for bit, and the field at every band vertex is within
    the field tolerance of the FP64 oracle, as for the small frames.

    Marching cubes: a case depends on the signs of eight field values
    relative to iso, so it is only as exact as the field.  On frames of this
    size the reference's own FP32 sum in window order drifts by more than the
    1e-6 near-iso exemption, so its cases are not the exact ones everywhere.
    The exact side is the FP64 oracle: outside near-iso cubes (a corner with
    |phi64 - iso| < NEAR_ISO) the GPU's valid flags, vertex counts and case
    indices must equal the cases of the FP64 field bit for bit.  The cubes
    where the FP32 oracle's cases differ from the GPU's are counted and, for
    each, it is recorded which side agrees with FP64."""
    from oracle import pipeline as P
    assert np.array_equal(rec.debug("perm"), o32.perm), "stable sort order differs"
    assert np.array_equal(rec.debug("ranges"), o32.ranges), "cell ranges differ"
    assert np.array_equal(rec.debug("sorted_xyz"), o32.pos), "sorted positions differ"
    assert np.array_equal(rec.debug("surface_flags"), o32.sflag), "surface particle flags differ"
    rep["particles"] = int(o32.perm.size)
    rep["surface_particles"] = int(o32.sflag.sum())
    if method == "yu13":
        assert np.array_equal(rec.debug("involved_counts"), o32.ninv), "involved counts differ"
        assert np.array_equal(rec.debug("mean"), o32.mean32), "weighted means differ"
        sm = rec.debug("smoothed")
        rep["smoothed_abs_max"] = float(np.abs(sm - o64.smoothed).max()) if sm.size else 0.0
        assert rep["smoothed_abs_max"] <= 1e-6, "smoothed positions"
        G = rec.debug("G")[o32.inv]
        rel = np.linalg.norm(G - o64.G, axis=1) / np.linalg.norm(o64.G, axis=1)
        rep["involved_particles"] = int(o32.inv.size)
        rep["G_rel_max"] = float(rel.max()) if rel.size else 0.0
        if rel.size:
            det = np.linalg.det(G.reshape(-1, 3, 3).astype(np.float64))
            det64 = np.linalg.det(o64.G.reshape(-1, 3, 3))
            rep["G_rel_median"] = float(np.median(rel))
            rep["detG_rel_max"] = float(np.max(np.abs(det - det64) / np.abs(det64)))
            rep["detG_rel_mean_signed"] = float(np.mean((det - det64) / np.abs(det64)))
        assert rep["G_rel_max"] <= 1e-5, f"G relative error {rep['G_rel_max']:.3e}"
    sv = rec.debug("band")
    assert np.array_equal(sv, o32.sv), "band vertices differ"
    rep["band_vertices"] = int(sv.size)

    phi = rec.debug("field").astype(np.float64)
    phi64 = o64.phi[o64.sv]
    tol = field_tolerance(method, h, phi64)
    err = np.abs(phi - phi64)
    rep["field_abs_max"] = float(err.max()) if err.size else 0.0
    rep["field_viol"] = int((err > tol).sum())
    err32 = np.abs(o32.phi[o32.sv].astype(np.float64) - phi64)
    rep["fp32_oracle_field_abs_max"] = float(err32.max()) if err32.size else 0.0
    rep["fp32_oracle_field_viol"] = int((err32 > tol).sum())
    if rep["field_viol"]:
        worst = np.argsort(-(err / tol))[:5]
        rep["field_worst"] = [{"vertex": int(sv[k]), "phi64": float(phi64[k]), "gpu": float(phi[k]),
                               "fp32_oracle": float(o32.phi[o32.sv][k]), "tol": float(tol[k])} for k in worst]
        print("FIELD_WORST " + repr(rep["field_worst"]), flush=True)
    assert rep["field_viol"] == 0, f"{rep['field_viol']} field values beyond tolerance (max {err.max():.3e})"

    info = rec.debug("mc_info")
    gcase, gnv, gvalid = info & 0xFF, (info >> 8) & 0xFF, (info >> 16) & 1
    res = o32.scalar.resolution
    V = o32.scalar.count
    x = sv % res[0]
    y = (sv // res[0]) % res[1]
    z = sv // (res[0] * res[1])
    inner = (x < res[0] - 1) & (y < res[1] - 1) & (z < res[2] - 1)
    near = np.zeros(sv.size, bool)
    iso = np.float64(o32.simparam.isoValue)
    if inner.any():
        ii = np.flatnonzero(inner)
        for a in range(0, ii.size, 1 << 20):
            blk = ii[a:a + (1 << 20)]
            corners = np.clip(corner_ids(sv[blk], res), 0, V - 1)
            near[blk] = np.any(np.abs(o64.phi[corners] - iso) < NEAR_ISO, axis=1)
    rep["near_iso_cubes"] = int(near.sum())

    def cases(kind, fr, valid):
        out = np.zeros(sv.size, np.uint32)
        vq = np.flatnonzero(valid)
        if vq.size:
            out[vq] = P.cube_cases(kind, fr, sv[vq])
        return out

    v64 = o64.valid.astype(np.uint32)
    v32 = o32.valid.astype(np.uint32)
    c64 = cases("oracle64", o64, v64)
    c32 = cases("oracle32", o32, v32)
    far = ~near
    # cases are compared where the cube is valid (k_mc_classify records the
    # case of every band cube; the oracle lists only valid ones)
    bad = far & ((gvalid != v64) | ((gcase != c64) & (v64 == 1)))
    if method != "akinci":
        bad |= far & (gnv != o64.nverts)
    rep["gpu_vs_fp64_case_diffs"] = int(bad.sum())
    assert not bad.any(), f"{int(bad.sum())} cubes differ from the FP64 oracle's cases outside near-iso cubes"
    # the reference's arithmetic (FP32 oracle) against the GPU: every such cube
    # outside the exemption is one where the FP32 oracle disagrees with FP64
    d32 = far & ((gvalid != v32) | ((gcase != c32) & (v32 == 1)))
    rep["fp32_oracle_case_diffs"] = int(d32.sum())
    rep["fp32_oracle_case_diffs_fp64_sides_with_gpu"] = int((d32 & (gvalid == v64) &
                                                            ((gcase == c64) | (v64 == 0))).sum())
    if d32.any():
        corners = np.clip(corner_ids(sv[d32], res), 0, V - 1)
        rep["fp32_oracle_case_diffs_min_abs_phi64_minus_iso"] = float(np.abs(o64.phi[corners] - iso).min(axis=1).max())
    rep["near_iso_case_diffs_vs_fp64"] = int((near & ((gvalid != v64) | ((gcase != c64) & (v64 == 1)))).sum())
    rep["near_iso_case_diffs_vs_fp32"] = int((near & ((gvalid != v32) | ((gcase != c32) & (v32 == 1)))).sum())

    mesh = rec.mesh()
    rep["triangles"] = int(mesh.n_triangles)
    rep["triangles_fp32_oracle"] = int(o32.n_triangles)
    rep["triangles_fp64_oracle"] = int(o64.n_triangles)
    # a cube yields at most 5 triangles: any difference in triangle count must
    # come from cubes whose case differs
    if method != "akinci":
        dv = int(np.abs(gnv.astype(np.int64) - o64.nverts.astype(np.int64))[near].sum())
        assert abs(rep["triangles"] - rep["triangles_fp64_oracle"]) * 3 <= dv, "triangle count vs FP64"
    else:
        assert abs(rep["triangles"] - rep["triangles_fp64_oracle"]) <= 5 * rep["near_iso_case_diffs_vs_fp64"]

    # marching cubes as a stage on the GPU's own field, as for small frames
    m64 = P.marching_cubes_on("oracle64", o32, phi.astype(np.float32))
    assert np.array_equal(gvalid, m64.valid.astype(np.uint32)), "MC valid flags on the GPU field"
    if method != "akinci":
        assert np.array_equal(gnv, m64.nverts), "MC vertex counts on the GPU field"
    assert mesh.positions.shape == m64.mesh_pos.shape, "mesh size on the GPU field"
    if mesh.positions.size:
        scale = np.maximum(np.abs(m64.mesh_pos), 1.0)
        rep["vertex_rel_max"] = float((np.abs(mesh.positions - m64.mesh_pos) / scale).max())
        assert rep["vertex_rel_max"] <= 1e-5, f"mesh vertices off by {rep['vertex_rel_max']:.3e}"
        del m64
        m32 = P.marching_cubes_on("oracle32", o32, phi.astype(np.float32))
        ln = m32.extra["normal_len"].astype(np.float64)
        fin = np.isfinite(m32.mesh_nrm).all(axis=1) & np.isfinite(ln)
        assert np.array_equal(np.isfinite(mesh.normals).all(axis=1), np.isfinite(m32.mesh_nrm).all(axis=1)), \
            "non-finite normals differ"
        good = fin & (ln >= NORMAL_MIN_LEN)
        rep["normal_ill_conditioned"] = int((fin & ~good).sum())
        rep["normal_abs_max"] = float(np.abs(mesh.normals[good] - m32.mesh_nrm[good]).max()) if good.any() else 0.0
        assert rep["normal_abs_max"] <= 1e-4, f"normals off by {rep['normal_abs_max']:.3e}"
    return rep
