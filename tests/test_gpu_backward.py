"""Adjoint kernels against FP64 central finite differences.

Loss (the differentiation workload's): L = mean over mesh vertices of
(|p - c| - R0)^2.  The GPU gradient dL/dx comes from fsr_backward; the
reference gradient is (L(x + d) - L(x - d)) / 2d with L evaluated by the FP64
oracle on the perturbed particles, d = 1e-4 r.  Coordinates whose
perturbation changes any discrete decision of the frame (band, cubes, cases,
involved cells) are skipped, and so are coordinates where the loss has a
corner (the one-sided differences disagree): the gradient holds the
structure fixed and is the derivative where one exists.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C0 = np.array([0.375, 0.375, 0.375])
R0 = 0.07


def _loss(pos):
    d = np.asarray(pos, np.float64) - C0
    r = np.linalg.norm(d, axis=1)
    return float(np.mean((r - R0) ** 2)), d, r


def _grad_mesh(pos):
    L, d, r = _loss(pos)
    n = pos.shape[0]
    return (2.0 * (r - R0) / np.maximum(r, 1e-12) / n)[:, None] * d


def _structure(o):
    keys = [o.perm, o.sflag, o.sv, o.valid, o.nverts if o.nverts is not None else np.zeros(1)]
    if o.method == "yu13":
        G = o.G
        iso = np.all(G[:, [1, 2, 3, 5, 6, 7]] == 0, axis=1) & (G[:, 0] == G[:, 4]) & (G[:, 4] == G[:, 8])
        keys += [o.ninv, o.inv, iso]
    return keys


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def _case(method, fr, n_sample=12, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P
    rec = api.Reconstructor(method, 0, **kw)
    xyz = torch.from_numpy(fr.pos).cuda()
    den = torch.from_numpy(fr.density).cuda()
    rec.reconstruct(xyz, den, api.header_of(fr))
    pos, _ = rec.mesh_tensors()
    gm = torch.from_numpy(_grad_mesh(pos.cpu().numpy()).astype(np.float32)).cuda()
    g = rec.backward(gm).cpu().numpy().astype(np.float64)
    rec.close()

    params = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass,
                           iso=kw.get("iso"), ratio=kw.get("grid_ratio"), cell_scale=kw.get("cell_size_scale"),
                           lam=kw.get("smoothing_lambda", 0.5),
                           aniso_radius=(kw["aniso_radius_over_h"] * fr.h if "aniso_radius_over_h" in kw else None))
    base = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    sbase = _structure(base)
    L0 = _loss(base.mesh_pos)[0]
    mag = np.linalg.norm(g, axis=1)
    rng = np.random.default_rng(0)
    order = np.argsort(-mag)
    sample = np.unique(np.concatenate([order[: n_sample - 4], rng.choice(fr.n, 4, replace=False)]))
    delta = 1e-4 * fr.particle_radius
    rows = []
    for i in sample:
        for k in range(3):
            pp, pm = fr.pos.copy(), fr.pos.copy()
            pp[i, k] = np.float32(fr.pos[i, k] + delta)
            pm[i, k] = np.float32(fr.pos[i, k] - delta)
            op = P.run_frame("oracle64", pp, fr.density, fr.bbox_min, fr.bbox_max, params)
            om = P.run_frame("oracle64", pm, fr.density, fr.bbox_min, fr.bbox_max, params)
            if not (_same(_structure(op), sbase) and _same(_structure(om), sbase)):
                continue
            Lp, Lm = _loss(op.mesh_pos)[0], _loss(om.mesh_pos)[0]
            # a kink (a neighbour crossing the radius where the weight
            # 1 - (d/R)^3 has a corner, a clamp switching) shows as one-sided
            # differences that disagree: no derivative to compare there
            fwd = (Lp - L0) / (float(pp[i, k]) - float(fr.pos[i, k]))
            bwd = (L0 - Lm) / (float(fr.pos[i, k]) - float(pm[i, k]))
            if abs(fwd - bwd) > 1e-3 * max(abs(fwd), abs(bwd)) + 1e-12:
                continue
            fd = (Lp - Lm) / (float(pp[i, k]) - float(pm[i, k]))
            rows.append((i, k, g[i, k], fd))
    rows = np.array(rows)
    assert rows.shape[0] >= 3 * n_sample // 2, "too many perturbations changed the frame's structure"
    scale = np.abs(rows[:, 3]).max()
    err = np.abs(rows[:, 2] - rows[:, 3])
    return rows, err, scale


@pytest.mark.parametrize("method", ["zb05", "tc01"])
def test_isotropic_fields_match_fp64_finite_differences(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    rows, err, scale = _case(method, fr)
    assert scale > 0
    assert err.max() <= 2e-3 * scale, (err.max() / scale, rows[np.argmax(err)])


ANISO_SETTINGS = {
    "reference": {},
    # the 1M-frame settings: lambda 0.9, neighbours within h, cell 1.25h, ratio 10
    "fine": dict(smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0),
}


@pytest.mark.parametrize("setting", sorted(ANISO_SETTINGS))
def test_anisotropic_field_matches_fp64_finite_differences(setting):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    rows, err, scale = _case("yu13", fr, **ANISO_SETTINGS[setting])
    assert scale > 0
    assert err.max() <= 2e-3 * scale, (err.max() / scale, rows[np.argmax(err)])


def test_zb05_particle_radius_gradient():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    from oracle import pipeline as P
    fr = synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    rec = api.Reconstructor("zb05", 0)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    pos, _ = rec.mesh_tensors()
    gm = torch.from_numpy(_grad_mesh(pos.cpu().numpy()).astype(np.float32)).cuda()
    _, gr = rec.backward(gm, with_radius=True)
    rec.close()
    d = 1e-4 * fr.particle_radius
    Ls = []
    for s in (+1, -1):
        params = P.FrameParams(method="zb05", h=fr.h, particle_radius=fr.particle_radius + s * d, mass=fr.mass)
        Ls.append(_loss(P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params).mesh_pos)[0])
    r32p, r32m = np.float32(fr.particle_radius + d), np.float32(fr.particle_radius - d)
    fd = (Ls[0] - Ls[1]) / (float(r32p) - float(r32m))
    assert abs(gr - fd) <= 2e-3 * abs(fd), (gr, fd)


def test_autograd_function():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    from fluidsurfacereconstructiongpu_gb300.autograd import reconstruct_surface
    fr = synthetic.lattice_cube(10, 0.0125, seed=2, origin=(0.3, 0.3, 0.3))
    rec = api.Reconstructor("yu13", 0)
    xyz = torch.from_numpy(fr.pos).cuda().requires_grad_(True)
    den = torch.from_numpy(fr.density).cuda()
    pos = reconstruct_surface(xyz, den, rec, api.header_of(fr))
    c = torch.tensor(C0, dtype=torch.float32, device="cuda")
    loss = ((pos - c).norm(dim=1) - R0).pow(2).mean()
    loss.backward()
    g_ref = rec.backward(torch.from_numpy(_grad_mesh(pos.detach().cpu().numpy()).astype(np.float32)).cuda())
    assert torch.allclose(xyz.grad, g_ref, rtol=1e-4, atol=1e-9)
    rec.close()


@pytest.mark.parametrize("method", ["zb05", "akinci"])
def test_autograd_radius_gradient(method):
    """The autograd wrapper returns dL/d(particle radius) for the fields that
    use it, equal to the C ABI's, and the radius tensor's value is the one
    the frame is reconstructed with."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    from fluidsurfacereconstructiongpu_gb300.autograd import reconstruct_surface
    fr = synthetic.lattice_cube(10, 0.0125, seed=2, origin=(0.3, 0.3, 0.3))
    rec = api.Reconstructor(method, 0)
    xyz = torch.from_numpy(fr.pos).cuda().requires_grad_(True)
    den = torch.from_numpy(fr.density).cuda()
    r = torch.tensor(fr.particle_radius * 1.05, dtype=torch.float32, device="cuda", requires_grad=True)
    pos = reconstruct_surface(xyz, den, rec, api.header_of(fr), radius=r)
    c = torch.tensor(C0, dtype=torch.float32, device="cuda")
    loss = ((pos - c).norm(dim=1) - R0).pow(2).mean()
    loss.backward()
    hdr = api.header_of(fr)
    hdr.particle_radius = float(r.item())
    rec.reconstruct(xyz.detach(), den, hdr)
    pos2, _ = rec.mesh_tensors()
    assert torch.equal(pos.detach(), pos2)
    g_ref, gr_ref = rec.backward(torch.from_numpy(_grad_mesh(pos2.cpu().numpy()).astype(np.float32)).cuda(),
                                 with_radius=True)
    assert gr_ref != 0.0
    assert abs(float(r.grad) - gr_ref) <= 1e-4 * abs(gr_ref)
    assert torch.allclose(xyz.grad, g_ref, rtol=1e-4, atol=1e-9)
    rec.close()
