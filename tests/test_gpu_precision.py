"""The precision policy's FP64 branch: near-degenerate covariances.

The covariance of the anisotropic path is seeded with h^2 I and normalised by
the weight sum (calculationOfTransformMatricesForParticles,
ReconstructionCUDA.cu:718-723), so its condition number is at most about
1 + R^2 sum(w) / h^2 times a shape factor: it passes 1e4 only where a
particle has thousands of neighbours spread along fewer than three
directions.  The frame here is such a case: a dense, thin fibre (particles
along a tilted segment, 2e-3 h thick) where every interior particle sees
about 36k neighbours along one direction.  The library's FP32 Jacobi solve
is redone in FP64 on the GPU for those particles (cov_solver.cuh,
covariance_to_G); the test checks that the branch runs
(fsr_stats.n_fp64_fallbacks > 0), that G of every involved particle is
within 1e-5 relative of the FP64 oracle's (cu:790-822 restated in FP64), and
the whole frame's parity (tests/parity.py, compare_frame_fullsize).  The
condition numbers of a sample of particles are computed here in FP64 from
the definition, and the G error of the sampled particles above 1e4 is
printed with the fallback count.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fibre(n=72_000, length=0.3, h=0.05, thickness=1e-4, seed=21):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    rng = np.random.default_rng(seed)
    d = np.array([1.0, 0.6, 0.35])
    d /= np.linalg.norm(d)
    e1 = np.cross(d, [0.0, 0.0, 1.0])
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(d, e1)
    t = rng.uniform(-length / 2, length / 2, n)
    a, b = rng.normal(0.0, thickness, n), rng.normal(0.0, thickness, n)
    p = np.array([0.5, 0.5, 0.5]) + t[:, None] * d + a[:, None] * e1 + b[:, None] * e2
    r = h / 4
    return synthetic.ParticleFrame(bbox_min=np.zeros(3, np.float32), bbox_max=np.ones(3, np.float32), h=h,
                                   particle_radius=r, mass=1000.0 * r ** 3, pos=p.astype(np.float32),
                                   density=np.full(n, 1000.0, np.float32), name=f"fibre N={n}")


def condition_numbers(pos, mean, rows, R, h, min_neighbors):
    """FP64 condition number of the seeded, normalised covariance of each
    listed (sorted) particle, from its definition: neighbours j with
    |x_j - mean_i| <= R, weights 1 - (d/R)^3, C = (h^2 I + sum w v v^T) / sum w.
    Particles with fewer than min_neighbors neighbours get 0 (G = I/h)."""
    p = pos.astype(np.float64)
    out = np.zeros(len(rows))
    for k, i in enumerate(rows):
        v = p - mean[i]
        d = np.sqrt(np.sum(v * v, axis=1))
        sel = d <= R
        if sel.sum() < min_neighbors:
            continue
        w = np.where(d < R, 1.0 - (d / R) ** 3, 0.0)
        C = (h * h * np.eye(3) + np.einsum("n,ni,nj->ij", w, v, v)) / w.sum()
        ev = np.linalg.eigvalsh(C)
        out[k] = ev[-1] / ev[0]
    return out


def test_fp64_resolve_on_a_fibre():
    import os
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P
    from tests.parity import compare_frame_fullsize

    fr = fibre()
    rec = api.Reconstructor("yu13", 0, keep_intermediates=True)  # the reference's settings: R = 2h
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    torch.cuda.synchronize()
    st = rec.stats()
    n_fb = int(st.n_fp64_fallbacks)
    prm = P.FrameParams(method="yu13", h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass)
    for kind in ("oracle32", "oracle64"):
        P.set_threads(kind, os.cpu_count() or 1)
    o32 = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    o64 = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    G = rec.debug("G")[o32.inv]
    rep = compare_frame_fullsize(rec, o32, o64, "yu13", fr.h)
    rec.close()
    assert n_fb > 0, "no covariance reached the FP64 re-solve"

    rng = np.random.default_rng(5)
    rows = rng.choice(o32.inv.size, 64, replace=False)
    R = float(prm.simparam().anisotropicRadius)
    cond = condition_numbers(o32.pos, o64.mean, o32.inv[rows], R, float(np.float32(fr.h)), 25)
    hi = cond > 1e4
    rel = np.linalg.norm(G[rows] - o64.G[rows], axis=1) / np.linalg.norm(o64.G[rows], axis=1)
    rep.update(fp64_fallbacks=n_fb, sampled=int(rows.size), sampled_cond_above_1e4=int(hi.sum()),
               sampled_cond_max=float(cond.max()), sampled_G_rel_max_cond_above_1e4=float(rel[hi].max())
               if hi.any() else None)
    print("PRECISION " + json.dumps(rep), flush=True)
    assert hi.any(), "the sample holds no covariance above condition 1e4"
    assert rel.max() <= 1e-5
