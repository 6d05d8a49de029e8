"""Full-size finite-difference check of the adjoint kernels (test infrastructure).

Workload: 262,144 jittered particles filling a sphere of radius 0.3, displaced
by Gaussian noise of 0.5 r (synthetic.sphere_ball); anisotropic field with the
reference's parameters; loss = mean over mesh vertices of (|v - c| - 0.32)^2.

  python tests/golden/fd_sphere262k.py grad GRAD.npz      (GPU: dL/dx of 256 random particles)
  python tests/golden/fd_sphere262k.py fd GRAD.npz ROWS.jsonl
        (CPU: FP64 central differences, delta = 1e-4 r, of the FP64 oracle's
         whole pipeline for the same particles; one JSON line per particle is
         appended to ROWS.jsonl, and a rerun skips the particles already there;
         hours of CPU time)
  python tests/golden/fd_sphere262k.py summary ROWS.jsonl SUMMARY.json [GRAD.npz]
        (GRAD.npz: a later gradient of the same particles replaces the one
         recorded in the rows)

The fd step skips coordinates whose perturbation changes a discrete decision
(sort order, surface flags, band, cubes, cases, involved cells) or where the
loss has a corner (one-sided differences disagree by more than 1e-3), and
reports the error of the remaining ones relative to the largest |fd|.
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

C0 = np.array([0.5, 0.5, 0.5])
R0 = 0.32
N_SAMPLE = 256
SEED = 4


def loss(pos):
    d = np.asarray(pos, np.float64) - C0
    r = np.linalg.norm(d, axis=1)
    return float(np.mean((r - R0) ** 2))


def grad_mesh(pos):
    d = np.asarray(pos, np.float64) - C0
    r = np.linalg.norm(d, axis=1)
    return (2.0 * (r - R0) / np.maximum(r, 1e-12) / pos.shape[0])[:, None] * d


def frame():
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    return synthetic.sphere_ball(262144, radius=0.3, seed=SEED)


def sample(n):
    return np.sort(np.random.default_rng(SEED).choice(n, N_SAMPLE, replace=False))


def run_grad(out):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    fr = frame()
    rec = api.Reconstructor("yu13", 0)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    pos, _ = rec.mesh_tensors()
    pm = pos.cpu().numpy()
    g = rec.backward(torch.from_numpy(grad_mesh(pm).astype(np.float32)).cuda()).cpu().numpy()
    st = rec.stats()
    rec.close()
    idx = sample(fr.n)
    np.savez(out, idx=idx, grad=g[idx], loss=loss(pm), n=fr.n, n_mesh=pm.shape[0],
             n_band=int(st.n_band_vertices), n_involved=int(st.n_involved_particles))
    print(json.dumps({"n": fr.n, "mesh_vertices": int(pm.shape[0]), "loss": loss(pm),
                      "nonzero_rows": int(np.count_nonzero(np.abs(g[idx]).sum(1)))}))


def structure(o):
    G = o.G
    iso = np.all(G[:, [1, 2, 3, 5, 6, 7]] == 0, axis=1) & (G[:, 0] == G[:, 4]) & (G[:, 4] == G[:, 8])
    return [o.perm, o.sflag, o.sv, o.valid, o.nverts, o.ninv, o.inv, iso]


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def run_fd(inp, rows_path):
    from oracle import pipeline as P
    d = np.load(inp)
    done = set()
    if os.path.exists(rows_path):
        for line in open(rows_path):
            if line.strip():
                done.add(json.loads(line)["particle"])
    fr = frame()
    P.set_threads("oracle64", os.cpu_count() or 1)
    params = P.FrameParams(method="yu13", h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass)
    t0 = time.time()
    base = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params)
    sb, L0 = structure(base), loss(base.mesh_pos)
    delta = 1e-4 * fr.particle_radius
    for n_done, (i, gi) in enumerate(zip(d["idx"], d["grad"])):
        if int(i) in done:
            continue
        rec = {"particle": int(i), "coords": []}
        for k in range(3):
            pp, pm = fr.pos.copy(), fr.pos.copy()
            pp[i, k] = np.float32(fr.pos[i, k] + delta)
            pm[i, k] = np.float32(fr.pos[i, k] - delta)
            op = P.run_frame("oracle64", pp, fr.density, fr.bbox_min, fr.bbox_max, params)
            om = P.run_frame("oracle64", pm, fr.density, fr.bbox_min, fr.bbox_max, params)
            c = {"axis": k, "grad": float(gi[k])}
            if not (same(structure(op), sb) and same(structure(om), sb)):
                c["skip"] = "structure"
            else:
                Lp, Lm = loss(op.mesh_pos), loss(om.mesh_pos)
                fwd = (Lp - L0) / (float(pp[i, k]) - float(fr.pos[i, k]))
                bwd = (L0 - Lm) / (float(fr.pos[i, k]) - float(pm[i, k]))
                if abs(fwd - bwd) > 1e-3 * max(abs(fwd), abs(bwd)) + 1e-15:
                    c["skip"] = "kink"
                c["fd"] = (Lp - Lm) / (float(pp[i, k]) - float(pm[i, k]))
            rec["coords"].append(c)
        with open(rows_path, "a") as f:
            f.write(json.dumps(rec) + "\n")
        print(f"{n_done + 1}/{len(d['idx'])} particles, {time.time() - t0:.0f} s", flush=True)


def run_summary(rows_path, out, grad_path=None):
    # the rows carry the gradient the fd step was started with; a later
    # gradient file (the same particles) replaces it
    override = None
    if grad_path:
        g = np.load(grad_path)
        override = {int(i): gi for i, gi in zip(g["idx"], g["grad"])}
    rows, skipped_structure, skipped_kink, n_particles = [], 0, 0, 0
    for line in open(rows_path):
        if not line.strip():
            continue
        rec = json.loads(line)
        n_particles += 1
        for c in rec["coords"]:
            if c.get("skip") == "structure":
                skipped_structure += 1
            elif c.get("skip") == "kink":
                skipped_kink += 1
            else:
                gval = float(override[rec["particle"]][c["axis"]]) if override is not None else c["grad"]
                rows.append((rec["particle"], c["axis"], gval, c["fd"]))
    r = np.array(rows)
    scale = float(np.abs(r[:, 3]).max()) if len(r) else 0.0
    err = np.abs(r[:, 2] - r[:, 3]) if len(r) else np.zeros(0)
    nz = np.abs(r[:, 3]) > 1e-3 * scale if len(r) else np.zeros(0, bool)
    summary = {
        "workload": "sphere_ball(262144, radius 0.3, seed 4): 262,144 particles, anisotropic field, reference parameters",
        "loss": "mean over mesh vertices of (|v - (0.5,0.5,0.5)| - 0.32)^2",
        "fd": "FP64 oracle, central differences, delta = 1e-4 r",
        "gradient": os.path.basename(grad_path) if grad_path else "as recorded in the rows",
        "particles": n_particles, "coordinates": 3 * n_particles, "compared": int(len(r)),
        "skipped_structure_change": skipped_structure, "skipped_kink": skipped_kink,
        "nonzero_fd": int(nz.sum()), "max_abs_fd": scale,
        "max_err_rel_to_max_fd": float(err.max() / scale) if scale else 0.0,
        "max_rel_err_nonzero": float(np.max(err[nz] / np.abs(r[nz, 3]))) if nz.any() else 0.0,
        "median_rel_err_nonzero": float(np.median(err[nz] / np.abs(r[nz, 3]))) if nz.any() else 0.0,
        "exact_zero_pairs": int(np.sum((r[:, 2] == 0) & (r[:, 3] == 0))) if len(r) else 0,
    }
    json.dump(summary, open(out, "w"), indent=1)
    print(json.dumps(summary, indent=1))


if __name__ == "__main__":
    if sys.argv[1] == "grad":
        run_grad(sys.argv[2])
    elif sys.argv[1] == "fd":
        run_fd(sys.argv[2], sys.argv[3])
    else:
        run_summary(sys.argv[2], sys.argv[3], sys.argv[4] if len(sys.argv) > 4 else None)
