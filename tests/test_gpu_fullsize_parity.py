"""Full-size parity: the benchmark's frames against the CPU oracle.

* the 1M-particle anisotropic frame of the benchmark (dam-break column +
  droplet + splash, 2^20 particles, lambda 0.9, neighbour radius h, cell
  1.25h, grid spacing 0.5r);
* one 400k-particle frame of each method of the batched workload (the
  lattice generator rescaled to 400k particles, grid spacing 0.5r).

Each frame runs once on the GPU with its intermediates kept and once through
the FP32 oracle (the reference's arithmetic) and the FP64 oracle, over the
whole frame: sorted order, cell ranges, sorted particles, surface flags,
involved counts, weighted means and band vertices bit for bit; G of every
involved particle and the field at every band vertex within 1e-5 relative of
FP64; marching-cubes cases, valid cubes and vertex counts equal to the FP64
field's outside near-iso cubes, with the cubes where the FP32 oracle differs
counted (tests/parity.py, compare_frame_fullsize).  The counts are printed
as one JSON line per frame.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ANISO = dict(smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0)


def _params(method, fr, kw):
    from oracle import pipeline as P
    return P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass,
                         iso=kw.get("iso"), ratio=kw.get("grid_ratio"), cell_scale=kw.get("cell_size_scale"),
                         lam=kw.get("smoothing_lambda", 0.5),
                         aniso_radius=(kw["aniso_radius_over_h"] * fr.h if "aniso_radius_over_h" in kw else None))


def _check(name, method, fr, kw):
    import os
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    from oracle import pipeline as P
    from tests.parity import compare_frame_fullsize

    rec = api.Reconstructor(method, 0, keep_intermediates=True, **kw)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    torch.cuda.synchronize()
    prm = _params(method, fr, kw)
    for kind in ("oracle32", "oracle64"):
        P.set_threads(kind, os.cpu_count() or 1)
    o32 = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    o64 = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    rep = compare_frame_fullsize(rec, o32, o64, method, fr.h)
    rec.close()
    rep = {"frame": name, "method": method, **rep}
    print("FULLSIZE_PARITY " + json.dumps(rep), flush=True)
    return rep


def test_aniso_1m_benchmark_frame():
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.dam_break(1 << 20, r=0.004, seed=2)
    rep = _check("aniso1m", "yu13", fr, ANISO)
    assert rep["band_vertices"] > 8_000_000 and rep["triangles"] > 900_000


@pytest.mark.parametrize("method", ["zb05", "akinci", "yu13"])
def test_batch_generator_400k(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    fr = synthetic.lattice_count(400_000, seed=3)
    kw = ANISO if method == "yu13" else dict(grid_ratio=8)
    rep = _check("lattice400k", method, fr, kw)
    assert rep["triangles"] > 10_000
