"""Batched frames (one CUDA graph launch) against the single-frame path.

Every frame of a batch must give exactly the single-frame results (the same
kernels run on the same particles; batching only changes when they run):
mesh positions, normals and every count, bit for bit.  The single-frame path
itself is checked against the oracle in the parity tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames(seed=3, count=7):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    rng = np.random.default_rng(seed)
    methods = ["zb05", "yu13", "akinci12", "tc01"]
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(40000))))
        out.append((methods[i % len(methods)], synthetic.lattice_count(n, seed=seed + i)))
    return out


def _single(method, fr, **kw):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    rec = api.Reconstructor(method, 0, **kw)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    m, st = rec.mesh(), rec.stats()
    rec.close()
    return m, st


def _check_same(b, i, method, fr, **kw):
    m1, s1 = _single(method, fr, **kw)
    m2, s2 = b.mesh(i), b.stats(i)
    for k in ("n_particles", "n_surface_particles", "n_involved_particles", "n_band_vertices", "n_valid_cubes",
              "n_mesh_vertices", "n_fp64_fallbacks"):
        assert getattr(s1, k) == getattr(s2, k), (i, method, k)
    assert np.array_equal(m1.positions, m2.positions), (i, method)
    assert np.array_equal(m1.normals, m2.normals), (i, method)


def test_batch_matches_single_frames_device_inputs():
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    frames = _frames()
    b = api.Batch(0)
    args = [(m, torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
            for m, fr in frames]
    b.reconstruct(args)
    t = b.tuning()
    assert t.lanes >= 1 and t.n_candidates >= 2 and t.kernels_per_launch > 0
    for i, (m, fr) in enumerate(frames):
        _check_same(b, i, m, fr)
    # same shape again: the graph is replayed on new particles
    frames2 = [(m, fr) for m, fr in frames]
    rng = np.random.default_rng(11)
    for _, fr in frames2:
        fr.pos = (fr.pos + rng.uniform(-1e-4, 1e-4, fr.pos.shape)).astype(np.float32)
    args2 = [(m, torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
             for m, fr in frames2]
    b.reconstruct(args2)
    t2 = b.tuning()
    assert (t2.lanes, t2.grid_div) == (t.lanes, t.grid_div)
    for i, (m, fr) in enumerate(frames2):
        _check_same(b, i, m, fr)
    b.close()


def test_batch_host_inputs_and_capacity_growth():
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic, _native as N
    # plan on small lattices, then replay the same shape on particles whose
    # band is larger: the frames must grow and re-run inside the batch call
    # (small initial pools: the planned frames grow them once, the scattered
    # frames' band is about twice the lattice's)
    small = [("zb05", synthetic.lattice_count(6000, seed=5)), ("tc01", synthetic.lattice_count(6000, seed=6))]
    pools = {"grid_ratio": 16, "flags": N.FLAG_SMALL_POOLS}
    b = api.Batch(0, params={"zb05": pools, "tc01": pools})
    b.reconstruct([(m, fr.pos, fr.density, api.header_of(fr)) for m, fr in small], autotune=False)
    for i, (m, fr) in enumerate(small):
        _check_same(b, i, m, fr, grid_ratio=16)
    r1 = [b.stats(i).n_retries for i in range(2)]
    grown = []
    rng = np.random.default_rng(7)
    for m, fr in small:
        g = synthetic.lattice_count(6000, seed=5)
        # scatter the same number of particles over the whole box: far more surface
        g.pos = rng.uniform(0.05, 0.95, size=fr.pos.shape).astype(np.float32)
        g.h, g.particle_radius, g.mass = fr.h, fr.particle_radius, fr.mass
        grown.append((m, g))
    b.reconstruct([(m, fr.pos, fr.density, api.header_of(fr)) for m, fr in grown], autotune=False)
    assert any(b.stats(i).n_retries > r1[i] for i in range(2))
    for i, (m, fr) in enumerate(grown):
        _check_same(b, i, m, fr, grid_ratio=16)
    b.close()


def test_batch_rejects_bad_frames():
    from fluidsurfacereconstructiongpu_gb300 import api, _native as N, synthetic
    fr = synthetic.lattice_count(3000, seed=1)
    b = api.Batch(0)
    with pytest.raises(N.FsrError):
        b.reconstruct([])
    bad = fr.pos.copy()
    bad[0] = (5.0, 5.0, 5.0)  # outside the expanded box
    with pytest.raises(N.FsrError) as e:
        b.reconstruct([("zb05", bad, fr.density, api.header_of(fr))], autotune=False)
    assert e.value.status == 2
    b.close()


def test_batch_at_the_benchmark_sizes():
    """The first 12 frames of the benchmark's batch (20k-400k particles,
    mixed fields, the anisotropic frames with the 1M frame's settings):
    every frame equals the single-frame path bit for bit, with the batch's
    autotuned lanes, grid division and block shape."""
    import torch
    import bench
    from fluidsurfacereconstructiongpu_gb300 import api
    frames = bench.batch_frames()[:12]
    params = bench.BATCH["params"]
    b = api.Batch(0, params=params)
    args = [(m, torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
            for m, fr in frames]
    b.reconstruct(args)
    t = b.tuning()
    assert t.block_threads in (128, 256)
    for i, (m, fr) in enumerate(frames):
        _check_same(b, i, m, fr, **params[m])
    b.close()
