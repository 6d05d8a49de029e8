"""fsr_count_pairs against a direct count on the host.

The pair counts feed the benchmark's FP32 throughput figures, so they are
checked here on small frames of every method: the candidate pairs are the
particles of each unit's cell window (ranges of the frame's own sorted
cells, +-2 cells for the anisotropic stages, +-1 for ZB05/TC01 and the
colour field) and the contributing pairs those inside the support, counted
in FP64 from the frame's kept intermediates.  Pairs whose squared distance
lies within 1e-5 relative of the support boundary may be counted either
way (the device evaluates it in FP32), so the contributing counts must
agree within the number of such borderline pairs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _windows(centres, sp, ext):
    mn = np.array(sp.minPos, np.float32)
    cs = np.float32(sp.cellSize)
    res = np.array(sp.res, np.int64)
    c = np.trunc(((centres.astype(np.float32) - mn).astype(np.float32) / cs).astype(np.float32)).astype(np.int64)
    return np.clip(c - ext, 0, res - 1), np.clip(c + ext, 0, res - 1), res


def _count(centres, lo, hi, res, ranges, test):
    cand = contrib = border = 0
    for u in range(centres.shape[0]):
        idx = []
        for z in range(lo[u, 2], hi[u, 2] + 1):
            for y in range(lo[u, 1], hi[u, 1] + 1):
                for x in range(lo[u, 0], hi[u, 0] + 1):
                    a, b = ranges[x + res[0] * (y + res[1] * z)]
                    if a != 0xFFFFFFFF:
                        idx.append(np.arange(a, b))
        if not idx:
            continue
        j = np.concatenate(idx)
        cand += j.size
        inside, near = test(u, j)
        contrib += int(inside.sum())
        border += int(near.sum())
    return cand, contrib, border


@pytest.mark.parametrize("method", ["zb05", "akinci", "yu13"])
def test_pair_counts_match_host_count(method):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    from oracle import pipeline as P
    fr = synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    rec = api.Reconstructor(method, 0, keep_intermediates=True)
    rec.reconstruct(torch.from_numpy(fr.pos).cuda(), torch.from_numpy(fr.density).cuda(), api.header_of(fr))
    pc = rec.pair_counts()
    p = rec.params
    sp, sc = P.grid_derive(fr.bbox_min, fr.bbox_max, fr.h, p.cell_size_scale, p.grid_ratio)
    pos = rec.debug("sorted_xyz").astype(np.float64)
    ranges = rec.debug("ranges")
    h = float(np.float32(fr.h))

    def ball(centres, r2):
        def test(u, j):
            d2 = np.sum((pos[j] - centres[u]) ** 2, axis=1)
            return d2 < r2, np.abs(d2 - r2) <= 1e-5 * r2
        return test

    def check(got_cand, got_contrib, want):
        cand, contrib, border = want
        assert got_cand == cand
        assert abs(got_contrib - contrib) <= border, (got_contrib, contrib, border)
        assert contrib > 0

    sv = rec.debug("band")
    vres = np.array(sc.res, np.int64)
    vi = np.stack([sv % vres[0], (sv // vres[0]) % vres[1], sv // (vres[0] * vres[1])], axis=1)
    vpos = (vi.astype(np.float32) * np.float32(sc.cellSize)).astype(np.float32) + np.array(sc.minPos, np.float32)
    if method == "yu13":
        R = float(np.float32(h * np.float32(p.aniso_radius_over_h)))
        lo, hi, res = _windows(pos, sp, 2)
        check(pc["smooth_candidates"], pc["smooth_contributing"], _count(pos, lo, hi, res, ranges, ball(pos, R * R)))
        inv_counts = rec.debug("involved_counts")
        # the covariance runs over the involved particles about their means
        # (the compensated mean is within 1e-6 of the FP32 mean kept for
        # the parity tests; pairs that close to R count as borderline)
        keys = np.repeat(np.arange(ranges.shape[0]), np.where(ranges[:, 0] == 0xFFFFFFFF, 0,
                                                               ranges[:, 1] - ranges[:, 0]))
        inv = np.flatnonzero(inv_counts[keys] > 0)
        mean = rec.debug("mean").astype(np.float64)[inv]
        lo, hi, res = _windows(pos[inv], sp, 2)

        def cov_test(u, j):
            d = np.sqrt(np.sum((pos[j] - mean[u]) ** 2, axis=1))
            return d < R, np.abs(d - R) <= 1e-5 * R
        check(pc["cov_candidates"], pc["cov_contributing"], _count(pos[inv], lo, hi, res, ranges, cov_test))
        assert pc["field_candidates"] > 0 and 0 < pc["field_contributing"] <= pc["field_candidates"]
    else:
        lo, hi, res = _windows(vpos, sp, 1)
        check(pc["field_candidates"], pc["field_contributing"],
              _count(vpos.astype(np.float64), lo, hi, res, ranges, ball(vpos.astype(np.float64), h * h)))
        if method == "akinci":
            lo, hi, res = _windows(pos, sp, 1)

            def col_test(u, j):
                d2 = np.sum((pos[j] - pos[u]) ** 2, axis=1)
                return (d2 < h * h) & (d2 > 0), np.abs(d2 - h * h) <= 1e-5 * h * h
            check(pc["color_candidates"], pc["color_contributing"], _count(pos, lo, hi, res, ranges, col_test))
    rec.close()
