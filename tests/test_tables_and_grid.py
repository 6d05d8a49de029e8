"""Marching-cubes tables and grid derivation (CPU only)."""
import hashlib
import json
import os
import re

import numpy as np

from oracle import pipeline as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def _packed_table(path, name):
    src = open(path).read()
    blk = src[src.index(name):]
    blk = blk[blk.index("{") + 1:blk.index("};")]
    vals = [int(x, 16) for x in re.findall(r"0x([0-9a-f]{16})ULL", blk)]
    assert len(vals) == 256
    out = []
    for v in vals:
        row = []
        for k in range(16):
            nib = (v >> (4 * k)) & 0xF
            if nib == 0xF:
                break
            row.append(nib)
        out.append(row)
    return out


def _as_reference_rows(tri):
    return [r + [-1] * (16 - len(r)) for r in tri]


def _sha(obj):
    return hashlib.sha256(json.dumps(obj).encode()).hexdigest()


def test_tables_equal_the_reference_tables():
    ref = json.load(open(os.path.join(GOLDEN, "mc_tables.json")))
    for path, name in ((os.path.join(ROOT, "oracle", "fsr_mc_tables.h"), "FSR_O_TRI[256]"),
                       (os.path.join(ROOT, "fluidsurfacereconstructiongpu_gb300", "csrc", "mc_tables.h"),
                        "kTriPacked[256]")):
        tri = _packed_table(path, name)
        assert _sha(_as_reference_rows(tri)) == ref["triangle_table_sha256"], path
        ef = []
        for c in range(256):
            m = 0
            for e, (a, b) in enumerate(EDGES):
                if ((c >> a) & 1) != ((c >> b) & 1):
                    m |= 1 << e
            ef.append(m)
        assert _sha(ef) == ref["edge_flags_sha256"]
        assert _sha([len(r) for r in tri]) == ref["num_vertices_sha256"]


def test_table_self_consistency():
    tri = _packed_table(os.path.join(ROOT, "oracle", "fsr_mc_tables.h"), "FSR_O_TRI[256]")
    for c, row in enumerate(tri):
        assert len(row) % 3 == 0 and len(row) <= 15
        cut = {e for e, (a, b) in enumerate(EDGES) if ((c >> a) & 1) != ((c >> b) & 1)}
        assert set(row) <= cut  # triangles only use cut edges
        assert (len(row) == 0) == (c in (0, 255))
        # complementary cases cut the same edges
        cut2 = {e for e, (a, b) in enumerate(EDGES) if (((255 - c) >> a) & 1) != (((255 - c) >> b) & 1)}
        assert cut == cut2


def test_grid_derivation_known_answers():
    # unit box, h = 0.05: (1.1 / 0.05 + 1) in FP32 truncates to 22, not 23
    sp, sc = P.grid_derive([0, 0, 0], [1, 1, 1], 0.05, 1.0, 8)
    assert sp.resolution == (22, 22, 22)
    assert sc.resolution == (176, 176, 176)
    # independent FP32 evaluation of the same expression
    cs = np.float32(0.05) * np.float32(1.0)
    mn, mx = np.float32(0) - cs, np.float32(1) + cs
    assert int(np.float32((mx - mn) / cs) + np.float32(1)) == 22
    sp, sc = P.grid_derive([0, 0, 0], [1, 1, 1], 0.016, 1.25, 10)
    assert sp.resolution == (52, 52, 52) and sc.resolution == (520, 520, 520)
