"""Generates tests/golden/*.npz from the reference's own kernels.

Run where the reference sources are available (oracle/build_ref.sh must have
produced oracle/_ref/libfsr_refkernels.so):

    python tests/golden/make_golden.py

Each fixture holds one seeded frame: its inputs and every stage output of
the reference's kernels compiled for the host (thrust's sort and scans
replaced by their exact definitions, see oracle/pipeline.py).  The tests
check the CPU oracle against these files, so the oracle stays pinned to the
reference where the reference itself is absent.  Also written:
mc_tables.json, a SHA-256 of the reference's marching-cubes tables.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fluidsurfacereconstructiongpu_gb300 import synthetic  # noqa: E402
from oracle import pipeline as P  # noqa: E402

# the reference checkout, as the oracle's build recipe resolves it (REF_ROOT)
REF_ROOT = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "--print-root"],
                          capture_output=True, text=True, check=True).stdout.strip()

CASES = [
    # name, method, frame factory, extra params
    ("zb05_lattice12", "zb05", lambda: synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3)), {}),
    ("tc01_lattice12", "tc01", lambda: synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3)), {}),
    ("akinci_lattice12", "akinci", lambda: synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3)), {}),
    ("yu13_lattice12", "yu13", lambda: synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3)), {}),
    ("zb05_lattice16_ratio8", "zb05", lambda: synthetic.lattice_cube(16, 0.0125, seed=3, origin=(0.2, 0.2, 0.2)),
     {"ratio": 8}),
    ("yu13_lattice14_seed5", "yu13", lambda: synthetic.lattice_cube(14, 0.0125, seed=5, origin=(0.35, 0.3, 0.25)),
     {}),
    ("zb05_format_example", "zb05", synthetic.format_example, {}),
    ("yu13_format_example", "yu13", synthetic.format_example, {}),
    ("akinci_format_example", "akinci", synthetic.format_example, {}),
]


def params_for(method, fr, extra):
    return P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass, **extra)


def fixture(fr, o):
    d = dict(pos=fr.pos, density=fr.density, bbox_min=fr.bbox_min, bbox_max=fr.bbox_max,
             header=np.array([fr.h, fr.particle_radius, fr.mass], np.float32),
             keys=o.keys, perm=o.perm, sflag_idx=np.flatnonzero(o.sflag).astype(np.uint32),
             occupied=np.flatnonzero(o.ranges[:, 0] != 0xFFFFFFFF).astype(np.uint32),
             sv=o.sv, phi_band=o.phi[o.sv].astype(np.float32), valid_idx=o.valid_idx,
             mesh_pos=o.mesh_pos.astype(np.float32), mesh_nrm=o.mesh_nrm.astype(np.float32),
             n_cells=np.array([o.spatial.count], np.uint64), n_vertices=np.array([o.scalar.count], np.uint64))
    d["ranges_occupied"] = o.ranges[d["occupied"]]
    if o.nverts is not None:
        d["nverts_valid"] = o.nverts[o.valid_idx]
    if o.method == "yu13":
        nz = np.flatnonzero(o.ninv)
        d.update(ninv_idx=nz.astype(np.uint32), ninv_val=o.ninv[nz], mean=o.mean.astype(np.float32),
                 smoothed=o.smoothed.astype(np.float32), inv=o.inv, G=o.G.astype(np.float32))
    return d


def table_hash():
    src = open(os.path.join(REF_ROOT, "FluidSurfaceReconstruction", "GPU", "MarchingCubesHelper.cpp")).read()
    blk = src[src.index("edgeIndexesOfTriangle[256][16]"):src.index("numVertices[256]")]
    rows = re.findall(r"\{([-0-9,\s]+)\}", blk)
    tri = [[int(x) for x in r.split(",")] for r in rows]
    ef_blk = src[src.index("edgeFlags[256]"):src.index("edgeIndexesOfTriangle[256][16]")]
    ef = [int(x, 16) for x in re.findall(r"0x[0-9a-fA-F]+", ef_blk)]
    nv_blk = src[src.index("numVertices[256]"):src.index("getCornerIndexes3D")]
    nv = [int(x) for x in re.findall(r"\b\d+\b", nv_blk.split("{", 1)[1])][:256]
    h = lambda obj: hashlib.sha256(json.dumps(obj).encode()).hexdigest()  # noqa: E731
    return {"triangle_table_sha256": h(tri), "edge_flags_sha256": h(ef), "num_vertices_sha256": h(nv)}


def main():
    if not P.available("ref"):
        sys.exit("oracle/_ref/libfsr_refkernels.so missing: run oracle/build_ref.sh first")
    for name, method, make, extra in CASES:
        fr = make()
        o = P.run_frame("ref", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, params_for(method, fr, extra))
        d = fixture(fr, o)
        d["method"] = np.array(method)
        d["extra"] = np.array(json.dumps(extra))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(f"{name}: N={fr.n} B={o.sv.size} T={o.n_triangles}")
    json.dump(table_hash(), open(os.path.join(HERE, "mc_tables.json"), "w"), indent=1)
    print("mc_tables.json written")


if __name__ == "__main__":
    main()
