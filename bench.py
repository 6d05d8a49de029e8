"""Benchmark: particles/s of one reconstruct frame on the GB300.

Workload (default, the anisotropic 1M-particle frame): a 0.4 x 0.8 x 0.4
dam-break column + droplet (R 0.08) + splash, 2^20 particles, particle
radius r = 0.004, h = 4r; anisotropic (Yu13-family) field with lambda 0.9,
neighbour radius 4r, spatial cell 1.25h and grid spacing 0.5r (ratio 10);
seeded synthetic data.  A step is one whole frame: hashing -> sort ->
surface -> band -> smoothing -> covariance/G -> field -> marching cubes ->
mesh sizes read back.

Output: one JSON line on rank 0 (see the keys below).  With
``--impl reference`` the reference's own pipeline (its kernels compiled for
the host CPU, OpenMP over the launch domains; the CPU oracle port where that
build is absent) is timed on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the anisotropic 1M frame (headline)
    "aniso1m": dict(kind="dam_break", n=1 << 20, r=0.004, seed=2, method="yu13", smoothing_lambda=0.9,
                    aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0),
    # 8M particles: the 32^3-lattice generator at r = 0.002 (200^3 lattice, a 0.4 cube), anisotropic
    # field with the 1M frame's settings (grid spacing 0.5r: a 1020^3 scalar grid, 1.06e9 vertices)
    "aniso8m": dict(kind="lattice", n_side=200, r=0.002, seed=1, method="yu13", smoothing_lambda=0.9,
                    aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0),
    # the anisotropic frame at 2^18 particles (profiling captures)
    "aniso256k": dict(kind="dam_break", n=1 << 18, r=0.004, seed=2, method="yu13", smoothing_lambda=0.9,
                      aniso_radius_over_h=1.0, cell_size_scale=1.25, grid_ratio=10, iso=0.0),
    # the same frame with the plain ZB05 path (grid spacing 0.5r: ratio 8 at cell = h)
    "plain1m": dict(kind="dam_break", n=1 << 20, r=0.004, seed=2, method="zb05", grid_ratio=8),
    # the plain and Akinci12 paths at 2^18 particles (profiling captures)
    "plain256k": dict(kind="dam_break", n=1 << 18, r=0.004, seed=2, method="zb05", grid_ratio=8),
    "akinci256k": dict(kind="dam_break", n=1 << 18, r=0.004, seed=2, method="akinci12", grid_ratio=8),
    # 32^3 lattice, ZB05, grid spacing 0.5r
    "plain32k": dict(kind="lattice", n_side=32, r=0.0125, seed=1, method="zb05", grid_ratio=8),
}
METRIC = "particles/s recon (fwd, fwd+bwd) @1M aniso vs plain path; % HBM roofline"
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2


def make_frame(w):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    if w["kind"] == "dam_break":
        return synthetic.dam_break(w["n"], r=w["r"], seed=w["seed"])
    return synthetic.lattice_cube(w["n_side"], w["r"], seed=w["seed"])


def recon_kwargs(w):
    keys = ("smoothing_lambda", "aniso_radius_over_h", "cell_size_scale", "grid_ratio", "iso")
    return {k: w[k] for k in keys if k in w}


def oracle_params(w, fr):
    from oracle import pipeline as P
    return P.FrameParams(method=w["method"], h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass,
                         iso=w.get("iso"), ratio=w.get("grid_ratio"), cell_scale=w.get("cell_size_scale"),
                         lam=w.get("smoothing_lambda", 0.5),
                         aniso_radius=(w["aniso_radius_over_h"] * fr.h if "aniso_radius_over_h" in w else None))


def cpu_kind():
    """The reference's kernels built for this host when present, else the port."""
    from oracle import pipeline as P
    if P.available("ref"):
        try:
            P.load("ref")
            return "ref", "reference"
        except OSError:
            pass
    return "oracle32", "port"


def cpu_frame(w, fr):
    """One whole CPU frame (every stage, the field at every band vertex);
    returns (seconds, kind, threads, description of the sample)."""
    from oracle import pipeline as P
    kind, label = cpu_kind()
    threads = P.set_threads(kind, os.cpu_count() or 1)
    t0 = time.perf_counter()
    P.run_frame(kind, fr.pos, fr.density, fr.bbox_min, fr.bbox_max, oracle_params(w, fr))
    wall = time.perf_counter() - t0
    return wall, label, threads, f"one whole {fr.n}-particle frame, every stage, timed end to end"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"fsr_clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(kernel_key):
    """DRAM bytes per algorithmic byte of the kernel, from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return d.get(kernel_key)


PAIR_FLOPS = {"yu13": 33, "zb05": 16, "tc01": 12, "smooth": 14, "cov": 25}  # FP32 flops per pair
BATCH = dict(frames=64, n_lo=20000, n_hi=400000, seed=3, methods=("akinci12", "zb05", "yu13"),
             # grid spacing 0.5r everywhere (ratio 8 at cell = h); the anisotropic
             # frames use the 1M anisotropic frame's settings
             params={"akinci12": dict(grid_ratio=8), "zb05": dict(grid_ratio=8),
                     "yu13": dict(smoothing_lambda=0.9, aniso_radius_over_h=1.0, cell_size_scale=1.25,
                                  grid_ratio=10, iso=0.0)})


def batch_frames(cfg=BATCH):
    """64 frames, particle counts log-uniform in [20k, 400k], each the 32^3
    lattice generator rescaled to its count, field drawn per frame."""
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    rng = np.random.default_rng(cfg["seed"])
    out = []
    for i in range(cfg["frames"]):
        n = int(np.exp(rng.uniform(np.log(cfg["n_lo"]), np.log(cfg["n_hi"]))))
        m = cfg["methods"][int(rng.integers(len(cfg["methods"])))]
        out.append((m, synthetic.lattice_count(n, seed=cfg["seed"] * 1000 + i)))
    return out


def run_batch_leg(dev, stream, steps, warmup, flush, cfg=BATCH):
    """The batched forward (one graph launch for all frames) against the
    single-frame path on the same frames; both device-resident."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api
    frames = batch_frames(cfg)
    total = sum(fr.n for _, fr in frames)
    args = [(m, torch.from_numpy(fr.pos).to(dev), torch.from_numpy(fr.density).to(dev), api.header_of(fr))
            for m, fr in frames]
    b = api.Batch(dev.index or 0, params=cfg["params"])
    b.reconstruct(args, stream=stream)  # plan + autotune
    for _ in range(max(warmup - 1, 1)):
        b.reconstruct(args, stream=stream)
    torch.cuda.synchronize(dev)
    ms_b = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.reconstruct(args, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms_b.append(e0.elapsed_time(e1))
    tun = b.tuning()
    launches = int(tun.kernels_per_launch)
    b.close()
    recs = {m: api.Reconstructor(m, dev.index or 0, **cfg["params"][m]) for m in set(m for m, _ in frames)}
    for _ in range(warmup):
        for m, x, d, hdr in args:
            recs[m].reconstruct(x, d, hdr, stream)
    torch.cuda.synchronize(dev)
    ms_s = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for m, x, d, hdr in args:
            recs[m].reconstruct(x, d, hdr, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms_s.append(e0.elapsed_time(e1))
    for r in recs.values():
        r.close()
    tb, ts = float(np.mean(ms_b)), float(np.mean(ms_s))
    return {"frames": len(frames), "particle_range": [cfg["n_lo"], cfg["n_hi"]], "particles": total,
            "methods": {m: sum(1 for q, _ in frames if q == m) for m in cfg["methods"]},
            "value": total / (tb / 1e3), "ms_per_step": tb, "single_frame_value": total / (ts / 1e3),
            "single_frame_ms": ts, "speedup_vs_single_frame": ts / tb, "lanes": int(tun.lanes),
            "grid_div": int(tun.grid_div), "block_threads": int(tun.block_threads),
            "autotune_candidates": int(tun.n_candidates),
            "gpu_launches_per_step": launches,
            "note": "step = one fsr_reconstruct_batch call (inputs copied device-to-device, one graph launch, "
                    "one synchronisation); single frame = the same frames through fsr_reconstruct one by one"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def run_reference(args, w, fr):
    """--impl reference: the reference's pipeline on the host cores, whole
    frames (every stage, the field at every band vertex), W warm-up frames
    (at most one: a CPU frame has nothing to warm) and K timed frames."""
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return
    warmup, steps = min(args.warmup, 1), max(1, args.steps)
    for _ in range(warmup):
        cpu_frame(w, fr)
    secs = []
    label = threads = sample = None
    for _ in range(steps):
        s, label, threads, sample = cpu_frame(w, fr)
        secs.append(s)
    t = float(np.mean(secs))
    val = fr.n / t
    line = {"metric": METRIC, "value": val, "unit": "particles/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": f"synthetic ({fr.name}, seeded)",
            "config": {"workload": args.workload, "particles": fr.n, "method": w["method"]}, "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "particles/s", "cores": threads, "kind": label,
                             "sample": sample},
            "e2e": {"value": val, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _write_xyz_text(path, fr):
    """.xyz text of a frame (%.9g, data_format.txt layout), written with numpy."""
    with open(path, "w") as f:
        f.write("%.9g %.9g %.9g\n" % tuple(fr.bbox_min))
        f.write("%.9g %.9g %.9g\n" % tuple(fr.bbox_max))
        f.write("%.9g\n%.9g\n%.9g\n" % (fr.h, fr.particle_radius, fr.mass))
        np.savetxt(f, np.concatenate([fr.pos, fr.density[:, None]], axis=1).astype(np.float64), fmt="%.9g")


def _best_ms(fn, reps):
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, (time.perf_counter() - t0) * 1e3)
    return best


def run_io_leg(args, w):
    """File-driven frames (.xyz in, .obj out) through the reference's
    interface, with the library's parallel reader and writer, the .xyzb
    sidecar and the read/compute/write overlap; beside them the reference's
    stream-based reader and writer (oracle/io_port.cpp, one thread)."""
    import ctypes
    import shutil
    import tempfile
    from fluidsurfacereconstructiongpu_gb300 import api
    fr = make_frame(w)
    d = tempfile.mkdtemp(prefix="fsr_io_")
    nfr = 3
    try:
        for k in range(nfr):
            _write_xyz_text(os.path.join(d, "frame_%03d.xyz" % k), fr)
        x0 = os.path.join(d, "frame_000.xyz")
        cores = os.cpu_count() or 1
        io = {"particles": int(fr.n), "xyz_bytes": os.path.getsize(x0), "threads": cores}
        api.set_io_threads(1)
        io["read_xyz_ms_1thread"] = _best_ms(lambda: api.read_xyz(x0), 2)
        api.set_io_threads(0)
        io["read_xyz_ms"] = _best_ms(lambda: api.read_xyz(x0), 3)
        hdr, xyz, den = api.read_xyz(x0)
        b0 = os.path.join(d, "frame_000.xyzb")
        api.write_xyz_binary(b0, hdr, xyz, den)
        io["read_xyzb_ms"] = _best_ms(lambda: api.read_xyz_binary(b0), 3)
        port = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libio_port.so"))
        port.io_port_read_xyz.restype = ctypes.c_int64
        port.io_port_read_xyz.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
        port.io_port_write_obj.restype = ctypes.c_int
        port.io_port_write_obj.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
        hbuf = np.zeros(9, np.float32)
        pbuf = np.zeros((fr.n, 4), np.float32)
        io["port_read_xyz_ms"] = _best_ms(
            lambda: port.io_port_read_xyz(x0.encode(), hbuf.ctypes.data, pbuf.ctypes.data, fr.n), 1)
        assert np.array_equal(pbuf[:, :3], xyz) and np.array_equal(pbuf[:, 3], den)
        # one frame's mesh for the writers
        import torch
        rec = api.Reconstructor(w["method"], 0, **recon_kwargs(w))
        rec.reconstruct(torch.from_numpy(xyz).cuda(), torch.from_numpy(den).cuda(), hdr)
        mesh = rec.mesh()
        rec.close()
        o1 = os.path.join(d, "m.obj")
        api.set_io_threads(1)
        io["write_obj_ms_1thread"] = _best_ms(lambda: api.write_obj(o1, mesh), 1)
        api.set_io_threads(0)
        io["write_obj_ms"] = _best_ms(lambda: api.write_obj(o1, mesh), 3)
        io["obj_bytes"] = os.path.getsize(o1)
        o2 = os.path.join(d, "port.obj")
        pos = np.ascontiguousarray(mesh.positions, np.float32)
        nrm = np.ascontiguousarray(mesh.normals, np.float32)
        io["port_write_obj_ms"] = _best_ms(
            lambda: port.io_port_write_obj(o2.encode(), pos.ctypes.data, nrm.ctypes.data, pos.shape[0]), 1)
        with open(o1, "rb") as f1, open(o2, "rb") as f2:
            io["obj_identical_to_port"] = f1.read() == f2.read()
        os.remove(b0)
        # the file-driven loop: text, then with sidecars (made by a first run)
        loop = api.ReconstructorGPUOursYu13(d + os.sep, "frame_%03d", 0, nfr, **recon_kwargs(w))
        loop.setOutputMeshFile(True)
        loop.reconstruct()  # warm-up
        loop.reconstruct()
        t_text = loop.ioTiming()
        loop.setBinarySidecar(True)
        loop.reconstruct()  # writes the sidecars
        loop.reconstruct()
        t_side = loop.ioTiming()
        loop.setIndexedMesh(True)  # welded meshes (FSR_FLAG_WELD), indexed .obj
        loop.reconstruct()
        loop.reconstruct()
        t_weld = loop.ioTiming()
        io["indexed_obj_bytes"] = os.path.getsize(os.path.join(d, "frame_000.obj"))
        fields = ("read_ms", "upload_ms", "reconstruct_ms", "write_ms", "wall_ms")
        io["loop_text"] = {k: getattr(t_text, k) / nfr for k in fields}
        io["loop_sidecar"] = {k: getattr(t_side, k) / nfr for k in fields}
        io["loop_sidecar_indexed"] = {k: getattr(t_weld, k) / nfr for k in fields}
        # the reference's loop, serial: stream reader + frame + stream writer
        serial_ms = io["port_read_xyz_ms"] + io["loop_text"]["upload_ms"] + io["loop_text"]["reconstruct_ms"] + \
            io["port_write_obj_ms"]
        out = {
            "metric": "frames/s file-driven (.xyz -> mesh -> .obj) @1M aniso",
            "value": 1e3 / io["loop_sidecar"]["wall_ms"],
            "unit": "frames/s",
            "n_gpus": 1,
            "frames": nfr,
            "higher_is_better": True,
            "data": "synthetic (%s N=%d, seeded; %%.9g text)" % (w["kind"], fr.n),
            "config": {"workload": args.workload, "method": w["method"]},
            "text_value": 1e3 / io["loop_text"]["wall_ms"],
            "indexed_value": 1e3 / io["loop_sidecar_indexed"]["wall_ms"],
            "cpu_baseline": {"value": 1e3 / serial_ms, "unit": "frames/s", "cores": 1, "kind": "port",
                             "sample": "the reference's stream reader and writer (one thread) around this "
                                       "library's frame, no overlap"},
            "io": io,
        }
        print(json.dumps(out))
    finally:
        api.set_io_threads(0)
        shutil.rmtree(d, ignore_errors=True)


def reference_gpu_leg(workloads, steps, warmup):
    """The reference's own CUDA kernels on this GPU (its ReconstructionCUDA.cu
    built for sm_103a as a cubin, oracle/ref_gpu), driven through its
    kernel-level ABI in its frame order with its synchronisation after every
    launch (oracle/ref_gpu/flow.py).  Timed over the reference's timer scope
    (ReconstructorGPU.cpp:46-54): spatial hashing + the frame's stages."""
    from oracle.ref_gpu import flow
    if not flow.available("reference"):
        return {"unavailable": "the reference's kernels were not built (no reference sources where build() ran)"}
    L = flow.launchers("reference")
    flow.bind_tables(L)
    out = {"kind": "reference CUDA kernels (sm_103a cubin of its ReconstructionCUDA.cu) under a host "
                   "restatement of its frame loop; FMA contraction as nvcc's default",
           "steps": steps, "warmup": warmup}
    for name in workloads:
        w = WORKLOADS[name]
        fr = make_frame(w)
        prm = oracle_params(w, fr)
        for _ in range(warmup):
            flow.frame(L, w["method"], fr, prm, outputs=False)
        ts = []
        res = None
        for _ in range(steps):
            res, dt = flow.frame(L, w["method"], fr, prm, outputs=False)
            ts.append(dt)
        err = L.last_error()
        t = float(np.mean(ts))
        out[name] = {"ms_per_frame": t * 1e3, "value": fr.n / t, "unit": "particles/s",
                     "band_vertices": int(res["n_band"]), "triangles": int(res.get("n_mesh_vertices", 0)) // 3,
                     "launcher_error": err or None}
    return out


def pipeline_bytes(method, n, C, V, B, I, Q, T):
    """Algorithmic compulsory bytes of one forward frame and of its backward
    pass: every input read once, every output written once, every
    unavoidable intermediate written and read once (FP32 / u32)."""
    fwd = (16 * n + 16 * n + 16 * n + 8 * C + C / 8)      # hash + sort + ranges
    fwd += 8 * C + n / 8                                   # surface / involved flags
    fwd += V / 8 + V / 8 + 4 * B                           # band bitset, its scan, band list
    if method == "yu13":
        fwd += 12 * n + 12 * n                             # smoothing
        fwd += 12 * I + 36 * I + 4 * I                     # covariance + G
        fwd += 16 * n + 36 * I + 4 * B                     # field
    else:
        fwd += 16 * n + 4 * B                              # field
    fwd += 4 * B + 4 * B + 4 * Q                           # MC classify + compaction
    fwd += 4 * B + 24 * 3 * T                              # MC generation
    bwd = fwd + 24 * 3 * T + 16 * n + (2 * 36 * I if method == "yu13" else 0)
    return float(fwd), float(bwd)


def time_steps(fn, stream, steps, flush):
    """CUDA-event time of each of `steps` calls of fn on `stream`, L2 flushed
    (outside the events) before each."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def make_backward(rec, stream, dev, n):
    """fsr_backward of a fixed dL/d(mesh): the gradient of the mean squared
    deviation of the mesh vertices' distances to their centroid."""
    import ctypes as _ct
    import torch
    from fluidsurfacereconstructiongpu_gb300 import _native
    mpos, _ = rec.mesh_tensors(stream)
    c = mpos.mean(dim=0)
    d = mpos - c
    rr = d.norm(dim=1, keepdim=True).clamp_min(1e-12)
    gmesh = (2.0 * (rr - rr.mean()) / rr / mpos.shape[0] * d).contiguous()
    gx = torch.empty((n, 3), dtype=torch.float32, device=dev)

    def bwd():
        _native.check(_native.lib.fsr_backward(rec._h, _ct.c_void_p(gmesh.data_ptr()), _ct.c_void_p(gx.data_ptr()),
                                               None, _ct.c_void_p(stream.cuda_stream)), rec._h)
    return bwd


def frame_leg(w, fr, dev, stream, steps, warmup, flush, fp32_tflops, peak_gbs, backward=True):
    """One workload on the GPU: the frame timed clean (no instrumentation),
    then stage times from a separate instrumented pass, the pair counts of
    the neighbour-sum stages, forward + backward, and the rooflines."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, _native
    hdr = api.header_of(fr)
    xyz = torch.from_numpy(fr.pos).to(dev)
    den = torch.from_numpy(fr.density).to(dev)
    rec = api.Reconstructor(w["method"], dev.index or 0, **recon_kwargs(w))
    for _ in range(warmup):
        rec.reconstruct(xyz, den, hdr, stream)
    ms = time_steps(lambda: rec.reconstruct(xyz, den, hdr, stream), stream, steps, flush)
    st = rec.stats()
    t = float(np.mean(ms)) / 1e3
    out = {"workload": w, "particles": fr.n, "ms_per_step": t * 1e3, "value": fr.n / t,
           "band_vertices": int(st.n_band_vertices), "triangles": int(st.n_mesh_vertices) // 3,
           "involved_particles": int(st.n_involved_particles), "fp64_fallbacks": int(st.n_fp64_fallbacks),
           "scalar_grid": list(st.scalar_res), "launches_per_frame": int(st.n_kernel_launches)}
    # forward + backward (neighbour lists recomputed by the adjoints)
    if backward:
        bwd = make_backward(rec, stream, dev, fr.n)
        for _ in range(warmup):
            rec.reconstruct(xyz, den, hdr, stream)
            bwd()
        msfb = time_steps(lambda: (rec.reconstruct(xyz, den, hdr, stream), bwd()), stream, steps, flush)
        msb = time_steps(bwd, stream, steps, flush)
        out["fwd_bwd"] = {"value": fr.n / (float(np.mean(msfb)) / 1e3), "ms_per_step": float(np.mean(msfb)),
                          "backward_ms": float(np.mean(msb)),
                          "backward_launches": int(rec.stats().n_backward_launches)}
    # device memory of the leg: the library's pools plus the caller's inputs
    # and the backward pass's dL/dmesh and dL/dx buffers
    out["device_bytes"] = int(rec.stats().device_bytes)
    out["peak_device_bytes"] = out["device_bytes"] + 16 * fr.n + \
        ((12 * fr.n + 12 * int(st.n_mesh_vertices)) if backward else 0)
    pc = rec.pair_counts(stream)
    rec.close()
    # stage times: a separate handle with per-stage events
    rst = api.Reconstructor(w["method"], dev.index or 0, stage_timing=True, **recon_kwargs(w))
    for _ in range(warmup):
        rst.reconstruct(xyz, den, hdr, stream)
    stage = np.zeros(_native.NUM_STAGES)
    for _ in range(steps):
        flush.zero_()
        rst.reconstruct(xyz, den, hdr, stream)
        stage += np.array(list(rst.stats().stage_ms))
    rst.close()
    stage /= steps
    out["stage_ms"] = {k: round(float(v), 4) for k, v in zip(_native.STAGE_NAMES, stage)}
    # rooflines: the whole pipeline against HBM, the pair kernels against FP32
    C = int(np.prod(st.spatial_res))
    V = int(np.prod(st.scalar_res))
    fb, bb = pipeline_bytes(w["method"], fr.n, C, V, out["band_vertices"], out["involved_particles"],
                            int(st.n_valid_cubes), out["triangles"])
    out["pipeline_roofline"] = {"bound": "hbm", "unit": "GB/s", "peak": peak_gbs,
                                "fwd": {"bytes": fb, "achieved": fb / t / 1e9, "frac": fb / t / 1e9 / peak_gbs}}
    if backward:
        tfb = out["fwd_bwd"]["ms_per_step"] / 1e3
        out["pipeline_roofline"]["fwd_bwd"] = {"bytes": bb, "achieved": bb / tfb / 1e9,
                                               "frac": bb / tfb / 1e9 / peak_gbs}
    fp = {}
    kinds = [("field", "field", PAIR_FLOPS[w["method"]] if w["method"] in PAIR_FLOPS else 16)]
    if w["method"] == "yu13":
        kinds += [("smoothing", "smooth", PAIR_FLOPS["smooth"]), ("covariance", "cov", PAIR_FLOPS["cov"])]
    for stage_name, key, flops in kinds:
        ms_k = out["stage_ms"][stage_name]
        contrib, cand = pc[key + "_contributing"], pc[key + "_candidates"]
        ach = contrib * flops / (ms_k / 1e3) / 1e12 if ms_k > 0 else 0.0
        fp[stage_name] = {"candidate_pairs": cand, "contributing_pairs": contrib, "flops_per_pair": flops,
                          "stage_ms": ms_k, "achieved_tflops": ach, "peak_tflops": fp32_tflops,
                          "frac": ach / fp32_tflops if fp32_tflops else None}
    out["fp32_pipe"] = fp
    out["pair_counts"] = pc
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="aniso1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-backward", action="store_true", help="skip the forward+backward leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-frames legs")
    ap.add_argument("--no-extra", action="store_true", help="skip the plain-path and 8M legs")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the GPU baseline of the reference's own kernels")
    ap.add_argument("--compute-density", action="store_true",
                    help="frames without densities: the GPU computes them (FSR_FLAG_COMPUTE_DENSITY); "
                         "no backward or batch legs")
    ap.add_argument("--io", action="store_true",
                    help="time the file-driven loop (.xyz in, .obj out) instead of the in-memory frame")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: W warm-up frames, then one frame and one backward pass, nothing else")
    ap.add_argument("--weld", action="store_true", help="profiling run: weld the mesh (FSR_FLAG_WELD)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    args.warmup = max(args.warmup, 3) if args.impl == "ours" and not args.profile else args.warmup
    if args.io:
        run_io_leg(args, w)
        return
    if args.compute_density:
        args.no_backward = True
        args.no_batch = True
        args.no_extra = True

    if args.impl == "reference":
        fr = make_frame(w)
        run_reference(args, w, fr)
        return

    import torch
    from fluidsurfacereconstructiongpu_gb300 import api, _native

    if args.profile:
        torch.cuda.set_device(0)
        fr = make_frame(w)
        rec = api.Reconstructor(w["method"], 0, compute_density=args.compute_density, weld=args.weld,
                                **recon_kwargs(w))
        xyz = torch.from_numpy(fr.pos).cuda()
        den = None if args.compute_density else torch.from_numpy(fr.density).cuda()
        hdr = api.header_of(fr)
        stream = torch.cuda.current_stream()
        for _ in range(args.warmup + 1):
            rec.reconstruct(xyz, den, hdr, stream)
        if not args.no_backward and not args.compute_density:
            make_backward(rec, stream, torch.device("cuda", 0), fr.n)()
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.workload, "launches_per_frame": int(rec.stats().n_kernel_launches)}))
        rec.close()
        return

    world, rank, local, pg = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w_rank = dict(w)
    w_rank["seed"] = w["seed"] + rank  # replicas: independent frames of the same workload
    fr = make_frame(w_rank)

    # CPU baseline first (rank 0, N = 1), before any GPU work
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and fr.n <= (1 << 21):
        s, label, threads, sample = cpu_frame(w, fr)
        cpu = {"value": fr.n / s, "unit": "particles/s", "cores": threads, "kind": label, "sample": sample,
               "ms_per_frame": s * 1e3}

    # the reference's own CUDA kernels on this GPU (rank 0, N = 1)
    ref_gpu = None
    if rank == 0 and world == 1 and not args.no_reference_gpu and args.workload == "aniso1m" and \
            not args.compute_density:
        ref_gpu = reference_gpu_leg(("aniso1m", "plain1m"), min(args.steps, 5), 1)
        torch.cuda.synchronize(dev)
        torch.cuda.empty_cache()

    rec = api.Reconstructor(w["method"], local, compute_density=args.compute_density, **recon_kwargs(w))
    hdr = api.header_of(fr)
    xyz = torch.from_numpy(fr.pos).to(dev)
    den = None if args.compute_density else torch.from_numpy(fr.density).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        rec.reconstruct(xyz, den, hdr, stream)

    # the headline: whole frames, no per-stage events, nothing read back
    # between steps but what the frame itself reads (its sizes)
    if pg:
        pg.barrier()
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(local)
    ms = time_steps(lambda: rec.reconstruct(xyz, den, hdr, stream), stream, args.steps, flush)
    t_step = float(np.mean(ms)) / 1e3
    if pg:
        tt = torch.tensor([t_step], dtype=torch.float64, device=dev)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        t_step = float(tt.item())
    value = fr.n * world / t_step
    st = rec.stats()
    n_launch = int(st.n_kernel_launches)

    # the same workload's detail: stage times, pair counts, backward, rooflines
    fp32 = ctypes_fp32_rate(local)
    peak, peak_kind = measured_peaks()
    detail = None
    if not args.compute_density:
        detail = frame_leg(w_rank, fr, dev, stream, args.steps, args.warmup, flush, fp32, peak,
                           backward=not args.no_backward)
    extra = {}
    if not args.no_extra and world == 1 and args.workload == "aniso1m":
        for name in ("plain1m", "aniso8m"):
            wx = WORKLOADS[name]
            frx = make_frame(wx)
            extra[name] = frame_leg(wx, frx, dev, stream, min(args.steps, 10), args.warmup, flush, fp32, peak)
            del frx
        # the small plain workload (32^3 lattice, ZB05) at the reference's iso (-1e-4) and at 0.5
        extra["plain32k"] = {}
        for iso in (-1e-4, 0.5):
            wx = dict(WORKLOADS["plain32k"], iso=iso)
            frx = make_frame(wx)
            r32 = api.Reconstructor("zb05", local, **recon_kwargs(wx))
            h32 = api.header_of(frx)
            x32 = torch.from_numpy(frx.pos).to(dev)
            d32 = torch.from_numpy(frx.density).to(dev)
            for _ in range(args.warmup):
                r32.reconstruct(x32, d32, h32, stream)
            ms32 = time_steps(lambda: r32.reconstruct(x32, d32, h32, stream), stream, min(args.steps, 10), flush)
            s32 = r32.stats()
            extra["plain32k"]["iso %g" % iso] = {
                "particles": frx.n, "ms_per_step": float(np.mean(ms32)), "value": frx.n / (float(np.mean(ms32)) / 1e3),
                "band_vertices": int(s32.n_band_vertices), "triangles": int(s32.n_mesh_vertices) // 3}
            r32.close()
    batched = None
    if not args.no_batch:
        batched = run_batch_leg(dev, stream, min(args.steps, 10), args.warmup, flush)
        small = dict(BATCH, n_lo=20000, n_hi=60000, seed=5)
        batched["small_frames"] = run_batch_leg(dev, stream, min(args.steps, 10), args.warmup, flush, small)
    clocks = sampler.stop()  # sampled over every timed GPU leg above

    # end to end through the host API: pinned inputs in, mesh out, every step
    pin_xyz = torch.from_numpy(fr.pos).pin_memory()
    pin_den = torch.from_numpy(fr.density).pin_memory()
    nv = int(st.n_mesh_vertices)
    cap = int(nv * 1.2) + 1024
    out_pos = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
    out_nrm = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
    import ctypes
    e2e_t = []
    nvo = ctypes.c_uint64(0)
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        rc = _native.lib.fsr_reconstruct_host(rec._h, ctypes.byref(hdr), pin_xyz.data_ptr(),
                                              None if args.compute_density else pin_den.data_ptr(),
                                              fr.n, out_pos.data_ptr(), out_nrm.data_ptr(), cap,
                                              ctypes.byref(nvo), ctypes.c_void_p(stream.cuda_stream))
        _native.check(rc, rec._h)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_t.append(t1 - t0)
    e2e_single = float(np.mean(e2e_t))
    h2d = fr.n * (12 if args.compute_density else 16)
    d2h = int(nvo.value) * 24 + 64
    # the same steps as one pipelined sequence through fsr_reconstruct_host_frames: step k's upload and
    # step k - 1's read-back overlap step k's kernels; every step still copies its particles in and its
    # triangle soup out (into one of two output buffers, alternately)
    outs = [(out_pos, out_nrm), (torch.empty((cap, 3), dtype=torch.float32).pin_memory(),
                                 torch.empty((cap, 3), dtype=torch.float32).pin_memory())]

    def host_frames(count):
        arr = (_native.HostFrame * count)()
        for k in range(count):
            arr[k].header = hdr
            arr[k].xyz = pin_xyz.data_ptr()
            arr[k].density = None if args.compute_density else pin_den.data_ptr()
            arr[k].n = fr.n
            arr[k].out_pos, arr[k].out_nrm = outs[k % 2][0].data_ptr(), outs[k % 2][1].data_ptr()
            arr[k].capacity = cap
        return arr

    if args.warmup:
        _native.check(_native.lib.fsr_reconstruct_host_frames(rec._h, host_frames(args.warmup), args.warmup,
                                                              ctypes.c_void_p(stream.cuda_stream)), rec._h)
    seq = host_frames(args.steps)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    _native.check(_native.lib.fsr_reconstruct_host_frames(rec._h, seq, args.steps,
                                                          ctypes.c_void_p(stream.cuda_stream)), rec._h)
    e2e_step = (time.perf_counter() - t0) / args.steps
    assert all(seq[k].n_vertices == nvo.value for k in range(args.steps))

    # roofline of the dominant kernel (the field), from the instrumented pass
    roofline = None
    if detail is not None:
        field_ms = detail["stage_ms"]["field"]
        n_inv = detail["involved_particles"]
        B = detail["band_vertices"]
        if w["method"] == "yu13":
            alg_bytes = 16 * fr.n + 36 * n_inv + 8 * B  # smoothed particles + G read once, band ids read, field written
        else:
            alg_bytes = 16 * fr.n + 8 * B
        achieved = alg_bytes / (field_ms / 1e3) / 1e9
        tr = committed_traffic(f"{w['method']}_field_bytes_per_band_vertex")
        roofline = {"bound": "hbm", "kernel": "k_field_aniso_grouped" if w["method"] == "yu13"
                    else "k_field_iso_grouped", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": peak_kind, "traffic": (tr * B if tr else None),
                    "algorithmic_bytes": alg_bytes, "launch_ms": field_ms,
                    "note": "compute-bound: the FP32-pipe fraction (fp32_pipe) is the binding roofline"}

    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": f"synthetic ({fr.name}, seeded; L2 flushed between steps)",
            "config": {"workload": args.workload, "particles": fr.n, "method": w["method"],
                       "band_vertices": int(st.n_band_vertices), "triangles": int(st.n_mesh_vertices) // 3,
                       "device_bytes": int(st.device_bytes), "fp64_fallbacks": int(st.n_fp64_fallbacks),
                       "scalar_grid": list(st.scalar_res), "l2": "flushed (256 MB write) between steps",
                       "densities": "computed on the GPU (SPH, poly6)" if args.compute_density else "input",
                       "parallelism": "replicas" if world > 1 else "single",
                       "timing": "frames timed without per-stage events; stage times from a separate pass"},
            "e2e": {"value": fr.n / e2e_step, "unit": "particles/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "fsr_reconstruct_host_frames (the steps as one pipelined "
                    "sequence; no L2 flush between them: a frame's working set is "
                    f"{int(st.device_bytes) / 1e9:.1f} GB)",
                    "single_call": {"value": fr.n / e2e_single, "api": "fsr_reconstruct_host per step, L2 flushed "
                                    "before each"}},
            "fwd_bwd": detail.get("fwd_bwd") if detail else None,
            "stage_ms": detail["stage_ms"] if detail else None,
            "pipeline_roofline": detail["pipeline_roofline"] if detail else None,
            "fp32_pipe": detail["fp32_pipe"] if detail else None,
            "fp32_peak_tflops": {"value": fp32, "source": "measured (fsr_measure_fp32_rate, FMA chains)"},
            "plain_path": extra.get("plain1m"),
            "aniso8m": extra.get("aniso8m"),
            "plain32k": extra.get("plain32k"),
            "batched": batched,
            "gpu_launches": n_launch * args.steps,
            "roofline": roofline, "clocks": clocks, "cpu_baseline": cpu, "reference_gpu": ref_gpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    rec.close()
    if pg:
        pg.barrier()
        pg.destroy_process_group()


def ctypes_fp32_rate(device):
    import ctypes
    from fluidsurfacereconstructiongpu_gb300 import _native
    v = ctypes.c_double(0.0)
    _native.check(_native.lib.fsr_measure_fp32_rate(int(device), ctypes.byref(v)))
    return float(v.value)


if __name__ == "__main__":
    main()
