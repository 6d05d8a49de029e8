"""The .xyz reader, the .obj writer and the .xyzb sidecar (host code, no GPU).

The reader parses numbers in parallel with std::from_chars and hands anything
unusual to strtof, so every number must come out as libc's strtof gives it
(the reference reads with std::stringstream >> float, ReconstructorGPU.cpp:
200-290, which converts the same way).  The writer formats in parallel with
std::to_chars and must give libc printf("%g") byte for byte (std::ostream's
default float output, ReconstructorGPUOurs.cpp:58-99), whatever the thread
count.
"""
import ctypes
import os
import struct

import numpy as np
import pytest

libc = ctypes.CDLL(None)
libc.strtof.restype = ctypes.c_float
libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
libc.snprintf.restype = ctypes.c_int


def _strtof(tok: str) -> int:
    return struct.unpack("<I", struct.pack("<f", libc.strtof(tok.encode(), None)))[0]


def _g(x) -> bytes:
    buf = ctypes.create_string_buffer(64)
    libc.snprintf(buf, 64, b"%g", ctypes.c_double(float(x)))
    return buf.value


def _tokens(rng, n):
    """Numbers written in the ways an .xyz may hold them."""
    out = []
    for i in range(n):
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-8, 8))
        kind = i % 12
        if kind == 0:
            out.append("%.9g" % v)
        elif kind == 1:
            out.append("%.3f" % v)
        elif kind == 2:
            out.append("%e" % v)
        elif kind == 3:
            out.append("+%.6g" % abs(v))
        elif kind == 4:
            out.append(float(np.float32(v)).hex())          # hex float: strtof reads it
        elif kind == 5:
            out.append("%.25g" % v)                          # more digits than a float holds
        elif kind == 6:
            out.append("%.1e" % (abs(v) * 1e-40))            # subnormal or zero
        elif kind == 7:
            out.append("%.3e" % (abs(v) * 1e38))             # near or beyond FLT_MAX
        elif kind == 8:
            out.append("%d" % int(v))
        elif kind == 9:
            out.append(("%.8f" % v).rstrip("0"))             # trailing point: "12."
        elif kind == 10:
            out.append("." + "%d" % rng.integers(0, 10**7))  # no leading digit
        else:
            # halfway between two floats: the correctly rounded result is even
            f = np.float32(abs(v) + 1.0)
            nxt = np.nextafter(f, np.float32(np.inf))
            out.append("%.20g" % ((float(f) + float(nxt)) / 2))
    return out


@pytest.mark.parametrize("threads", [1, 7])
def test_reader_matches_strtof(tmp_path, threads):
    from fluidsurfacereconstructiongpu_gb300 import api
    rng = np.random.default_rng(11)
    toks = _tokens(rng, 4 * 30011)
    seps = [" ", "\t", "  ", " \t "]
    path = tmp_path / "f.xyz"
    with open(path, "w") as f:
        f.write("0 0 0\n1 1 1\n0.05\n0.0125\n0.001\n")
        for i in range(0, len(toks), 4):
            sep = seps[(i // 4) % 4]
            f.write(sep.join(toks[i:i + 4]) + ("\r\n" if i % 7 == 0 else "\n"))
            if i % 1000 == 0:
                f.write("   \n")  # blank lines are skipped
    api.set_io_threads(threads)
    try:
        hdr, xyz, den = api.read_xyz(str(path))
    finally:
        api.set_io_threads(0)
    got = np.concatenate([xyz, den[:, None]], axis=1).reshape(-1).view(np.uint32)
    want = np.array([_strtof(t) for t in toks], np.uint32)
    assert got.shape == want.shape
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, [(toks[i], hex(got[i]), hex(want[i])) for i in bad[:5]]
    assert hdr.particle_mass == np.float32(0.001)


def test_reader_rejects_what_strtof_rejects(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, _native
    head = "0 0 0\n1 1 1\n0.1\n0.01\n0.001\n"
    for body in ["1 2 3\n", "1 2 3 4 5\n", "1 2 3 x\n", "+-1 2 3 4\n", "1 2 3 4e\n", "1,2,3,4\n"]:
        p = tmp_path / "bad.xyz"
        p.write_text(head + "0.5 0.5 0.5 1000\n" + body)
        with pytest.raises(_native.FsrError) as e:
            api.read_xyz(str(p))
        assert e.value.status == 6, body


def test_obj_matches_printf(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api
    rng = np.random.default_rng(5)
    nv = 3 * 41000  # more than one block of lines per thread
    pos = (rng.standard_normal((nv, 3)) * 10.0 ** rng.integers(-6, 6, (nv, 1))).astype(np.float32)
    special = np.array([0.0, -0.0, 0.001953125, 1234565.0, 1e-5, -1e-5, 123456.5, 999999.5, 0.5, 3.4028235e38,
                        1.4e-45, np.inf, -np.inf, 1e16, 100000.0, 1000000.0], np.float32)
    pos[: special.size, 0] = special
    nrm = rng.standard_normal((nv, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[:3] = [[np.nan, 0, 1], [-0.0, 0.0, 1.0], [1e-20, -1e-20, 0.75]]
    lines = [b"v " + b" ".join(_g(x) for x in p) + b"\n" for p in pos]
    lines += [b"vn " + b" ".join(_g(x) for x in p) + b"\n" for p in nrm]
    lines += [b"f %d//%d %d//%d %d//%d \n" % (i, i, i + 1, i + 1, i + 2, i + 2) for i in range(1, nv + 1, 3)]
    want = b"".join(lines)
    mesh = api.Mesh(positions=pos, normals=nrm)
    for threads in (1, 3, 8):
        api.set_io_threads(threads)
        out = tmp_path / f"m{threads}.obj"
        try:
            api.write_obj(str(out), mesh)
        finally:
            api.set_io_threads(0)
        got = out.read_bytes()
        if got != want:
            a, b = got.split(b"\n"), want.split(b"\n")
            k = next(i for i in range(min(len(a), len(b))) if a[i] != b[i])
            raise AssertionError((threads, k, a[k], b[k]))


def test_empty_obj(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api
    out = tmp_path / "e.obj"
    api.write_obj(str(out), api.Mesh(positions=np.zeros((0, 3), np.float32), normals=np.zeros((0, 3), np.float32)))
    assert out.read_bytes() == b""


def test_sidecar_roundtrip(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic, _native
    fr = synthetic.lattice_cube(9, 0.0125, seed=3)
    xyz_path = str(tmp_path / "a.xyz")
    api.write_xyz(xyz_path, fr)
    hdr, xyz, den = api.read_xyz(xyz_path)
    b = str(tmp_path / "a.xyzb")
    api.write_xyz_binary(b, hdr, xyz, den)
    assert os.path.getsize(b) == 80 + 16 * xyz.shape[0]
    hdr2, xyz2, den2 = api.read_xyz_binary(b)
    assert np.array_equal(xyz2.view(np.uint32), xyz.view(np.uint32))
    assert np.array_equal(den2.view(np.uint32), den.view(np.uint32))
    assert bytes(hdr2) == bytes(hdr)
    # empty particle set
    e = str(tmp_path / "e.xyzb")
    api.write_xyz_binary(e, hdr, np.zeros((0, 3), np.float32), np.zeros(0, np.float32))
    assert api.read_xyz_binary(e)[1].shape == (0, 3)
    # a truncated file and a foreign file are format errors
    data = open(b, "rb").read()
    open(b, "wb").write(data[:-4])
    with pytest.raises(_native.FsrError) as ex:
        api.read_xyz_binary(b)
    assert ex.value.status == 6
    open(b, "wb").write(b"NOTXYZB1" + data[8:])
    with pytest.raises(_native.FsrError) as ex:
        api.read_xyz_binary(b)
    assert ex.value.status == 6
    with pytest.raises(_native.FsrError) as ex:
        api.read_xyz_binary(str(tmp_path / "missing.xyzb"))
    assert ex.value.status == 5


@pytest.mark.gpu
def test_files_loop_with_sidecar(tmp_path):
    """The pipelined file loop gives the same .obj files with and without the
    sidecar; a stale sidecar (the .xyz changed) is ignored and rewritten."""
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    d = tmp_path
    for k in range(3):
        api.write_xyz(str(d / f"frame_{k:03d}.xyz"), synthetic.lattice_cube(10 + k, 0.0125, seed=k))
    r = api.ReconstructorGPUOursZB05(str(d) + "/", "frame_%03d", 0, 3)
    r.setOutputMeshFile(True)
    r.reconstruct()
    plain = [(d / f"frame_{k:03d}.obj").read_bytes() for k in range(3)]
    assert all(len(p) > 0 for p in plain)
    r.setBinarySidecar(True)
    r.reconstruct()   # parses the .xyz files and writes their sidecars
    assert all((d / f"frame_{k:03d}.xyzb").exists() for k in range(3))
    r.reconstruct()   # reads the sidecars
    assert [(d / f"frame_{k:03d}.obj").read_bytes() for k in range(3)] == plain
    tm = r.ioTiming()
    assert tm.wall_ms > 0 and tm.read_ms > 0 and tm.write_ms > 0
    # replace frame 1's particles: its sidecar is stale and must not be used
    api.write_xyz(str(d / "frame_001.xyz"), synthetic.lattice_cube(12, 0.0125, seed=9))
    os.utime(d / "frame_001.xyz", ns=(1, 1))
    r.reconstruct()
    via_sidecar_mode = (d / "frame_001.obj").read_bytes()
    assert via_sidecar_mode != plain[1]
    r2 = api.ReconstructorGPUOursZB05(str(d) + "/", "frame_%03d", 1, 2)
    r2.setOutputMeshFile(True)
    (d / "frame_001.obj").unlink()
    r2.reconstruct()
    assert (d / "frame_001.obj").read_bytes() == via_sidecar_mode
    _, xyz_b, _ = api.read_xyz_binary(str(d / "frame_001.xyzb"))
    _, xyz_t, _ = api.read_xyz(str(d / "frame_001.xyz"))
    assert np.array_equal(xyz_b, xyz_t)


def test_same_bytes_as_the_stream_code(tmp_path):
    """The reference's stream-based reader and writer (restated in
    oracle/io_port.cpp) give the same particles and the same .obj bytes."""
    import subprocess
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    so = os.path.join(os.path.dirname(__file__), "..", "oracle", "_build", "libio_port.so")
    if not os.path.exists(so):
        subprocess.run(["bash", os.path.join(os.path.dirname(so), "..", "build_oracle.sh")], check=True,
                       capture_output=True)
    port = ctypes.CDLL(so)
    port.io_port_read_xyz.restype = ctypes.c_int64
    port.io_port_read_xyz.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    port.io_port_write_obj.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    fr = synthetic.dam_break(20000, r=0.004, seed=4)
    x = str(tmp_path / "a.xyz")
    api.write_xyz(x, fr)
    hdr, xyz, den = api.read_xyz(x)
    hb = np.zeros(9, np.float32)
    pb = np.zeros((fr.n, 4), np.float32)
    assert port.io_port_read_xyz(x.encode(), hb.ctypes.data, pb.ctypes.data, fr.n) == fr.n
    assert np.array_equal(pb[:, :3].view(np.uint32), xyz.view(np.uint32))
    assert np.array_equal(pb[:, 3].view(np.uint32), den.view(np.uint32))
    assert np.array_equal(hb[[6, 7, 8]], np.array([hdr.kernel_radius, hdr.particle_radius, hdr.particle_mass],
                                                  np.float32))
    rng = np.random.default_rng(2)
    nv = 3 * 5000
    pos = (rng.random((nv, 3)) * 0.8).astype(np.float32)
    nrm = rng.standard_normal((nv, 3)).astype(np.float32)
    a, b = str(tmp_path / "a.obj"), str(tmp_path / "b.obj")
    api.write_obj(a, api.Mesh(positions=pos, normals=nrm))
    port.io_port_write_obj(b.encode(), pos.ctypes.data, nrm.ctypes.data, nv)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_indexed_obj_writer(tmp_path):
    """Host-only: the indexed .obj layout, and out-of-range indices rejected."""
    from fluidsurfacereconstructiongpu_gb300 import api, _native
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    nrm = np.ones((4, 3), np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    out = tmp_path / "w.obj"
    api.write_obj(str(out), api.IndexedMesh(pos, nrm, tri))
    lines = out.read_text().splitlines()
    assert lines[:4] == ["v 0 0 0", "v 1 0 0", "v 0 1 0", "v 0 0 1"]
    assert lines[4:8] == ["vn 1 1 1"] * 4
    assert lines[8:] == ["f 1//1 2//2 3//3 ", "f 1//1 3//3 4//4 "]
    with pytest.raises(_native.FsrError) as e:
        api.write_obj(str(out), api.IndexedMesh(pos, nrm, np.array([[0, 1, 4]], np.uint32)))
    assert e.value.status == 1
