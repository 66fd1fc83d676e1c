"""The C++ layer over the C-ABI (include/vecgeom_gb300.hpp: SOA3D, NavStatePool, PlacedVolume,
UnplacedVolume, GlobalLocator, BVHNavigator in the reference's method shapes). A small C++
program (tests/cpp/adapter_check.cpp) loads a saved barrel geometry and runs every wrapped
call; its outputs must equal, bit for bit, the same calls made through the C-ABI from Python
(which the other GPU tests hold to the oracle). On CPU the program is compiled and linked."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp")


def build_check(tmp_path):
    import __graft_entry__
    from vecgeom_gb300 import build as b

    __graft_entry__.build()
    exe = str(tmp_path / "adapter_check")
    libdir = os.path.dirname(b.LIB)
    cmd = [b._nvcc(), "-std=c++17", "-O2", "-x", "c++", SRC, "-I", os.path.join(ROOT, "include"), "-L", libdir,
           "-lvecgeom_gb300", "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_adapter_compiles_and_links(tmp_path):
    assert os.path.exists(build_check(tmp_path))


def _inputs(n):
    from vecgeom_gb300 import workloads as W
    (x, y, z), (dx, dy, dz) = W.tracks_in_cylinder(n // 2, seed=31)
    g = W.rng(31, 2)
    r = 1250.0 * np.sqrt(g.random(n - n // 2))
    ph = 2 * np.pi * g.random(n - n // 2)
    wz = 600.0 * (2 * g.random(n - n // 2) - 1)
    wd = W.isotropic(W.rng(31, 3), n - n // 2)
    pts = [np.concatenate([a, b]) for a, b in zip((x, y, z), (r * np.cos(ph), r * np.sin(ph), wz))]
    dirs = [np.concatenate([a, b]) for a, b in zip((dx, dy, dz), wd)]
    return [np.ascontiguousarray(a, dtype=np.float64) for a in (*pts, *dirs)]


@pytest.mark.gpu
def test_adapter_matches_c_abi(cuda, tmp_path):
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W

    torch = cuda
    exe = build_check(tmp_path)
    geo = vg.Geometry()
    W.build_barrel(geo)
    gpath = str(tmp_path / "barrel.geom")
    geo.save(gpath)
    n = 1 << 14
    arrs = _inputs(n)
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.uint64(n).tobytes())
        for a in arrs:
            f.write(a.tobytes())
    pv = geo.info()["n_pv"] - 2  # the outermost layer's tube, placed in the world
    shape = 3                    # the first layer's tube shape
    r = subprocess.run([exe, gpath, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(pv), str(shape)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = open(tmp_path / "out.bin", "rb").read()
    pos = 0

    def take(dtype, count=n):
        nonlocal pos
        dt = np.dtype(dtype)
        a = np.frombuffer(got, dtype=dt, count=count, offset=pos)
        pos += dt.itemsize * count
        return a

    dev = [torch.from_numpy(a).to("cuda:0") for a in arrs]
    x, y, z, dx, dy, dz = dev
    for kind in ("placed", "unplaced"):
        ins = torch.empty(n, dtype=torch.int32, device="cuda:0")
        con = torch.empty(n, dtype=torch.uint8, device="cuda:0")
        d = [torch.empty(n, dtype=torch.float64, device="cuda:0") for _ in range(4)]
        if kind == "placed":
            geo.inside(pv, x, y, z, ins)
            geo.contains(pv, x, y, z, con)
            geo.distance_to_in(pv, x, y, z, dx, dy, dz, d[0])
            geo.distance_to_out(pv, x, y, z, dx, dy, dz, d[1])
            geo.safety_to_in(pv, x, y, z, d[2])
            geo.safety_to_out(pv, x, y, z, d[3])
        else:
            geo.shape_query("inside", shape, x, y, z, ins)
            geo.shape_query("contains", shape, x, y, z, con)
            geo.shape_query("distance_to_in", shape, x, y, z, d[0], dx, dy, dz)
            geo.shape_query("distance_to_out", shape, x, y, z, d[1], dx, dy, dz)
            geo.shape_query("safety_to_in", shape, x, y, z, d[2])
            geo.shape_query("safety_to_out", shape, x, y, z, d[3])
        assert np.array_equal(take(np.int32), ins.cpu().numpy()), kind
        assert np.array_equal(take(np.uint8), con.cpu().numpy()), kind
        for k, a in enumerate(d):
            assert np.array_equal(take(np.float64).view(np.uint64), a.cpu().numpy().view(np.uint64)), (kind, k)

    st = torch.empty(n * 12, dtype=torch.uint8, device="cuda:0")
    geo.locate_point(x, y, z, st)
    assert np.array_equal(take(np.uint8, 12 * n), st.cpu().numpy())
    out = torch.empty(n * 12, dtype=torch.uint8, device="cuda:0")
    step = torch.empty(n, dtype=torch.float64, device="cuda:0")
    for flags in (vg.PREC_FP64, vg.PREC_MIXED | vg.NAV_SORT | vg.NAV_QUEUE):
        geo.compute_step_and_next_volume(x, y, z, dx, dy, dz, st, out, step, flags=flags)
        assert np.array_equal(take(np.uint8, 12 * n), out.cpu().numpy()), flags
        assert np.array_equal(take(np.float64).view(np.uint64), step.cpu().numpy().view(np.uint64)), flags
    saf = torch.empty(n, dtype=torch.float64, device="cuda:0")
    geo.compute_step_and_safety(x, y, z, dx, dy, dz, st, out, step, saf)
    assert np.array_equal(take(np.uint8, 12 * n), out.cpu().numpy())
    assert np.array_equal(take(np.float64).view(np.uint64), step.cpu().numpy().view(np.uint64))
    assert np.array_equal(take(np.float64).view(np.uint64), saf.cpu().numpy().view(np.uint64))
    assert pos == len(got)
    # the located states are real states (not all outside the world), so the steps were exercised
    assert (st.cpu().numpy().view(vg.NAVSTATE_DTYPE)["nav_ind"] != 0).mean() > 0.9
