"""Host-side logic of libpms, CPU only: the library loads and exports every
symbol include/pms.h declares; config.txt parsing follows the reference's INI
rules and defaults; parameter and grid derivation match the oracle bit for
bit; VTK frames round-trip; the PLY writer produces tinyply 2.3's ASCII
layout; the marching-cubes tables in use are the reference's."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden, golden_cases


def test_library_exports_every_declared_symbol(pms_lib):
    header = open(os.path.join(ROOT, "include", "pms.h")).read()
    body = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    names = set(re.findall(r"\b(pms_[a-z_0-9]+)\s*\(", body))
    assert len(names) >= 30
    L = pms_lib.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_config_parsing_reference_rules(pms_lib, tmp_config):
    text = "\n".join([
        "; leading comment",
        "[Sim]",
        "Mass = 2   ; inline comment",
        "ParticleSpacing = 0.005",
        "[Surface]",
        "SmoothingRadiusRatio = 4.9",
        "isovalue = 0.25",
        "[Diffuse]",
        "MinKineticEnergyThreshold = 5.0.",
        "TimeStep = 0.02#not a comment",
        "// a line without an equals sign is skipped",
        "[Config]",
        "IsSurfaceReconstruct = yes",
        "IsDiffuseGeneration = off",
        "FluidPath = ../frames/",
        "Framefrom = 3.7",
    ])
    c = pms_lib.load_config(tmp_config(text))
    assert c.mass == 2.0 and c.particle_spacing == 0.005
    assert c.smoothing_radius_ratio == 4.9 and c.iso_value == 0.25
    assert c.min_kinetic_energy == 5.0 and c.time_step == 0.02
    assert c.is_surface == 1 and c.is_diffuse == 0
    assert c.fluid_path == b"../frames/" and c.frame_start == 3
    # defaults of Params.cpp for keys that are absent
    assert c.min_num_neighbors == 8 and c.lambda_for_smoothed == 0.5 and c.sc_scale == 2
    assert c.frame_end == 10 and c.num_zeros == 4
    p = pms_lib.derive_params(c)
    assert p.smoothing_radius_ratio == 4 and p.h == np.float32(4) * np.float32(0.005)


def test_missing_config_is_an_error(pms_lib):
    with pytest.raises(pms_lib.PmsError) as ei:
        pms_lib.load_config("/nonexistent/config.txt")
    assert ei.value.status == 6


@pytest.mark.parametrize("over", [{}, {"surface.smoothingradiusratio": 4}, {"sim.particlespacing": 0.005},
                                  {"domain.sclargridsizescale": 3, "sim.particlespacing": 0.1}])
def test_params_and_grid_match_oracle(pms_lib, oracle, tmp_config, over):
    from postmps_gb300 import synth
    text = synth.config_text(**over)
    p = pms_lib.derive_params(pms_lib.load_config(tmp_config(text)))
    po = oracle.derive_params(oracle.config_from_keys(oracle.parse_ini(text)))
    for f, _ in pms_lib.Params._fields_:
        assert getattr(p, f) == getattr(po, f), f
    rng = np.random.default_rng(3)
    for _ in range(20):
        pos = (rng.random((50, 3)) * rng.random() * 3 - 1).astype(np.float32)
        g = pms_lib.grid_from_bbox(p, pos.min(0), pos.max(0))
        go = oracle.grid_from_positions(po, pos)
        for f, _ in pms_lib.Grid._fields_:
            a, b = getattr(g, f), getattr(go, f)
            a = list(a) if hasattr(a, "__len__") else a
            b = list(b) if hasattr(b, "__len__") else b
            assert a == b, f


@pytest.mark.parametrize("case", golden_cases())
def test_grid_matches_reference_fixture(pms_lib, tmp_config, case):
    d = load_golden(case)
    p = pms_lib.derive_params(pms_lib.load_config(tmp_config(d["config"])))
    g = pms_lib.grid_from_bbox(p, d["pos"].min(0), d["pos"].max(0))
    np.testing.assert_array_equal(np.array(g.min_pos[:]), d["min_pos"])
    np.testing.assert_array_equal(np.array(g.scmin_pos[:]), d["scmin_pos"])
    np.testing.assert_array_equal(np.array(g.spres[:]), d["spres"])
    np.testing.assert_array_equal(np.array(g.scres[:]), d["scres"])


@pytest.mark.parametrize("n", [1000, 400_000])
def test_vtk_round_trip_binary(pms_lib, tmp_path, n):
    # 400k particles take the threaded decode (more than 262144 values per array)
    rng = np.random.default_rng(0)
    pos = rng.random((n, 3)).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    rho = (1000 + rng.random(n)).astype(np.float32)
    path = str(tmp_path / "PartFluid_0001.vtk")
    pms_lib.write_vtk(path, pos, vel, rho)
    p2, v2, r2 = pms_lib.read_vtk(path)
    np.testing.assert_array_equal(p2, pos)
    np.testing.assert_array_equal(v2, vel)
    np.testing.assert_array_equal(r2, rho)


def test_vtk_ascii_legacy_polydata(pms_lib, tmp_path):
    text = """# vtk DataFile Version 3.0
fluid frame
ASCII
DATASET POLYDATA
POINTS 3 double
0 0 0  1 0.5 0.25
-1 2 3
VERTICES 3 6
1 0
1 1
1 2
POINT_DATA 3
SCALARS Rhop float 1
LOOKUP_TABLE default
1000 1001 1002
VECTORS Vel float
1 2 3 4 5 6 7 8 9
"""
    path = tmp_path / "a.vtk"
    path.write_text(text)
    p, v, r = pms_lib.read_vtk(str(path))
    np.testing.assert_array_equal(p, np.array([[0, 0, 0], [1, 0.5, 0.25], [-1, 2, 3]], np.float32))
    np.testing.assert_array_equal(v.reshape(-1), np.arange(1, 10, dtype=np.float32))
    np.testing.assert_array_equal(r, np.array([1000, 1001, 1002], np.float32))


def test_vtk_missing_file(pms_lib):
    with pytest.raises(pms_lib.PmsError) as ei:
        pms_lib.read_vtk("/nonexistent.vtk")
    assert ei.value.status == 5


def test_ply_ascii_layout(pms_lib, tmp_path):
    verts = np.array([[0.5, 1.25, -2.0], [1e-7, 123456.78, 3.0], [0.1, 0.2, 0.3]], np.float32)
    path = tmp_path / "m.ply"
    pms_lib.write_ply(str(path), verts)
    lines = path.read_text().split("\n")
    assert lines[:10] == ["ply", "format ascii 1.0", "comment generated by tinyply 2.3", "element vertex 3",
                          "property float x", "property float y", "property float z", "element face 1",
                          "property list uchar uint vertex_indices", "end_header"]
    # C++ stream default formatting of float (printf %g), a space after every value
    assert lines[10] == "0.5 1.25 -2 "
    assert lines[11] == "1e-07 123457 3 "
    assert lines[12] == "0.1 0.2 0.3 "
    assert lines[13] == "3 0 1 2 "


def test_mc_tables_in_use_are_the_reference_tables(pms_lib, oracle):
    e, t, nv, ev, from_ref = pms_lib.mc_tables()
    d = load_golden("block10")
    import hashlib
    h = hashlib.sha256()
    for a in (e, t, nv, ev):
        h.update(np.ascontiguousarray(a).tobytes())
    if not from_ref:
        pytest.skip("libpms was built without the reference tree (derived tables)")
    assert h.hexdigest() == str(d["mc_tables_sha256"])


def test_derived_mc_tables_cross_the_same_edges(pms_lib):
    e, t, nv, ev, _ = pms_lib.mc_tables(derived=True)
    # an edge is crossed exactly when its two corners lie on different sides
    for c in range(256):
        want = 0
        for k, (a, b) in enumerate(ev):
            if ((c >> a) & 1) != ((c >> b) & 1):
                want |= 1 << k
        assert e[c] == want
    assert nv[0] == 0 and nv[255] == 0


def test_derived_mc_tables_match_reference_counts_and_close_their_loops(pms_lib):
    """The tables libpms derives when built without the reference tree emit, in
    every one of the 256 cases, the reference's number of mesh vertices (golden
    counts from MarchingCubesHelper.cpp), use only crossed edges, and form closed
    surfaces: inside one case every crossed edge is shared by an even number of
    triangle sides, each side once in each direction."""
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "mc_tables_counts.npz"))
    e, t, nv, ev, _ = pms_lib.mc_tables(derived=True)
    np.testing.assert_array_equal(nv, d["num_vertices"])
    np.testing.assert_array_equal(e, d["edge_flags"])
    for c in range(256):
        tris = t[c][: nv[c]].reshape(-1, 3)
        used = set(tris.reshape(-1).tolist())
        assert all((e[c] >> k) & 1 for k in used), c
        # every directed side (a -> b) of one triangle is matched by (b -> a) of another
        # (or runs along a cube face, where the loop crosses it): count undirected sides
        sides = {}
        for a, b, cc in tris:
            for x, y in ((a, b), (b, cc), (cc, a)):
                key = (min(x, y), max(x, y))
                sides[key] = sides.get(key, 0) + (1 if x < y else -1)
        # interior diagonals cancel in direction; boundary sides (on faces) appear once
        assert all(v in (-1, 0, 1) for v in sides.values()), c


def _read_ply(path):
    """A small PLY reader (ascii / binary_little_endian; float xyz, uchar-uint faces)."""
    raw = open(path, "rb").read()
    end = raw.index(b"end_header\n") + len(b"end_header\n")
    head = raw[:end].decode().splitlines()
    fmt = head[1].split()[1]
    nv = int([h for h in head if h.startswith("element vertex")][0].split()[2])
    nf = int([h for h in head if h.startswith("element face")][0].split()[2])
    body = raw[end:]
    if fmt == "ascii":
        toks = body.decode().split()
        v = np.array(toks[: 3 * nv], np.float32).reshape(-1, 3)
        f = np.array(toks[3 * nv:], np.int64).reshape(-1, 4)
        assert np.all(f[:, 0] == 3)
        return fmt, v, f[:, 1:]
    v = np.frombuffer(body[: 12 * nv], "<f4").reshape(-1, 3)
    rec = np.frombuffer(body[12 * nv: 12 * nv + 13 * nf], np.dtype([("n", "u1"), ("i", "<u4", 3)]))
    assert np.all(rec["n"] == 3) and len(body) == 12 * nv + 13 * nf
    return fmt, v, rec["i"].astype(np.int64)


@pytest.mark.parametrize("binary", [False, True])
def test_ply_indexed_and_binary_layouts(pms_lib, tmp_path, binary):
    rng = np.random.default_rng(4)
    pos = rng.uniform(-1, 1, (10, 3)).astype(np.float32)
    idx = np.array([[0, 1, 2], [2, 3, 4], [9, 8, 7]], np.uint32)
    p = tmp_path / "m.ply"
    pms_lib.write_ply_mesh(str(p), pos, idx, binary=binary)
    fmt, v, f = _read_ply(str(p))
    assert fmt == ("binary_little_endian" if binary else "ascii")
    np.testing.assert_array_equal(v, pos)
    np.testing.assert_array_equal(f, idx)
    # the soup in binary: faces 3k, 3k+1, 3k+2
    q = tmp_path / "s.ply"
    pms_lib.write_ply_mesh(str(q), pos[:9], None, binary=True)
    fmt, v, f = _read_ply(str(q))
    np.testing.assert_array_equal(f, np.arange(9).reshape(-1, 3))
    # an index past the vertices is refused
    with pytest.raises(pms_lib.PmsError):
        pms_lib.write_ply_mesh(str(p), pos, np.array([[0, 1, 10]], np.uint32))


def test_float_form_of_the_double_lerp_threshold():
    """The emission decides getLerpFac's |delta| < 1e-7 (a double literal) on the float
    delta as |delta| < 1e-7f; both give the same answer for every float, checked on the
    floats around the threshold and on a spread of magnitudes."""
    t = np.float32(1e-7)
    near = [t]
    for _ in range(64):
        near.append(np.nextafter(near[-1], np.float32(1)))
    lo = [t]
    for _ in range(64):
        lo.append(np.nextafter(lo[-1], np.float32(0)))
    rng = np.random.default_rng(5)
    d = np.concatenate([np.array(near + lo, np.float32),
                        (10.0 ** rng.uniform(-12, 2, 100000)).astype(np.float32),
                        np.array([0.0, np.float32(1e-45)], np.float32)])
    d = np.concatenate([d, -d])
    ref = (d.astype(np.float64) > -1.0e-7) & (d.astype(np.float64) < 1.0e-7)
    np.testing.assert_array_equal(ref, np.abs(d) < np.float32(1e-7))


def test_float_form_of_the_wendland_tail(pms_lib):
    """The diffuse update evaluates Wwendland's last factor (float)((double)d *
    ((double)(2q) + 1.0)) in float (one fma, an exact residual and a midpoint test
    that falls back to the double form); it returns the double form's bits for every
    input, here over log-uniform and integer-valued d, the whole t = 2q range, tiny t
    and the floats next to 0, 1, 2 and 4."""
    rng = np.random.default_rng(11)
    n = 1 << 20
    d = np.concatenate([(10.0 ** rng.uniform(-30, 6, n)).astype(np.float32),
                        rng.integers(1, 1 << 24, n).astype(np.float32),
                        np.array([0.0, 1e-45, 1e-38, 1.0, 3.0, 16777215.0], np.float32)])
    t = np.concatenate([rng.uniform(0, 4, n).astype(np.float32),
                        (10.0 ** rng.uniform(-14, 0.6, n)).astype(np.float32),
                        np.array([0.0, 1e-45, 2.0 ** -29, 2.0 ** -30, 1.0, 4.0], np.float32)])
    edge = []
    for c in (0.0, 1.0, 2.0, 4.0):
        x = np.float32(c)
        for _ in range(200):
            x = np.nextafter(x, np.float32(-1))
            if x >= 0:
                edge.append(x)
        x = np.float32(c)
        for _ in range(200):
            x = np.nextafter(x, np.float32(5))
            if x <= 4:
                edge.append(x)
    edge = np.array(edge, np.float32)
    d = np.concatenate([d, rng.choice(d, len(edge))]).astype(np.float32)
    t = np.concatenate([t, edge]).astype(np.float32)
    d, t = np.ascontiguousarray(d), np.ascontiguousarray(t)
    out = np.empty_like(d)
    L = pms_lib.lib()
    f = L.pms_debug_wendland_tail
    f.restype = None
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]
    f(d.ctypes.data, t.ctypes.data, out.ctypes.data, len(d))
    want = (d.astype(np.float64) * (t.astype(np.float64) + 1.0)).astype(np.float32)
    bad = np.flatnonzero(out.view(np.uint32) != want.view(np.uint32))
    assert bad.size == 0, (d[bad[:5]], t[bad[:5]], out[bad[:5]], want[bad[:5]])
