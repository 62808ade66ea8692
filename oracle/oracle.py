"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker.  It loads

* ``oracle/_build/liboracle.so`` -- the plain-C restatement of the reference's
  algorithm (``pms_oracle.c``, ``pms_diffuse_oracle.c``), and
* ``oracle/_ref/libref_emu.so`` (optional) -- the reference's own kernels
  compiled for the CPU by ``make -C oracle ref``; present only where the
  reference tree is mounted.

``run_surface`` chains the oracle stages exactly like the reference's host code
(NeighborSearch.cu:37-76, Anisotropic.cu:30-254, MarchingCube.cu:32-151).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field as dc_field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_emu.so")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


class Config(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("particle_spacing", C.c_double), ("smoothing_radius_ratio", C.c_double),
        ("min_num_neighbors", C.c_long), ("isolate_num_neighbors", C.c_long),
        ("lambda_for_smoothed", C.c_double), ("iso_value", C.c_double),
        ("min_wave_crests", C.c_double), ("max_wave_crests", C.c_double),
        ("min_trapped_air", C.c_double), ("max_trapped_air", C.c_double),
        ("min_kinetic_energy", C.c_double), ("max_kinetic_energy", C.c_double),
        ("trapped_air_multiplier", C.c_double), ("wave_crests_multiplier", C.c_double),
        ("time_step", C.c_double), ("life_time", C.c_double),
        ("buoyancy_control", C.c_double), ("drag_control", C.c_double),
        ("sp_scale", C.c_double), ("sc_scale", C.c_double),
    ]


class Params(C.Structure):
    _fields_ = [
        ("mass", C.c_float), ("particle_spacing", C.c_float), ("smoothing_radius_ratio", C.c_int),
        ("h", C.c_float), ("h_inv", C.c_float), ("h_sq", C.c_float), ("aniso_radius", C.c_float),
        ("min_num_neighbors", C.c_int), ("isolate_num_neighbors", C.c_int),
        ("lambda_for_smoothed", C.c_float), ("iso_value", C.c_float),
        ("hd", C.c_float), ("hd_inv", C.c_float), ("hd_sq", C.c_float), ("hd_aniso", C.c_float),
        ("coefficient", C.c_float), ("d_min_num_neighbors", C.c_int),
        ("min_wc", C.c_float), ("max_wc", C.c_float), ("min_ta", C.c_float), ("max_ta", C.c_float),
        ("min_ke", C.c_float), ("max_ke", C.c_float),
        ("ta_mult", C.c_int), ("wc_mult", C.c_int), ("life_time", C.c_int),
        ("time_step", C.c_float), ("buoyancy", C.c_float), ("drag", C.c_float),
        ("sp_scale", C.c_int), ("sc_scale", C.c_int), ("sp_grid_size", C.c_float), ("sc_grid_size", C.c_float),
        ("spexpand", C.c_int), ("scexpand", C.c_int), ("spexpand_diffuse", C.c_int),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("min_pos", C.c_float * 3), ("max_pos", C.c_float * 3),
        ("scmin_pos", C.c_float * 3), ("scmax_pos", C.c_float * 3),
        ("sp_grid_size", C.c_float), ("sc_grid_size", C.c_float),
        ("spres", C.c_uint32 * 3), ("scres", C.c_uint32 * 3),
        ("spexpand", C.c_int32), ("scexpand", C.c_int32), ("spexpand_diffuse", C.c_int32),
        ("sp_size", C.c_uint32), ("sc_size", C.c_uint32),
    ]


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (and libref_emu.so when the reference tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=out)
    ref = os.environ.get("PMS_REFERENCE_DIR")       # the reference checkout, when there is one
    if ref and os.path.isdir(os.path.join(ref, "src", "cuda")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], stdout=out)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_derive_params.argtypes = [C.POINTER(Config), C.POINTER(Params)]
        L.orc_bbox.argtypes = [_f32p, C.c_uint32, _f32p, _f32p]
        L.orc_grid_from_bbox.argtypes = [C.POINTER(Params), _f32p, _f32p, C.POINTER(Grid)]
        L.orc_hash.argtypes = [C.POINTER(Grid), _f32p, C.c_uint32, _u32p]
        L.orc_stable_sort.argtypes = [_u32p, C.c_uint32, C.c_uint32, _u32p]
        L.orc_cell_ranges.argtypes = [_u32p, C.c_uint32, C.c_uint32, _u32p, _u32p]
        L.orc_surface_cells.argtypes = [C.POINTER(Grid), _u32p, _u32p, _u32p]
        L.orc_exclusive_scan_u32.argtypes = [_u32p, C.c_uint64, _u32p]
        L.orc_exclusive_scan_u32.restype = C.c_uint64
        L.orc_surface_list.argtypes = [C.POINTER(Grid), _u32p, _u32p, _u32p, _u32p]
        L.orc_density.argtypes = [C.POINTER(Params), C.POINTER(Grid), _f32p, C.c_uint32, _u32p, _u32p, _f64p]
        L.orc_scalar_values.argtypes = [C.POINTER(Params), C.POINTER(Grid), _f32p, _f32p, _f64p, _u32p, _u32p, _f32p,
                                        C.c_uint64, _f64p]
        L.orc_anisotropy.argtypes = [C.POINTER(Params), C.POINTER(Grid), _f32p, C.c_uint32, _u32p, _u32p,
                                     _u32p, C.c_uint32, _f64p, _f64p, _f64p, _f64p, _u8p, _u32p]
        L.orc_band_bitmap.argtypes = [C.POINTER(Grid), C.c_float, _f32p, _u32p, C.c_uint32, _f32p, _u8p, _u32p]
        L.orc_bitmap_to_list.argtypes = [_u32p, C.c_uint64, C.c_void_p]
        L.orc_bitmap_to_list.restype = C.c_uint64
        L.orc_field.argtypes = [C.POINTER(Params), C.POINTER(Grid), _f32p, C.c_uint32, _f64p, _u32p, _u32p,
                                _u32p, _u32p, _f64p, _f64p, _u32p, C.c_uint32, _f64p]
        L.orc_mc_set_tables.argtypes = [_u32p, _i32p, _u32p, _u32p]
        L.orc_mc_classify.argtypes = [C.POINTER(Grid), C.c_float, _u32p, _u32p, C.c_uint32, _f32p, _u32p, _u32p]
        L.orc_mc_classify.restype = C.c_uint64
        L.orc_mc_emit.argtypes = [C.POINTER(Grid), C.c_float, _u32p, _u32p, C.c_uint32, _f64p, _u32p, _u32p,
                                  _u64p, _f64p, _f64p]
        L.orc_hausdorff_vertices_to_mesh.argtypes = [_f64p, C.c_uint64, _f64p, C.c_uint64, C.c_double]
        L.orc_hausdorff_vertices_to_mesh.restype = C.c_double
        P, G = C.POINTER(Params), C.POINTER(Grid)
        L.orc_spawn_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64]
        L.orc_spawn_uniform.restype = C.c_float
        L.orc_df_normals.argtypes = [P, G, _f32p, C.c_uint32, _u32p, _u32p, C.c_uint32, _f64p]
        L.orc_df_trapped.argtypes = [P, G, _f32p, _f32p, C.c_uint32, _u32p, _u32p, _f64p, _f64p]
        L.orc_df_crests.argtypes = [P, G, _f32p, _f32p, _u32p, _u32p, _u32p, C.c_uint32, _f32p, _f64p]
        L.orc_df_counts.argtypes = [P, _f32p, C.c_uint32, _f32p, _i32p]
        L.orc_df_counts_from_clamped.argtypes = [P, _f32p, C.c_uint32, _i32p]
        L.orc_df_spawn.argtypes = [P, G, _f32p, _f32p, C.c_uint32, _u32p, _u32p, _i32p, C.c_uint64, C.c_uint32, _f32p]
        L.orc_df_spawn.restype = C.c_uint64
        L.orc_df_update.argtypes = [P, G, _f32p, _f32p, _u32p, _u32p, _f32p, C.c_uint32]
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# configuration
# --------------------------------------------------------------------------
def parse_ini(text: str) -> dict:
    """config.txt text -> {"section.key": value} with inih's rules (ini.c:60-181):
    case-insensitive keys, '#'/';' line comments, ';' inline comments after
    whitespace, lines without '='/':' ignored, repeated keys joined by newlines."""
    out: dict[str, str] = {}
    section = ""
    prev = ""
    for raw in text.splitlines():
        line = raw.rstrip()
        stripped = line.lstrip()
        if not stripped or stripped[0] in "#;":
            continue
        if prev and len(stripped) < len(line):
            out[prev] = out[prev] + "\n" + stripped
            continue
        if stripped[0] == "[":
            end = stripped.find("]")
            if end > 0:
                section = stripped[1:end]
                prev = ""
            continue
        eq = stripped.find("=")
        if eq < 0:
            eq = stripped.find(":")
        if eq < 0:
            continue
        name = stripped[:eq].rstrip()
        value = stripped[eq + 1:].lstrip()
        for k in range(1, len(value)):
            if value[k] == ";" and value[k - 1].isspace():
                value = value[:k]
                break
        key = (section + "." + name).lower()
        value = value.rstrip()
        out[key] = (out[key] + "\n" + value) if out.get(key) else value
        prev = key
    return out


def _num(v, default):
    """strtod-like: the longest numeric prefix, else the default."""
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)", str(v))
    return float(m.group(0)) if m else float(default)


def config_from_keys(keys: dict) -> Config:
    """Build an orc_config from a {"section.key": value} mapping, with the
    reference's defaults (Params.cpp:31-106)."""
    def g(name, default):
        return _num(keys.get(name.lower(), default), default)
    c = Config()
    c.mass = g("sim.mass", 0)
    c.particle_spacing = g("sim.particlespacing", 0.01)
    c.smoothing_radius_ratio = g("surface.smoothingradiusratio", 4)
    c.min_num_neighbors = int(g("surface.minnumneighbors", 8))
    c.isolate_num_neighbors = int(g("surface.isolatenumneighbors", 4))
    c.lambda_for_smoothed = g("surface.lambdaforsmoothed", 0.5)
    c.iso_value = g("surface.isovalue", 0.5)
    c.min_wave_crests = g("diffuse.minwavecreststhreshold", 0)
    c.max_wave_crests = g("diffuse.maxwavecreststhreshold", 100)
    c.min_trapped_air = g("diffuse.mintrappedairthreshold", 0)
    c.max_trapped_air = g("diffuse.maxtrappedairthreshold", 100)
    c.min_kinetic_energy = g("diffuse.minkineticenergythreshold", 0)
    c.max_kinetic_energy = g("diffuse.maxkineticenergythreshold", 100)
    c.trapped_air_multiplier = g("diffuse.diffusetrappedairmultiplier", 800)
    c.wave_crests_multiplier = g("diffuse.diffusewavecrestsmultiplier", 4000)
    c.time_step = g("diffuse.timestep", 0.01)
    c.life_time = g("diffuse.lifefimemultiplier", 10)
    c.buoyancy_control = g("diffuse.buoyancycontrol", 0.8)
    c.drag_control = g("diffuse.dragcontrol", 0.5)
    c.sp_scale = g("domain.spatialgridsizescale", 2)
    c.sc_scale = g("domain.sclargridsizescale", 2)
    return c


def derive_params(cfg: Config) -> Params:
    p = Params()
    lib().orc_derive_params(C.byref(cfg), C.byref(p))
    return p


def grid_from_positions(p: Params, pos: np.ndarray) -> Grid:
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    bmin = np.zeros(3, np.float32)
    bmax = np.zeros(3, np.float32)
    lib().orc_bbox(pos, pos.size // 3, bmin, bmax)
    g = Grid()
    lib().orc_grid_from_bbox(C.byref(p), bmin, bmax, C.byref(g))
    return g


# --------------------------------------------------------------------------
# marching-cubes tables
# --------------------------------------------------------------------------
def set_mc_tables(edge_flags, tri, num_vertices, edge_vertices) -> None:
    lib().orc_mc_set_tables(np.ascontiguousarray(edge_flags, np.uint32), np.ascontiguousarray(tri, np.int32).reshape(-1),
                            np.ascontiguousarray(num_vertices, np.uint32),
                            np.ascontiguousarray(edge_vertices, np.uint32).reshape(-1))


# --------------------------------------------------------------------------
# the full plain pipeline
# --------------------------------------------------------------------------
@dataclass
class SurfaceResult:
    grid: Grid
    keys_sorted: np.ndarray
    perm: np.ndarray
    pos_sorted: np.ndarray
    cell_start: np.ndarray
    cell_end: np.ndarray
    surf_count: np.ndarray
    surf_scan: np.ndarray
    surf_list: np.ndarray
    rho: np.ndarray = None
    mean: np.ndarray = None
    G: np.ndarray = None
    maxv: np.ndarray = None
    nrm: np.ndarray = None
    flag: np.ndarray = None
    nnb: np.ndarray = None
    bitmap: np.ndarray = None
    band: np.ndarray = None
    field: np.ndarray = None
    cases: np.ndarray = None
    nvert: np.ndarray = None
    vpos: np.ndarray = None
    vnrm: np.ndarray = None
    extra: dict = dc_field(default_factory=dict)


def hash_sort(p: Params, g: Grid, pos: np.ndarray):
    L = lib()
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    n = pos.size // 3
    keys = np.zeros(n, np.uint32)
    L.orc_hash(C.byref(g), pos, n, keys)
    perm = np.zeros(n, np.uint32)
    L.orc_stable_sort(keys, n, g.sp_size, perm)
    sk = np.ascontiguousarray(keys[perm])
    start = np.zeros(g.sp_size, np.uint32)
    end = np.zeros(g.sp_size, np.uint32)
    L.orc_cell_ranges(sk, n, g.sp_size, start, end)
    return keys, perm, sk, start, end


def surface_particles(g: Grid, start, end):
    L = lib()
    surf = np.zeros(g.sp_size, np.uint32)
    L.orc_surface_cells(C.byref(g), start, end, surf)
    scan = np.zeros(g.sp_size, np.uint32)
    ns = L.orc_exclusive_scan_u32(surf, g.sp_size, scan)
    lst = np.zeros(max(ns, 1), np.uint32)
    L.orc_surface_list(C.byref(g), surf, scan, start, lst)
    return surf, scan, lst[:ns]


def band_bitmap(g: Grid, h: float, spos, surf_list, nrm32, flag8):
    L = lib()
    words = (g.sc_size + 31) // 32
    bm = np.zeros(max(words, 1), np.uint32)
    L.orc_band_bitmap(C.byref(g), h, np.ascontiguousarray(spos, np.float32).reshape(-1),
                      np.ascontiguousarray(surf_list, np.uint32), len(surf_list),
                      np.ascontiguousarray(nrm32, np.float32).reshape(-1), np.ascontiguousarray(flag8, np.uint8), bm)
    nb = L.orc_bitmap_to_list(bm, g.sc_size, None)
    lst = np.zeros(max(nb, 1), np.uint32)
    L.orc_bitmap_to_list(bm, g.sc_size, lst.ctypes.data)
    return bm, lst[:nb]


def mc_classify(g: Grid, iso: float, bm, band, field32):
    cases = np.zeros(len(band), np.uint32)
    nvert = np.zeros(len(band), np.uint32)
    total = lib().orc_mc_classify(C.byref(g), iso, bm, np.ascontiguousarray(band, np.uint32), len(band),
                                  np.ascontiguousarray(field32, np.float32), cases, nvert)
    return cases, nvert, int(total)


def mc_emit(g: Grid, iso: float, bm, band, field64, cases, nvert):
    offs = np.zeros(len(band), np.uint64)
    if len(band):
        offs[1:] = np.cumsum(nvert[:-1].astype(np.uint64))
    m = int(nvert.sum())
    vpos = np.zeros(3 * max(m, 1), np.float64)
    vnrm = np.zeros(3 * max(m, 1), np.float64)
    lib().orc_mc_emit(C.byref(g), iso, bm, np.ascontiguousarray(band, np.uint32), len(band),
                      np.ascontiguousarray(field64, np.float64), cases, nvert, offs, vpos, vnrm)
    return vpos[: 3 * m].reshape(-1, 3), vnrm[: 3 * m].reshape(-1, 3)


def scalar_values(p: Params, g: Grid, spos, svel, rho, start, end, verts) -> np.ndarray:
    """estimationOfScalarValue at mesh vertices, float64: (m, 5) {vel xyz, |vel|, rhop}."""
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1)
    m = verts.size // 3
    out = np.zeros(5 * max(m, 1))
    lib().orc_scalar_values(C.byref(p), C.byref(g), np.ascontiguousarray(spos, np.float32).reshape(-1),
                            np.ascontiguousarray(svel, np.float32).reshape(-1), np.ascontiguousarray(rho, np.float64),
                            np.ascontiguousarray(start, np.uint32), np.ascontiguousarray(end, np.uint32), verts, m, out)
    return out[: 5 * m].reshape(-1, 5)


def run_surface(p: Params, pos: np.ndarray, g: Grid | None = None) -> SurfaceResult:
    """FP64 oracle of the plain surface path on one frame."""
    L = lib()
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    n = len(pos)
    if g is None:
        g = grid_from_positions(p, pos)
    keys, perm, sk, start, end = hash_sort(p, g, pos)
    spos = np.ascontiguousarray(pos[perm]).reshape(-1)
    surf, scan, slist = surface_particles(g, start, end)
    r = SurfaceResult(grid=g, keys_sorted=sk, perm=perm, pos_sorted=spos.reshape(-1, 3), cell_start=start,
                      cell_end=end, surf_count=surf, surf_scan=scan, surf_list=slist)
    rho = np.zeros(n, np.float64)
    L.orc_density(C.byref(p), C.byref(g), spos, n, start, end, rho)
    ns = len(slist)
    mean = np.zeros(3 * max(ns, 1)); G = np.zeros(9 * max(ns, 1)); maxv = np.zeros(max(ns, 1))
    nrm = np.zeros(3 * max(ns, 1)); flag = np.zeros(max(ns, 1), np.uint8); nnb = np.zeros(max(ns, 1), np.uint32)
    if ns:
        L.orc_anisotropy(C.byref(p), C.byref(g), spos, n, start, end, slist, ns, mean, G, maxv, nrm, flag, nnb)
    r.rho, r.mean, r.G, r.maxv = rho, mean[: 3 * ns].reshape(-1, 3), G[: 9 * ns].reshape(-1, 9), maxv[:ns]
    r.nrm, r.flag, r.nnb = nrm[: 3 * ns].reshape(-1, 3), flag[:ns], nnb[:ns]
    bm, band = band_bitmap(g, p.h, spos, slist, r.nrm.astype(np.float32), r.flag)
    r.bitmap, r.band = bm, band
    field = np.zeros(max(len(band), 1))
    if len(band):
        L.orc_field(C.byref(p), C.byref(g), spos, n, rho, start, end, surf, scan,
                    np.ascontiguousarray(r.G.reshape(-1)), np.ascontiguousarray(r.maxv), band, len(band), field)
    r.field = field[: len(band)]
    return r


# --------------------------------------------------------------------------
# the reference's own kernels, compiled for the CPU (pinning only)
# --------------------------------------------------------------------------
class RefResult(C.Structure):
    _fields_ = [
        ("min_pos", C.c_float * 3), ("max_pos", C.c_float * 3), ("scmin_pos", C.c_float * 3), ("scmax_pos", C.c_float * 3),
        ("sp_grid_size", C.c_float), ("sc_grid_size", C.c_float),
        ("spres", C.c_uint32 * 3), ("scres", C.c_uint32 * 3), ("spexpand", C.c_int32), ("scexpand", C.c_int32),
        ("sp_size", C.c_uint32), ("sc_size", C.c_uint32),
        ("h", C.c_float), ("h_inv", C.c_float), ("h_sq", C.c_float), ("aniso_radius", C.c_float),
        ("iso", C.c_float), ("mass", C.c_float), ("min_nn", C.c_int32),
        ("n", C.c_uint32), ("n_surface", C.c_uint32), ("n_band", C.c_uint32), ("n_valid", C.c_uint32),
        ("n_mesh", C.c_uint32),
        ("keys_sorted", C.POINTER(C.c_uint32)), ("perm", C.POINTER(C.c_uint32)), ("pos_sorted", C.POINTER(C.c_float)),
        ("rho", C.POINTER(C.c_float)), ("nrm", C.POINTER(C.c_float)), ("flag", C.POINTER(C.c_float)),
        ("cell_start", C.POINTER(C.c_uint32)), ("cell_end", C.POINTER(C.c_uint32)), ("surf_count", C.POINTER(C.c_uint32)),
        ("surf_list", C.POINTER(C.c_uint32)), ("mean", C.POINTER(C.c_float)), ("G", C.POINTER(C.c_float)),
        ("band_flags", C.POINTER(C.c_uint32)), ("band_list", C.POINTER(C.c_uint32)), ("field", C.POINTER(C.c_float)),
        ("cube_flag", C.POINTER(C.c_uint32)), ("nvert", C.POINTER(C.c_uint32)),
        ("vpos", C.POINTER(C.c_float)), ("vnrm", C.POINTER(C.c_float)), ("sval", C.POINTER(C.c_float)),
    ]


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def _arr(ptr, count, dtype):
    if not ptr or count == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True)


def ref_surface_run(config_path: str, pos, vel=None, rhop=None) -> dict:
    """Runs the reference kernels (CPU emulation) on one frame; returns numpy arrays."""
    R = C.CDLL(REF_PATH)
    R.ref_surface_run.argtypes = [C.c_char_p, _f32p, _f32p, _f32p, C.c_uint32, C.POINTER(RefResult)]
    R.ref_surface_run.restype = C.c_int
    R.ref_free.argtypes = [C.POINTER(RefResult)]
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    n = pos.size // 3
    vel = np.zeros(3 * n, np.float32) if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1)
    rhop = np.full(n, 1000.0, np.float32) if rhop is None else np.ascontiguousarray(rhop, np.float32)
    res = RefResult()
    rc = R.ref_surface_run(config_path.encode(), pos, vel, rhop, n, C.byref(res))
    out = {"rc": rc}
    for k in ("min_pos", "max_pos", "scmin_pos", "scmax_pos", "spres", "scres"):
        out[k] = np.array(getattr(res, k)[:])
    for k in ("sp_grid_size", "sc_grid_size", "spexpand", "scexpand", "sp_size", "sc_size", "h", "h_inv", "h_sq",
              "aniso_radius", "iso", "mass", "min_nn", "n", "n_surface", "n_band", "n_valid", "n_mesh"):
        out[k] = getattr(res, k)
    n, ns, nb, nm, S, Sc = res.n, res.n_surface, res.n_band, res.n_mesh, res.sp_size, res.sc_size
    out["keys_sorted"] = _arr(res.keys_sorted, n, np.uint32)
    out["perm"] = _arr(res.perm, n, np.uint32)
    out["pos_sorted"] = _arr(res.pos_sorted, 3 * n, np.float32).reshape(-1, 3)
    out["rho"] = _arr(res.rho, n, np.float32)
    out["nrm"] = _arr(res.nrm, 3 * n, np.float32).reshape(-1, 3)
    out["flag"] = _arr(res.flag, n, np.float32)
    out["cell_start"] = _arr(res.cell_start, S, np.uint32)
    out["cell_end"] = _arr(res.cell_end, S, np.uint32)
    out["surf_count"] = _arr(res.surf_count, S, np.uint32)
    out["surf_list"] = _arr(res.surf_list, ns, np.uint32)
    out["mean"] = _arr(res.mean, 3 * ns, np.float32).reshape(-1, 3)
    out["G"] = _arr(res.G, 10 * ns, np.float32).reshape(-1, 10)
    out["band_flags"] = _arr(res.band_flags, Sc, np.uint32)
    out["band_list"] = _arr(res.band_list, nb, np.uint32)
    out["field"] = _arr(res.field, nb, np.float32)
    out["cube_flag"] = _arr(res.cube_flag, nb, np.uint32)
    out["nvert"] = _arr(res.nvert, nb, np.uint32)
    out["vpos"] = _arr(res.vpos, 3 * nm, np.float32).reshape(-1, 3)
    out["vnrm"] = _arr(res.vnrm, 3 * nm, np.float32).reshape(-1, 3)
    out["sval"] = _arr(res.sval, 5 * nm, np.float32).reshape(-1, 5) if res.sval else np.zeros((0, 5), np.float32)
    R.ref_free(C.byref(res))
    return out


def ref_mc_tables():
    R = C.CDLL(REF_PATH)
    e = np.zeros(256, np.uint32); t = np.zeros(256 * 16, np.int32); nv = np.zeros(256, np.uint32); ev = np.zeros(24, np.uint32)
    R.ref_mc_tables.argtypes = [_u32p, _i32p, _u32p, _u32p]
    R.ref_mc_tables(e, t, nv, ev)
    return e, t.reshape(256, 16), nv, ev.reshape(12, 2)


# --------------------------------------------------------------------------
# diffuse particles
# --------------------------------------------------------------------------
def spawn_uniforms(seed: int, frame: int, count: int) -> np.ndarray:
    L = lib()
    return np.array([L.orc_spawn_uniform(seed, frame, k) for k in range(count)], np.float32)


def diffuse_frame(p: Params, g: Grid, spos, svel, start, end, free_list, nrm_init, seed: int, frame: int,
                  old=None, nrm_for_crests=None, pot_clamped=None):
    """Float64 oracle of one diffuse frame on sorted particles.  Returns a dict
    with normals, raw and clamped potentials, counts, generated particles (8
    floats each: pos, vel, ttl, type), the advected old particles and the live
    list (generated then old, type 3 dropped).  `nrm_for_crests` (float32)
    replaces the oracle's own normals in the wave-crest sum; `pot_clamped`
    replaces its clamped potentials when deriving the counts."""
    L = lib()
    spos = np.ascontiguousarray(spos, np.float32).reshape(-1)
    svel = np.ascontiguousarray(svel, np.float32).reshape(-1)
    n = spos.size // 3
    nrm = np.ascontiguousarray(nrm_init, np.float64).reshape(-1).copy()
    L.orc_df_normals(C.byref(p), C.byref(g), spos, n, start, end, len(free_list), nrm)
    ita = np.zeros(n); en = np.zeros(n); wc = np.zeros(n)
    L.orc_df_trapped(C.byref(p), C.byref(g), spos, svel, n, start, end, ita, en)
    nc = np.ascontiguousarray(nrm.astype(np.float32) if nrm_for_crests is None else nrm_for_crests, np.float32).reshape(-1)
    L.orc_df_crests(C.byref(p), C.byref(g), spos, svel, start, end, np.ascontiguousarray(free_list, np.uint32),
                    len(free_list), nc, wc)
    raw = np.ascontiguousarray(np.stack([wc, ita, en], 1).astype(np.float32).reshape(-1))
    clamped = np.zeros_like(raw)
    num = np.zeros(n, np.int32)
    L.orc_df_counts(C.byref(p), raw, n, clamped, num)
    if pot_clamped is not None:
        num = np.zeros(n, np.int32)
        L.orc_df_counts_from_clamped(C.byref(p), np.ascontiguousarray(pot_clamped, np.float32).reshape(-1), n, num)
    total = int(np.clip(num, 0, None).sum())
    gen = np.zeros(8 * max(total, 1), np.float32)
    k = L.orc_df_spawn(C.byref(p), C.byref(g), spos, svel, n, start, end, num, seed, frame, gen)
    gen = gen[: 8 * k].reshape(-1, 8)
    old_after = np.zeros((0, 8), np.float32)
    if old is not None and len(old):
        rec = np.ascontiguousarray(old, np.float32).reshape(-1).copy()
        L.orc_df_update(C.byref(p), C.byref(g), spos, svel, start, end, rec, len(old))
        old_after = rec.reshape(-1, 8)
    live = np.concatenate([gen[gen[:, 7] != 3], old_after[old_after[:, 7] != 3]]) if (len(gen) or len(old_after)) \
        else np.zeros((0, 8), np.float32)
    return {"nrm": nrm.reshape(-1, 3), "pot_raw": raw.reshape(-1, 3), "pot": clamped.reshape(-1, 3), "num": num,
            "gen": gen, "old_after": old_after, "live": live}


class RefDiffuse(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_free", C.c_uint32), ("n_spawning", C.c_uint32), ("n_generated", C.c_uint32),
                ("n_old", C.c_uint32), ("n_live", C.c_uint32),
                ("perm", C.POINTER(C.c_uint32)), ("free_list", C.POINTER(C.c_uint32)), ("nrm", C.POINTER(C.c_float)),
                ("pot", C.POINTER(C.c_float)), ("num", C.POINTER(C.c_int32)), ("gen", C.POINTER(C.c_float)),
                ("old_after", C.POINTER(C.c_float)), ("live", C.POINTER(C.c_float))]


def ref_diffuse_frame(config_path: str, pos, vel, rho, run_surface: bool, old, seed: int, frame: int) -> dict:
    """The reference's diffuse kernels (CPU emulation) on one frame, with the
    spawn uniforms of the counter-based generator injected."""
    R = C.CDLL(REF_PATH)
    R.ref_diffuse_frame.argtypes = [C.c_char_p, _f32p, _f32p, _f32p, C.c_uint32, C.c_int, _f32p, C.c_uint32, _f32p,
                                    C.c_uint64, C.POINTER(RefDiffuse)]
    R.ref_diffuse_frame.restype = C.c_int
    R.ref_diffuse_free.argtypes = [C.POINTER(RefDiffuse)]
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1)
    rho = np.ascontiguousarray(rho, np.float32)
    n = pos.size // 3
    old = np.zeros((0, 8), np.float32) if old is None else np.ascontiguousarray(old, np.float32)
    old_flat = np.ascontiguousarray(old.reshape(-1) if len(old) else np.zeros(8, np.float32))
    # enough uniforms for any plausible spawn count: grow until the frame fits
    count = 3 * max(1024, 64 * n)
    uni = np.array([lib().orc_spawn_uniform(seed, frame, k) for k in range(count)], np.float32)
    res = RefDiffuse()
    rc = R.ref_diffuse_frame(config_path.encode(), pos, vel, rho, n, 1 if run_surface else 0, old_flat, len(old), uni,
                             len(uni), C.byref(res))
    out = {"rc": rc}
    out["perm"] = _arr(res.perm, res.n, np.uint32)
    out["free_list"] = _arr(res.free_list, res.n_free, np.uint32)
    out["nrm"] = _arr(res.nrm, 3 * res.n, np.float32).reshape(-1, 3)
    out["pot"] = _arr(res.pot, 3 * res.n, np.float32).reshape(-1, 3)
    out["num"] = _arr(res.num, res.n, np.int32)
    out["gen"] = _arr(res.gen, 8 * res.n_generated, np.float32).reshape(-1, 8)
    out["old_after"] = _arr(res.old_after, 8 * res.n_old, np.float32).reshape(-1, 8)
    out["live"] = _arr(res.live, 8 * res.n_live, np.float32).reshape(-1, 8)
    for k in ("n_free", "n_spawning", "n_generated", "n_old", "n_live"):
        out[k] = getattr(res, k)
    R.ref_diffuse_free(C.byref(res))
    return out
