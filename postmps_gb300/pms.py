"""ctypes binding of libpms (include/pms.h) -- the Python face of the C ABI.

The classes mirror the reference's host objects: ``load_config`` is
Params::setParams (Params.cpp:24-152), ``Context`` is one GPUPOST with its
GPUmemory, and its stage methods are NeighborSearch::SpatialGridBuilding,
Anisotropic::processingOfParticles / processingOfVertices /
estimationOfscalarField, MarchingCube::triangulation and
DiffuseGeneration::runsimulation.  Errors raise ``PmsError`` carrying the
library's status and message.  There is no fallback: if libpms.so is missing
the import of a Context fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpms.so")

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "capacity exceeded", 5: "I/O error",
    6: "configuration error", 7: "stage called out of order", 8: "device wait timed out", 9: "unsupported input",
}

ARRAY = {
    "keys_sorted": (1, np.uint32), "perm": (2, np.uint32), "cell_start": (3, np.uint32), "cell_end": (4, np.uint32),
    "surf_count": (5, np.uint32), "surf_list": (6, np.uint32), "density": (7, np.float32), "mean": (8, np.float32),
    "G": (9, np.float32), "normal": (10, np.float32), "flag": (11, np.uint8), "band_bitmap": (12, np.uint32),
    "band_list": (13, np.uint32), "field": (14, np.float32), "cube_case": (15, np.uint32),
    "cube_nvert": (16, np.uint32), "pos_sorted": (17, np.float32), "neighbors": (18, np.uint32),
    "diffuse_potential": (19, np.float32), "diffuse_count": (20, np.int32), "free_normal": (21, np.float32),
    "band_certified": (22, np.uint32),
}


class PmsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Config(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("particle_spacing", C.c_double), ("smoothing_radius_ratio", C.c_double),
        ("min_num_neighbors", C.c_long), ("isolate_num_neighbors", C.c_long),
        ("lambda_for_smoothed", C.c_double), ("iso_value", C.c_double),
        ("min_wave_crests", C.c_double), ("max_wave_crests", C.c_double),
        ("min_trapped_air", C.c_double), ("max_trapped_air", C.c_double),
        ("min_kinetic_energy", C.c_double), ("max_kinetic_energy", C.c_double),
        ("trapped_air_multiplier", C.c_double), ("wave_crests_multiplier", C.c_double),
        ("time_step", C.c_double), ("life_time", C.c_double), ("buoyancy_control", C.c_double),
        ("drag_control", C.c_double), ("sp_scale", C.c_double), ("sc_scale", C.c_double),
        ("domain_min", C.c_double * 3), ("domain_max", C.c_double * 3),
        ("gpu_id", C.c_int), ("frame_start", C.c_int), ("frame_end", C.c_int), ("frame_step", C.c_int),
        ("num_zeros", C.c_int), ("is_surface", C.c_int), ("is_diffuse", C.c_int),
        ("fluid_path", C.c_char * 512), ("fluid_prefix", C.c_char * 128),
        ("surface_path", C.c_char * 512), ("surface_prefix", C.c_char * 128),
        ("diffuse_path", C.c_char * 512), ("diffuse_prefix", C.c_char * 128),
        ("fp64_svd_cond", C.c_double), ("rng_seed", C.c_uint64), ("band_model", C.c_char * 512),
        ("ply_binary", C.c_int), ("weld_mesh", C.c_int),
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
        ("min_ke", C.c_float), ("max_ke", C.c_float), ("ta_mult", C.c_int), ("wc_mult", C.c_int),
        ("life_time", C.c_int), ("time_step", C.c_float), ("buoyancy", C.c_float), ("drag", C.c_float),
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


class Counts(C.Structure):
    _fields_ = [
        ("n_particles", C.c_uint32), ("n_surface_particles", C.c_uint32), ("n_band_vertices", C.c_uint32),
        ("n_valid_cubes", C.c_uint32), ("n_mesh_vertices", C.c_uint64), ("n_free_surface", C.c_uint32),
        ("n_generated_diffuse", C.c_uint32), ("n_spawning", C.c_uint32), ("n_diffuse", C.c_uint32),
        ("n_spray", C.c_uint32), ("n_foam", C.c_uint32), ("n_bubble", C.c_uint32), ("n_fp64_svd", C.c_uint32),
        ("n_band_candidates", C.c_uint32), ("n_band_predicted", C.c_uint32), ("n_band_exact", C.c_uint32),
        ("n_band_certified", C.c_uint32), ("n_band_rechecked", C.c_uint32), ("n_field_pairs", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# pms_diffuse_particle, the streamed and batched diffuse records
DIFFUSE_RECORD = np.dtype([("pos", np.float32, 3), ("ttl", np.int32), ("vel", np.float32, 3), ("type", np.int32)])


class Tune(C.Structure):
    """pms_tune: launch shapes of the neighbour walks."""
    _fields_ = [("field_threads", C.c_int), ("field_waves", C.c_int), ("density_threads", C.c_int),
                ("moments_threads", C.c_int), ("field_vpt", C.c_int), ("anisotropy_ms", C.c_float),
                ("field_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Frame(C.Structure):
    """pms_frame: one frame of a batch (host or device pointers)."""
    _fields_ = [("pos_xyz", C.c_void_p), ("vel_xyz", C.c_void_p), ("rhop", C.c_void_p), ("n", C.c_uint32)]


BATCH_LEARNED, BATCH_CERTIFIED = 1, 2
BAND_PLAIN, BAND_LEARNED, BAND_CERTIFIED = 0, 1, 2
MLP_INPUTS, MLP_HIDDEN, MLP_PARAMS = 64, 64, 4225


class BandModel(C.Structure):
    """pms_band_model: bf16 weights (as uint16 bits), fp32 biases, logit threshold."""
    _fields_ = [
        ("w1", C.c_uint16 * (MLP_INPUTS * MLP_HIDDEN)), ("b1", C.c_float * MLP_HIDDEN),
        ("w2", C.c_uint16 * MLP_HIDDEN), ("b2", C.c_float), ("threshold", C.c_float),
    ]

    def arrays(self) -> dict:
        return {"w1": np.ctypeslib.as_array(self.w1).copy(), "b1": np.ctypeslib.as_array(self.b1).copy(),
                "w2": np.ctypeslib.as_array(self.w2).copy(), "b2": float(self.b2), "threshold": float(self.threshold)}

    @classmethod
    def from_arrays(cls, d: dict) -> "BandModel":
        m = cls()
        np.ctypeslib.as_array(m.w1)[:] = np.asarray(d["w1"], np.uint16).reshape(-1)
        np.ctypeslib.as_array(m.b1)[:] = np.asarray(d["b1"], np.float32).reshape(-1)
        np.ctypeslib.as_array(m.w2)[:] = np.asarray(d["w2"], np.uint16).reshape(-1)
        m.b2 = float(d["b2"])
        m.threshold = float(d["threshold"])
        return m


_lib = None
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def lib() -> C.CDLL:
    """Loads libpms.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libpms.so is not built ({LIB_PATH}); run postmps_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        S = C.c_int
        vp = C.c_void_p
        L.pms_config_default.argtypes = [C.POINTER(Config)]
        L.pms_config_load.argtypes = [C.c_char_p, C.POINTER(Config)]
        L.pms_params_derive.argtypes = [C.POINTER(Config), C.POINTER(Params)]
        L.pms_grid_from_bbox.argtypes = [C.POINTER(Params), _f32p, _f32p, C.POINTER(Grid)]
        L.pms_create.argtypes = [C.POINTER(Config), C.c_int, C.POINTER(vp)]
        L.pms_destroy.argtypes = [vp]
        L.pms_destroy.restype = None
        L.pms_last_error.argtypes = [vp]
        L.pms_last_error.restype = C.c_char_p
        L.pms_status_string.argtypes = [S]
        L.pms_status_string.restype = C.c_char_p
        L.pms_set_stream.argtypes = [vp, vp]
        L.pms_reserve.argtypes = [vp, C.c_uint32, C.c_uint64]
        L.pms_upload_particles.argtypes = [vp, vp, vp, vp, C.c_uint32]
        L.pms_upload_particles_device.argtypes = [vp, vp, vp, vp, C.c_uint32]
        L.pms_stage_particles.argtypes = [vp, vp, vp, vp, C.c_uint32]
        L.pms_upload_staged.argtypes = [vp]
        for name in ("pms_build_grid", "pms_anisotropy", "pms_band", "pms_field", "pms_marching_cubes", "pms_surface",
                     "pms_diffuse", "pms_run_frame"):
            getattr(L, name).argtypes = [vp]
        L.pms_get_counts.argtypes = [vp, C.POINTER(Counts)]
        L.pms_get_grid.argtypes = [vp, C.POINTER(Grid)]
        L.pms_download_mesh.argtypes = [vp, vp, vp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.pms_download_diffuse.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_uint32, C.POINTER(C.c_uint32)]
        L.pms_debug_download.argtypes = [vp, C.c_int, vp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.pms_debug_set_wait_limit.argtypes = [vp, C.c_int64]
        L.pms_stage_times.argtypes = [vp, _f32p, C.c_int]
        L.pms_kernel_launches.argtypes = [vp]
        L.pms_kernel_launches.restype = C.c_uint64
        L.pms_read_vtk_particles.argtypes = [C.c_char_p, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(C.c_uint32)]
        L.pms_write_vtk_particles.argtypes = [C.c_char_p, vp, vp, vp, C.c_uint32]
        L.pms_write_ply.argtypes = [C.c_char_p, vp, C.c_uint64]
        L.pms_write_diffuse_vtk.argtypes = [C.c_char_p, vp, vp, vp, vp, vp, C.c_uint32, C.c_float]
        L.pms_free_host.argtypes = [vp]
        L.pms_free_host.restype = None
        L.pms_run_config.argtypes = [C.c_char_p, C.c_int]
        L.pms_mc_tables.argtypes = [_u32p, _i32p, _u32p, _u32p, C.c_int]
        L.pms_scalar_values.argtypes = [vp]
        L.pms_download_scalar_values.argtypes = [vp, vp, vp, vp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.pms_write_surface_vtk.argtypes = [C.c_char_p, vp, vp, vp, vp, vp, C.c_uint64]
        L.pms_set_band_model.argtypes = [vp, C.POINTER(BandModel)]
        L.pms_set_band_mode.argtypes = [vp, C.c_int]
        L.pms_weld_mesh.argtypes = [vp, C.c_int]
        L.pms_download_welded_mesh.argtypes = [vp, vp, vp, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64),
                                               C.POINTER(C.c_uint64)]
        L.pms_write_ply_mesh.argtypes = [C.c_char_p, vp, C.c_uint64, vp, C.c_uint64, C.c_int]
        L.pms_run_batch.argtypes = [vp, C.POINTER(Frame), C.c_uint32, C.c_int]
        L.pms_autotune.argtypes = [vp, C.POINTER(Tune)]
        L.pms_set_tune.argtypes = [vp, C.POINTER(Tune)]
        L.pms_get_tune.argtypes = [vp, C.POINTER(Tune)]
        L.pms_batch_frame.argtypes = [vp, C.c_uint32, C.POINTER(Counts), C.POINTER(C.c_float)]
        L.pms_batch_mesh.argtypes = [vp, C.c_uint32, vp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.pms_batch_diffuse.argtypes = [vp, C.c_uint32, vp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.pms_batch_stream_meshes.argtypes = [vp, vp, C.c_uint64]
        L.pms_batch_mesh_range.argtypes = [vp, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.pms_batch_info.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.pms_save_band_model.argtypes = [C.c_char_p, C.POINTER(BandModel), C.c_char_p]
        L.pms_load_band_model.argtypes = [C.c_char_p, C.POINTER(BandModel)]
        L.pms_band_learned.argtypes = [vp]
        L.pms_surface_learned.argtypes = [vp]
        L.pms_learn_prepare.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.pms_learn_candidates.argtypes = [vp, vp, vp, vp, C.c_uint32, C.POINTER(C.c_uint32)]
        L.pms_learn_features.argtypes = [vp, vp, C.c_uint32, vp]
        L.pms_trainer_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(vp)]
        L.pms_trainer_destroy.argtypes = [vp]
        L.pms_trainer_destroy.restype = None
        L.pms_trainer_step.argtypes = [vp, vp, C.c_uint32, C.c_uint64, C.c_float, C.c_float, C.POINTER(C.c_float)]
        L.pms_trainer_grad.argtypes = [vp, vp, vp, C.c_uint32, C.c_float, vp, C.POINTER(C.c_float)]
        L.pms_trainer_get_params.argtypes = [vp, vp]
        L.pms_trainer_set_params.argtypes = [vp, vp]
        L.pms_trainer_get_model.argtypes = [vp, C.POINTER(BandModel)]
        _lib = L
    return _lib


def _check(st: int, ctx=None) -> None:
    if st != 0:
        msg = lib().pms_last_error(ctx).decode() if ctx else ""
        raise PmsError(st, msg or lib().pms_status_string(st).decode())


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------------------
# configuration
# ---------------------------------------------------------------------------
def default_config() -> Config:
    c = Config()
    _check(lib().pms_config_default(C.byref(c)))
    return c


def load_config(path: str) -> Config:
    c = Config()
    _check(lib().pms_config_load(str(path).encode(), C.byref(c)))
    return c


def derive_params(cfg: Config) -> Params:
    p = Params()
    _check(lib().pms_params_derive(C.byref(cfg), C.byref(p)))
    return p


def grid_from_bbox(p: Params, bmin, bmax) -> Grid:
    g = Grid()
    _check(lib().pms_grid_from_bbox(C.byref(p), np.asarray(bmin, np.float32), np.asarray(bmax, np.float32), C.byref(g)))
    return g


def mc_tables(derived: bool = False):
    e = np.zeros(256, np.uint32); t = np.zeros(256 * 16, np.int32); nv = np.zeros(256, np.uint32); ev = np.zeros(24, np.uint32)
    from_ref = lib().pms_mc_tables(e, t, nv, ev, 1 if derived else 0)
    return e, t.reshape(256, 16), nv, ev.reshape(12, 2), bool(from_ref)


# ---------------------------------------------------------------------------
# files
# ---------------------------------------------------------------------------
def write_ply_mesh(path: str, pos, indices=None, binary: bool = False) -> None:
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    idx = None if indices is None else np.ascontiguousarray(indices, np.uint32).reshape(-1)
    _check(lib().pms_write_ply_mesh(str(path).encode(), _ptr(pos), C.c_uint64(len(pos)), _ptr(idx),
                                    C.c_uint64(0 if idx is None else len(idx)), 1 if binary else 0))


def read_vtk(path: str):
    p, v, r = C.c_void_p(), C.c_void_p(), C.c_void_p()
    n = C.c_uint32()
    _check(lib().pms_read_vtk_particles(str(path).encode(), C.byref(p), C.byref(v), C.byref(r), C.byref(n)))
    N = n.value
    def take(ptr, count):
        if not ptr.value:
            return np.zeros(count, np.float32)
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), shape=(count,)).copy()
        lib().pms_free_host(ptr)
        return a
    return take(p, 3 * N).reshape(-1, 3), take(v, 3 * N).reshape(-1, 3), take(r, N)


def write_vtk(path: str, pos, vel=None, rho=None) -> None:
    pos = np.ascontiguousarray(pos, np.float32)
    vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
    rho = None if rho is None else np.ascontiguousarray(rho, np.float32)
    _check(lib().pms_write_vtk_particles(str(path).encode(), _ptr(pos), _ptr(vel), _ptr(rho), len(pos)))


def write_surface_vtk(path: str, verts, normals=None, vel=None, vel_len=None, rhop=None) -> None:
    arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (verts, normals, vel, vel_len, rhop)]
    _check(lib().pms_write_surface_vtk(path.encode(), *[_ptr(a) for a in arrs], len(arrs[0])))


def write_ply(path: str, verts) -> None:
    v = np.ascontiguousarray(verts, np.float32)
    _check(lib().pms_write_ply(str(path).encode(), _ptr(v), len(v)))


def run_config(path: str, verbose: bool = False) -> None:
    _check(lib().pms_run_config(str(path).encode(), 1 if verbose else 0))


# ---------------------------------------------------------------------------
# the GPU context
# ---------------------------------------------------------------------------
class Context:
    """One GPU pipeline (GPUPOST + GPUmemory).  Not thread-safe."""

    def __init__(self, cfg: Config, device: int = 0):
        self._h = C.c_void_p()
        _check(lib().pms_create(C.byref(cfg), device, C.byref(self._h)))
        self.cfg = cfg

    def close(self) -> None:
        if self._h:
            lib().pms_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _call(self, name: str, *args) -> None:
        _check(getattr(lib(), name)(self._h, *args), self._h)

    # stages
    def upload(self, pos, vel=None, rho=None) -> None:
        pos = np.ascontiguousarray(pos, np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        rho = None if rho is None else np.ascontiguousarray(rho, np.float32)
        self._keep = (pos, vel, rho)
        self._call("pms_upload_particles", _ptr(pos), _ptr(vel), _ptr(rho), len(pos))

    def stage(self, pos, vel=None, rho=None) -> None:
        """pms_stage_particles: the next frame's inputs, staged while a frame may run on
        another thread (the arrays are copied before the call returns)."""
        pos = np.ascontiguousarray(pos, np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        rho = None if rho is None else np.ascontiguousarray(rho, np.float32)
        _check(lib().pms_stage_particles(self._h, _ptr(pos), _ptr(vel), _ptr(rho), len(pos)))

    def upload_staged(self) -> None:
        self._call("pms_upload_staged")

    def upload_device(self, d_pos: int, d_vel: int | None, d_rho: int | None, n: int) -> None:
        self._call("pms_upload_particles_device", d_pos, d_vel, d_rho, n)

    def set_stream(self, stream_handle: int | None) -> None:
        self._call("pms_set_stream", stream_handle)

    def reserve(self, max_particles: int, max_scalar_vertices: int = 0) -> None:
        self._call("pms_reserve", max_particles, max_scalar_vertices)

    def build_grid(self): self._call("pms_build_grid")
    def anisotropy(self): self._call("pms_anisotropy")
    def band(self): self._call("pms_band")
    def field(self): self._call("pms_field")
    def marching_cubes(self): self._call("pms_marching_cubes")
    def surface(self): self._call("pms_surface")
    def diffuse(self): self._call("pms_diffuse")
    def run_frame(self): self._call("pms_run_frame")

    # density and velocity at the mesh vertices
    def scalar_values(self) -> dict:
        self._call("pms_scalar_values")
        n = C.c_uint64()
        self._call("pms_download_scalar_values", None, None, None, 0, C.byref(n))
        m = n.value
        out = {"vel": np.zeros((m, 3), np.float32), "vel_len": np.zeros(m, np.float32), "rhop": np.zeros(m, np.float32)}
        if m:
            self._call("pms_download_scalar_values", _ptr(out["vel"]), _ptr(out["vel_len"]), _ptr(out["rhop"]), m,
                       C.byref(n))
        return out

    # learned band
    def set_band_model(self, model: BandModel) -> None:
        self._call("pms_set_band_model", C.byref(model))

    def set_band_mode(self, mode) -> None:
        """False / "plain": the reference's band; True / "learned": the network plus
        the exact sign certification; "certified": the certification alone."""
        m = {False: BAND_PLAIN, True: BAND_LEARNED, "plain": BAND_PLAIN, "learned": BAND_LEARNED,
             "certified": BAND_CERTIFIED}[mode]
        self._call("pms_set_band_mode", m)

    def band_learned(self): self._call("pms_band_learned")
    def surface_learned(self): self._call("pms_surface_learned")

    def learn_prepare(self) -> tuple[int, int]:
        nc, nv = C.c_uint32(), C.c_uint32()
        self._call("pms_learn_prepare", C.byref(nc), C.byref(nv))
        return nc.value, nv.value

    def learn_candidates(self, logits: bool = True) -> dict:
        n = C.c_uint32()
        st = lib().pms_learn_candidates(self._h, None, None, None, 0, C.byref(n))
        if st not in (0, 4):
            _check(st, self._h)
        m = n.value
        ids = np.zeros(m, np.uint32)
        lg = np.zeros(m, np.float32) if logits else None
        lab = np.zeros(m, np.uint8)
        self._call("pms_learn_candidates", _ptr(ids), _ptr(lg), _ptr(lab), m, C.byref(n))
        return {"cube": ids, "logit": lg, "label": lab}

    # autotuner
    def autotune(self) -> dict:
        t = Tune()
        self._call("pms_autotune", C.byref(t))
        return t.as_dict()

    def set_tune(self, d: dict) -> None:
        t = Tune(**{k: d[k] for k in ("field_threads", "field_waves", "density_threads", "moments_threads")},
                 field_vpt=d.get("field_vpt", 2))
        self._call("pms_set_tune", C.byref(t))

    def get_tune(self) -> dict:
        t = Tune()
        self._call("pms_get_tune", C.byref(t))
        return t.as_dict()

    # batched frames
    def run_batch(self, frames, learned=False) -> None:
        """frames: sequence of (pos, vel, rho) numpy arrays (vel / rho may be None),
        or of pms_frame-like (pos_ptr, vel_ptr, rho_ptr, n) tuples of raw pointers."""
        arr = (Frame * max(1, len(frames)))()
        self._keep = []
        for i, fr in enumerate(frames):
            if len(fr) == 4:
                arr[i] = Frame(fr[0], fr[1], fr[2], fr[3])
                continue
            pos, vel, rho = fr
            pos = np.ascontiguousarray(pos, np.float32)
            vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
            rho = None if rho is None else np.ascontiguousarray(rho, np.float32)
            self._keep += [pos, vel, rho]
            arr[i] = Frame(_ptr(pos), _ptr(vel), _ptr(rho), len(pos))
        flag = {False: 0, True: BATCH_LEARNED, "plain": 0, "learned": BATCH_LEARNED, "certified": BATCH_CERTIFIED}[learned]
        self._call("pms_run_batch", arr, len(frames), flag)

    def batch_frame(self, f: int) -> tuple[Counts, float]:
        c = Counts()
        ms = C.c_float()
        self._call("pms_batch_frame", f, C.byref(c), C.byref(ms))
        return c, float(ms.value)

    def batch_mesh(self, f: int) -> np.ndarray:
        n = C.c_uint64()
        self._call("pms_batch_mesh", f, None, 0, C.byref(n))
        out = np.zeros((n.value, 3), np.float32)
        if n.value:
            self._call("pms_batch_mesh", f, _ptr(out), n.value, C.byref(n))
        return out

    def batch_stream_meshes(self, ptr: int, cap_vertices: int) -> None:
        """Register a page-locked host arena (raw address) that each following batch
        fills with its frames' soups inside the graph; ptr 0 unregisters."""
        self._call("pms_batch_stream_meshes", C.c_void_p(ptr or None), C.c_uint64(cap_vertices))

    def batch_mesh_range(self, f: int) -> tuple[int, int]:
        """(first vertex, vertex count) of frame f's soup in the last batch's arenas."""
        a, n = C.c_uint64(), C.c_uint64()
        self._call("pms_batch_mesh_range", f, C.byref(a), C.byref(n))
        return a.value, n.value

    def batch_diffuse(self, f: int) -> np.ndarray:
        """Live diffuse particles of frame f of the last batch: records of pos (3 float),
        ttl (int32), vel (3 float), type (int32)."""
        n = C.c_uint64()
        self._call("pms_batch_diffuse", f, None, 0, C.byref(n))
        out = np.zeros(n.value, DIFFUSE_RECORD)
        if n.value:
            self._call("pms_batch_diffuse", f, out.ctypes.data, n.value, C.byref(n))
        return out

    def batch_info(self) -> dict:
        a, b = C.c_uint32(), C.c_uint32()
        self._call("pms_batch_info", C.byref(a), C.byref(b))
        return {"graph_kernels": a.value, "captures": b.value}

    def learn_features(self, cubes) -> np.ndarray:
        cubes = np.ascontiguousarray(cubes, np.uint32)
        x = np.zeros((len(cubes), MLP_INPUTS), np.uint16)
        self._call("pms_learn_features", _ptr(cubes), len(cubes), _ptr(x))
        return x

    # results
    def counts(self) -> Counts:
        c = Counts()
        self._call("pms_get_counts", C.byref(c))
        return c

    def grid(self) -> Grid:
        g = Grid()
        self._call("pms_get_grid", C.byref(g))
        return g

    def mesh(self, normals: bool = True):
        n = C.c_uint64()
        st = lib().pms_download_mesh(self._h, None, None, 0, C.byref(n))
        if st not in (0, 4):
            _check(st, self._h)
        m = n.value
        pos = np.zeros((m, 3), np.float32)
        nrm = np.zeros((m, 3), np.float32) if normals else None
        if m:
            self._call("pms_download_mesh", _ptr(pos), _ptr(nrm), m, C.byref(n))
        return pos, nrm

    def stream_mesh_to_host(self, pos_ptr: int, nrm_ptr: int | None, cap_vertices: int) -> None:
        """Register page-locked host buffers (raw addresses) that each following
        frame's marching cubes fill on a copy stream while the later stages run;
        pos_ptr 0 unregisters.  Frames already streaming keep their buffers, so
        alternating two sets lets frame k+1 run before frame k is waited for."""
        self._call("pms_stream_mesh_to_host", C.c_void_p(pos_ptr or None), C.c_void_p(nrm_ptr or None),
                   C.c_uint64(cap_vertices))

    def wait_mesh(self) -> int:
        """Wait for the oldest streamed mesh not yet waited for; returns its vertex count."""
        n = C.c_uint64()
        self._call("pms_wait_mesh", C.byref(n))
        return n.value

    def weld(self, normals: bool = False):
        """The welded mesh of the current frame: (positions (m, 3), normals or None,
        triangle indices (t, 3))."""
        self._call("pms_weld_mesh", 1 if normals else 0)
        nv, ni = C.c_uint64(), C.c_uint64()
        self._call("pms_download_welded_mesh", None, None, C.c_uint64(0), None, C.c_uint64(0), C.byref(nv), C.byref(ni))
        pos = np.zeros((nv.value, 3), np.float32)
        nrm = np.zeros((nv.value, 3), np.float32) if normals else None
        idx = np.zeros(ni.value, np.uint32)
        self._call("pms_download_welded_mesh", _ptr(pos), _ptr(nrm), C.c_uint64(nv.value), _ptr(idx), C.c_uint64(ni.value),
                   C.byref(nv), C.byref(ni))
        return pos, nrm, idx.reshape(-1, 3)

    def stream_diffuse_to_host(self, ptr: int, cap: int) -> None:
        """Register a page-locked host buffer (raw address) of `cap` 32-byte
        pms_diffuse_particle records that each frame's diffuse stage fills on a
        copy stream; ptr 0 unregisters."""
        self._call("pms_stream_diffuse_to_host", C.c_void_p(ptr or None), C.c_uint64(cap))

    def wait_diffuse(self) -> int:
        """Wait for the oldest streamed live diffuse set not yet waited for; returns its count."""
        n = C.c_uint64()
        self._call("pms_wait_diffuse", C.byref(n))
        return n.value

    def reset_diffuse(self) -> None:
        """Drop the carried diffuse particles and restart the spawn's frame counter."""
        self._call("pms_reset_diffuse")

    def diffuse_particles(self, type_: int = -1) -> dict:
        n = C.c_uint32()
        st = lib().pms_download_diffuse(self._h, type_, None, None, None, None, None, None, None, 0, C.byref(n))
        if st not in (0, 4):
            _check(st, self._h)
        m = n.value
        out = {"pos": np.zeros((m, 3), np.float32), "vel": np.zeros((m, 3), np.float32), "type": np.zeros(m, np.int32),
               "ttl": np.zeros(m, np.int32), "wave_crest": np.zeros(m, np.float32),
               "trapped_air": np.zeros(m, np.float32), "energy": np.zeros(m, np.float32)}
        if m:
            self._call("pms_download_diffuse", type_, _ptr(out["pos"]), _ptr(out["vel"]), _ptr(out["type"]),
                       _ptr(out["ttl"]), _ptr(out["wave_crest"]), _ptr(out["trapped_air"]), _ptr(out["energy"]), m,
                       C.byref(n))
        return out

    def debug(self, name: str) -> np.ndarray:
        aid, dt = ARRAY[name]
        need = C.c_uint64()
        self._call("pms_debug_download", aid, None, 0, C.byref(need))
        buf = np.zeros(need.value // np.dtype(dt).itemsize, dt)
        if need.value:
            self._call("pms_debug_download", aid, buf.ctypes.data, need.value, C.byref(need))
        if name in ("mean", "normal", "pos_sorted", "free_normal", "diffuse_potential"):
            buf = buf.reshape(-1, 3)
        elif name == "G":
            buf = buf.reshape(-1, 10)
        return buf

    def stage_times(self) -> dict:
        ms = np.zeros(6, np.float32)
        _check(lib().pms_stage_times(self._h, ms, 6), self._h)
        return dict(zip(("grid", "anisotropy", "band", "field", "marching_cubes", "diffuse"), ms.tolist()))

    def set_wait_limit(self, polls: int) -> None:
        """First bounded wait on the tensor cores: give up after `polls` polls
        (0: at once; negative: the default bound).  For tests of the timeout path."""
        self._call("pms_debug_set_wait_limit", polls)

    @property
    def launches(self) -> int:
        return int(lib().pms_kernel_launches(self._h))


def save_band_model(path: str, model: BandModel, meta: str = "") -> None:
    _check(lib().pms_save_band_model(path.encode(), C.byref(model), meta.encode()))


def load_band_model(path: str) -> BandModel:
    m = BandModel()
    _check(lib().pms_load_band_model(path.encode(), C.byref(m)))
    return m


class Trainer:
    """pms_trainer: fp32 master weights and Adam state of the band MLP; the
    forward and backward passes run in libpms's BF16 tensor-core kernels."""

    def __init__(self, device: int = 0, seed: int = 1):
        h = C.c_void_p()
        _check(lib().pms_trainer_create(device, seed, C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pms_trainer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ctx: "Context", batch: int, seed: int, lr: float, pos_weight: float, want_loss: bool = True):
        """One Adam step on a batch sampled from ctx's prepared candidates, on ctx's
        stream; returns the batch loss (a synchronisation), or None without waiting."""
        loss = C.c_float()
        _check(lib().pms_trainer_step(self._h, ctx.handle, batch, seed, lr, pos_weight,
                                      C.byref(loss) if want_loss else None), ctx.handle)
        return float(loss.value) if want_loss else None

    def grad(self, x_bf16: np.ndarray, y: np.ndarray, pos_weight: float) -> tuple[np.ndarray, float]:
        x = np.ascontiguousarray(x_bf16, np.uint16)
        yy = np.ascontiguousarray(y, np.uint8)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        _check(lib().pms_trainer_grad(self._h, _ptr(x), _ptr(yy), len(yy), pos_weight, _ptr(g), C.byref(loss)))
        return g, float(loss.value)

    def params(self) -> np.ndarray:
        w = np.zeros(MLP_PARAMS, np.float32)
        _check(lib().pms_trainer_get_params(self._h, _ptr(w)))
        return w

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32)
        _check(lib().pms_trainer_set_params(self._h, _ptr(w)))

    def model(self, threshold: float = 0.0) -> BandModel:
        m = BandModel()
        _check(lib().pms_trainer_get_model(self._h, C.byref(m)))
        m.threshold = threshold
        return m
