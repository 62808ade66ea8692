"""Benchmark: particles/s of the particle-to-surface pipeline on one GB300.

Workloads (seeded synthetic data; --workload):
  crown    (default) the 2M-particle crown splash -- a 200x200x40 jittered pool
           slab (lattice 0.005) plus a seeded 400k-particle ring launched
           radially at N(1.5, 0.3) m/s and advected 0.05 s; h = 0.01, scalar
           cell 0.0025, iso 0.5, diffuse generation on.  A step is one frame.
  block    the 262,144-particle water block (64^3, spacing 0.01), diffuse off.
  slosh16  16 sloshing-tank frames of 100k-1.5M particles (14.3M in all),
           spacing 0.01, reconstructed by one pms_run_batch call (one CUDA
           graph launch); a step is the whole batch.
  dam      the 8M-particle dam break (400x100x200, spacing 0.005), diffuse off.
  crown4   four consecutive crown frames (8M particles), diffuse generation on
           and carried from frame to frame, one pms_run_batch call; a step is
           the whole batch (the carried particles dropped between steps).

Bands (--band): "learned" runs the learned narrow band (the network picks the
band vertices evaluated exactly at once, the exact sign certification covers
the rest), "certified" the certification alone, "plain" the reference's band;
the default runs all three on the same frames, reports the learned arm as the
headline (when a trained model is present, its meshes equal the plain ones and
it is faster end to end) and the others beside it, and judges each mesh
against the plain mesh (identical soups, triangle-count delta, Hausdorff
distance in units of h).

`value` is measured with the inputs already on the device (device-to-device
upload inside the step); `e2e` goes through the C ABI as a pipelined frame
loop, frames in flight on both ends: each step takes the frame staged during
the step before, stages the next frame from pinned host buffers
(pms_stage_particles, on another thread, while its own frame runs), streams its
triangle soup (and live diffuse particles) into one of two alternating pinned
host buffer sets and waits for the step before's, whose copies ran beside it.
One CUDA-event interval covers the K steps and the drain of the last one's
results.  L2 is flushed (a 256 MiB write) between steps; in the end-to-end loop
the flushes lie inside the interval.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl pms|reference]

--impl reference times the reference algorithm's CPU restatement (the float64
oracle, OpenMP over all host cores) on the whole frame of the same workload and
configuration (the reference itself has no CPU implementation of this path);
the GPU arm's line carries the reference's own CUDA build, timed on this GPU,
as `reference_cuda`.
Multi-GPU runs (torchrun) are frame-level replicas: each rank reconstructs its
own frames, no collective touches the data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particles/s end-to-end, plain vs learned-band, at <=0.05h Hausdorff vs FP64"
UNIT = "particles/s"
STAGES = ("grid", "anisotropy", "band", "field", "marching_cubes", "diffuse")


def workload(name: str):
    """(frames, keys, description, diffuse): frames is a list of (pos, vel, rho)."""
    from postmps_gb300 import synth
    if name == "crown":
        frames = [synth.crown_splash()]
        keys = dict(synth.CROWN_KEYS)
        desc = {"workload": "crown_splash_2M", "particles": int(len(frames[0][0])), "h": 0.01, "grid_cell": 0.0025,
                "iso": 0.5, "clamp_ratio": 4}
        return frames, keys, desc, True
    if name == "block":
        frames = [synth.water_block(64)]
        desc = {"workload": "water_block_262k", "particles": int(len(frames[0][0])), "h": 0.02, "grid_cell": 0.005,
                "iso": 0.5}
        return frames, {}, desc, False
    if name == "slosh16":
        frames = [synth.sloshing_tank(k, 16) for k in range(16)]
        ns = [len(f[0]) for f in frames]
        desc = {"workload": "sloshing_tank_16_frames", "frames": 16, "particles": int(sum(ns)),
                "particles_per_frame": [min(ns), max(ns)], "h": 0.02, "grid_cell": 0.005, "iso": 0.5}
        return frames, {}, desc, False
    if name == "crown4":
        # four consecutive frames of the crown (the ring advected 4 ms per frame), diffuse
        # particles carried from frame to frame: one batch, diffuse inside the graph
        base = synth.crown_splash()
        frames = [((base[0] + np.float32(0.004 * i) * base[1]).astype(np.float32), base[1], base[2]) for i in range(4)]
        keys = dict(synth.CROWN_KEYS)
        desc = {"workload": "crown_splash_4_frames", "frames": 4, "particles": int(sum(len(f[0]) for f in frames)),
                "h": 0.01, "grid_cell": 0.0025, "iso": 0.5, "clamp_ratio": 4}
        return frames, keys, desc, True
    if name == "dam":
        frames = [synth.dam_break()]
        keys = {"sim.particlespacing": 0.005}
        desc = {"workload": "dam_break_8M", "particles": int(len(frames[0][0])), "h": 0.01, "grid_cell": 0.0025,
                "iso": 0.5}
        return frames, keys, desc, False
    raise SystemExit(f"unknown workload {name}")


def write_config(keys: dict) -> str:
    from postmps_gb300 import synth
    fd, path = tempfile.mkstemp(suffix=".txt")
    with os.fdopen(fd, "w") as f:
        f.write(synth.config_text(**keys))
    return path


# ---------------------------------------------------------------------------
# algorithmic bytes per stage, from the frame's own counts
# ---------------------------------------------------------------------------
def dominant_stage(stage_ms: dict, alg: dict, diffuse: bool) -> str:
    """The stage whose kernel the roofline reports: the longest on the frame's stream.  With
    surface and diffuse on, the diffuse stage runs on its own stream beside the band, field
    and marching cubes, so its time is a span from the anisotropy's end, not a cost of its
    own, and it is left out."""
    serial = [k for k in alg if not (diffuse and k == "diffuse")]
    return max(serial, key=lambda k: stage_ms.get(k, 0.0))


def algorithmic_bytes(c: dict, sp_size: int, sc_size: int, diffuse: bool, learned: bool) -> dict:
    N, Ns, Vs, Cv, M = c["n_particles"], c["n_surface_particles"], c["n_band_vertices"], c["n_valid_cubes"], \
        c["n_mesh_vertices"]
    Ssp, Ssc = sp_size, sc_size
    P = max(1, -(-int(np.ceil(np.log2(max(Ssp, 2)))) // 8))
    grid = (16 * N + Ssp / 8) + 16 * N * P + (32 * N + (24 * N if diffuse else 0)) + (4 * N + 8 * Ssp)
    aniso = (Ssp / 8 + 8 * Ssp + 4 * Ns) + (16 * N + 68 * Ns) + 20 * N
    band = 2 * Ssc / 8 + (Ssc / 8 + 4 * Vs)
    if learned:
        coarse = Ssc / 8
        # on top of the plain band: coarse counts (read positions, write counts), prediction
        # (read counts, write cube bits), the split (read cube and band bits, write two
        # bitmaps) and its two lists
        band += (16 * N + 4 * coarse) + (4 * coarse + Ssc / 8) + 3 * Ssc / 8 + 4 * Vs
    field = 16 * N + 44 * Ns + 8 * Vs
    mc = (4 * Vs + Ssc / 8 + 9 * Vs) + (12 * 8 * Cv + 24 * M)
    dif = (64 * N + 44 * (c["n_generated_diffuse"] + c["n_diffuse"])) if diffuse else 0
    return {"grid": grid, "anisotropy": aniso, "band": band, "field": field, "marching_cubes": mc, "diffuse": dif}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU legs (the float64 oracle)
# ---------------------------------------------------------------------------
def cpu_baseline(frame, keys: dict, diffuse: bool) -> dict:
    """The float64 oracle on one whole frame of the workload (all host cores)."""
    t = time.perf_counter()
    info = cpu_frame(frame, keys, diffuse)
    dt = time.perf_counter() - t
    cores = os.cpu_count() or 1
    return {"value": len(frame[0]) / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one whole frame ({len(frame[0])} particles, {'surface + diffuse' if diffuse else 'surface'}), "
                      f"float64 oracle on {cores} threads, {dt:.2f} s; {info}"}


def _cube_ranges(band, nvert):
    """Valid cubes (origin ids), their cases' vertex counts and first mesh vertex."""
    nv = np.asarray(nvert, np.int64)
    off = np.concatenate([[0], np.cumsum(nv)])[:-1]
    sel = nv > 0
    return np.asarray(band)[sel], off[sel], nv[sel]


def fp64_judge(ctx, frame, keys: dict, arms, model, h: float) -> dict:
    """Every arm's frame against the float64 oracle at the benchmark configuration
    (outside the timed region): integer stages bit for bit, the field on the band
    vertices both hold (relative to max(|f|, iso), below the 2 iso early exit),
    mesh vertices of the cubes both classify alike (in cells), and the symmetric
    Hausdorff distance between the GPU and the float64 meshes (in h): vertex for
    vertex on those cubes, point to surface for the others."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from postmps_gb300 import synth
    O.build()
    pos = frame[0]
    t0 = time.perf_counter()
    p = O.derive_params(O.config_from_keys(synth.keys_of(**keys)))
    g = O.grid_from_positions(p, pos)
    r = O.run_surface(p, pos, g)
    from postmps_gb300 import pms
    e, tt, nvt, ev, _ = pms.mc_tables()
    O.set_mc_tables(e, tt, nvt, ev)
    iso = float(p.iso_value)
    cases_o, nvert_o, _ = O.mc_classify(g, iso, r.bitmap, r.band, r.field.astype(np.float32))
    mesh_o, _ = O.mc_emit(g, iso, r.bitmap, r.band, r.field, cases_o, nvert_o)
    t_oracle = time.perf_counter() - t0
    cs = float(g.sc_grid_size)
    ids_o, off_o, cnt_o = _cube_ranges(r.band, nvert_o)
    case_o = np.asarray(cases_o)[np.asarray(nvert_o) > 0]
    out = {"oracle_seconds": round(t_oracle, 2), "cores": os.cpu_count(), "triangles_fp64": int(len(mesh_o) // 3)}
    first = True
    for arm in arms:
        ctx.set_band_mode(arm)
        ctx.upload(*frame)
        ctx.build_grid()
        if arm == "plain":
            ctx.surface()
        else:
            ctx.surface_learned()
        ctx.set_band_mode("plain")
        if first:
            # integer stages: identical for every arm (computed before the band)
            ok = {k: bool(np.array_equal(ctx.debug(k), ref)) for k, ref in
                  (("keys_sorted", r.keys_sorted), ("perm", r.perm), ("cell_start", r.cell_start),
                   ("cell_end", r.cell_end), ("surf_list", r.surf_list))}
            out["integer_stages_bit_exact"] = ok
            first = False
        band = ctx.debug("band_list")
        field = ctx.debug("field").astype(np.float64)
        nvert = ctx.debug("cube_nvert")
        case = ctx.debug("cube_case")
        mesh = ctx.mesh(normals=False)[0].astype(np.float64)
        # field on the common band vertices (a learned or certified band keeps only a sign,
        # a placeholder above iso, at the vertices it certified: those are left out)
        common, ig, io = np.intersect1d(band, r.band, assume_unique=True, return_indices=True)
        fg, fo = field[ig], r.field[io]
        below = (fo < 2 * iso * 0.999) & (fg < 2 * iso * 0.999)
        certified = 0
        if arm != "plain":
            cb = ctx.debug("band_certified")
            held = ((cb[band[ig] >> 5] >> (band[ig] & 31)) & 1).astype(bool)
            certified = int(held.sum())
            below &= ~held
        ferr = float((np.abs(fg - fo) / np.maximum(np.abs(fo), iso))[below].max(initial=0.0))
        # cubes classified alike: vertex for vertex
        ids_g, off_g, cnt_g = _cube_ranges(band, nvert)
        case_g = case[nvert > 0]
        cc, jg, jo = np.intersect1d(ids_g, ids_o, assume_unique=True, return_indices=True)
        same = case_g[jg] == case_o[jo]
        vmax = 0.0
        if same.any():
            a_first = np.repeat(off_g[jg][same], cnt_g[jg][same])
            b_first = np.repeat(off_o[jo][same], cnt_o[jo][same])
            k = np.arange(len(a_first)) - np.repeat(np.cumsum(cnt_g[jg][same]) - cnt_g[jg][same], cnt_g[jg][same])
            vmax = float(np.abs(mesh[a_first + k] - mesh_o[b_first + k]).max(initial=0.0))
        # the rest (cubes in one set only, or classified differently): point to surface
        only_g = np.ones(len(ids_g), bool)
        only_g[jg[same]] = False
        only_o = np.ones(len(ids_o), bool)
        only_o[jo[same]] = False

        def verts(m, off, cnt, sel):
            if not sel.any():
                return np.zeros((0, 3))
            f = np.repeat(off[sel], cnt[sel])
            k = np.arange(len(f)) - np.repeat(np.cumsum(cnt[sel]) - cnt[sel], cnt[sel])
            return np.ascontiguousarray(m[f + k])

        qa, qb = verts(mesh, off_g, cnt_g, only_g), verts(mesh_o, off_o, cnt_o, only_o)
        da = O.lib().orc_hausdorff_vertices_to_mesh(qa.reshape(-1), len(qa), np.ascontiguousarray(mesh_o).reshape(-1),
                                                    len(mesh_o), cs) if len(qa) else 0.0
        db = O.lib().orc_hausdorff_vertices_to_mesh(qb.reshape(-1), len(qb), np.ascontiguousarray(mesh).reshape(-1),
                                                    len(mesh), cs) if len(qb) else 0.0
        hd = max(vmax, da, db)
        out[arm] = {"hausdorff_h_vs_fp64": hd / h, "max_vertex_err_cells": vmax / cs, "max_field_rel_err": ferr,
                    "field_placeholders": certified,
                    "band_vertices_differing": int(len(band) + len(r.band) - 2 * len(common)),
                    "valid_cubes_differing": int(only_g.sum() + only_o.sum()),
                    "cases_bit_exact_on_common_cubes": bool(same.all()),
                    "triangle_delta_vs_fp64": int(len(mesh) // 3 - len(mesh_o) // 3)}
    out["seconds"] = round(time.perf_counter() - t0, 2)
    return out


class RefCudaResult(C.Structure):
    _fields_ = [("seconds_per_frame", C.c_double), ("mesh_vertices", C.c_uint64), ("spray", C.c_uint64),
                ("foam", C.c_uint64), ("bubble", C.c_uint64), ("frames", C.c_int)]


def reference_cuda(frame, keys: dict, diffuse: bool, frames: int = 5) -> dict:
    """The reference's own CUDA code (its GPUPOST frame loop, compiled unmodified
    for this GPU by oracle/ref_cuda from the sources build() copied to
    baseline/_ref/src) on `frames` copies of the frame: particles from host
    memory, mesh (and diffuse particles) read back as the reference does, no file
    I/O.  Wall time per frame of its whole host + device loop."""
    lib_path = os.path.join(ROOT, "baseline", "_ref", "libref_cuda.so")
    src = os.path.join(ROOT, "baseline", "_ref", "src", "cuda")
    if not os.path.isdir(src):
        return {"unavailable": "the reference's sources were not copied to baseline/_ref/src (no reference checkout at build time)"}
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_cuda"), f"-j{os.cpu_count() or 4}"],
                       capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(lib_path):
        return {"unavailable": "the reference's CUDA sources did not build: " + (r.stderr or r.stdout)[-300:]}
    from postmps_gb300 import synth
    pos, vel, rho = (np.ascontiguousarray(a, np.float32) for a in frame)
    lib = C.CDLL(lib_path)
    lib.ref_cuda_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.POINTER(RefCudaResult)]
    res = RefCudaResult()
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "config.txt"), "w") as f:
            f.write(synth.config_text(**keys, **{"config.framefrom": 0, "config.frameto": frames - 1,
                                                "config.issurfacereconstruct": "true",
                                                "config.isdiffusegeneration": "true" if diffuse else "false"}))
        os.chdir(td)
        try:
            rc = lib.ref_cuda_run(pos.ctypes.data, vel.ctypes.data, rho.ctypes.data, len(pos), frames, 1, C.byref(res))
        finally:
            os.chdir(cwd)
    if rc != 0:
        return {"unavailable": f"ref_cuda_run returned {rc}"}
    return {"ms_per_frame": 1e3 * res.seconds_per_frame, "particles_per_s": len(pos) / res.seconds_per_frame,
            "mesh_vertices": int(res.mesh_vertices), "spray": int(res.spray), "foam": int(res.foam),
            "bubble": int(res.bubble), "frames": int(res.frames),
            "what": "the reference's GPUPOST frame loop compiled unmodified for sm_103a (texture references as "
                    "device pointers, FileData served from memory): host arrays in, mesh read back, no file I/O"}


def cpu_frame(frame, keys: dict, diffuse: bool, seed: int = 4) -> dict:
    """One whole frame through the float64 oracle (all host cores): grid, surface
    particles, density, anisotropy, plain band, field, marching cubes with the
    mesh emitted, and -- when the GPU arm has it -- the diffuse chain."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from postmps_gb300 import pms, synth
    O.build()
    pos, vel, _ = frame
    p = O.derive_params(O.config_from_keys(synth.keys_of(**keys)))
    g = O.grid_from_positions(p, pos)
    r = O.run_surface(p, pos, g)
    e, tt, nvt, ev, _ = pms.mc_tables()
    O.set_mc_tables(e, tt, nvt, ev)
    cases, nvert, _ = O.mc_classify(g, p.iso_value, r.bitmap, r.band, r.field.astype(np.float32))
    mesh, _ = O.mc_emit(g, p.iso_value, r.bitmap, r.band, r.field, cases, nvert)
    out = {"mesh_vertices": int(len(mesh))}
    if diffuse:
        d = O.diffuse_frame(p, g, r.pos_sorted, np.asarray(vel, np.float32)[r.perm], r.cell_start, r.cell_end,
                            r.surf_list, np.zeros((len(pos), 3)), seed, 0)
        out["generated_diffuse"] = int(len(d["gen"]))
    return out


def run_reference(args) -> None:
    """The reference path on the host cores: the float64 oracle (the reference has
    no CPU implementation of this pipeline) on the same frame and configuration as
    the GPU arm, every step the whole frame (surface and, where the GPU arm has it,
    diffuse).  Warm-up steps run the 262,144-particle block (CPU code needs no warm
    up beyond its first page faults), so the run stays within a few minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    frames, keys, desc, diffuse = workload(args.workload)
    if args.no_diffuse:
        diffuse = False
    from postmps_gb300 import synth
    small = synth.water_block(64)
    for _ in range(args.warmup):
        cpu_frame(small, {}, False)
    n_total = sum(len(fr[0]) for fr in frames)
    dts, info = [], {}
    for _ in range(args.steps):
        t = time.perf_counter()
        for fr in frames:
            info = cpu_frame(fr, keys, diffuse)
        dts.append(time.perf_counter() - t)
    ms = 1e3 * float(np.mean(dts))
    v = n_total / (ms / 1e3)
    cores = os.cpu_count() or 1
    cb = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
          "sample": f"the whole workload every step ({n_total} particles, "
                    f"{'surface + diffuse' if diffuse else 'surface'}), float64 oracle on {cores} threads; "
                    f"last frame: {info}"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(desc, path=("surface + diffuse" if diffuse else "surface (diffuse off)"), band="plain",
                           parallelism=f"replicas x{args.gpus}", step="one frame"),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# replicas: one frame set per rank, no collective on the data path
# ---------------------------------------------------------------------------
def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time (the job's time); a no-op on one rank."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, world: int, ms: float) -> float:
    """Whole-job units/s: every rank processed units_per_rank in at most ms."""
    return world * units_per_rank / (ms / 1e3)


# ---------------------------------------------------------------------------
# GPU arms
# ---------------------------------------------------------------------------
class Timer:
    """CUDA-event timing of K steps on the context's stream, L2 flushed between
    steps, max over ranks."""

    def __init__(self, torch, stream, world):
        self.torch, self.stream, self.world = torch, stream, world
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def __call__(self, fn, k, after=None):
        torch = self.torch
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        if self.world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for i in range(k):
            self.flush.zero_()
            ev[i][0].record(self.stream)
            fn()
            ev[i][1].record(self.stream)
            if after:
                after()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / k
        return max_over_ranks(ms, self.world, "cuda")

    def loop(self, fn, k, drain):
        """One CUDA-event interval over k pipelined steps and the drain that waits for
        the last step's results, the L2 flushes between steps included."""
        torch = self.torch
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if self.world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        self.flush.zero_()
        e0.record(self.stream)
        for i in range(k):
            if i:
                self.flush.zero_()
            fn()
        drain()
        e1.record(self.stream)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / k, self.world, "cuda")


def single_frame_arm(pms, ctx, frame, mode: str, args, timer, torch, diffuse: bool, clocks=None) -> dict:
    pos, vel, rho = frame
    n = len(pos)
    d_pos, d_vel, d_rho = (torch.from_numpy(a).cuda() for a in (pos, vel, rho))
    h_pos, h_vel, h_rho = (torch.from_numpy(a).pin_memory() for a in (pos, vel, rho))
    ctx.set_band_mode(mode)
    host = {}

    def step_device():
        ctx.upload_device(d_pos.data_ptr(), d_vel.data_ptr(), d_rho.data_ptr(), n)
        ctx.run_frame()

    stage_err = []

    def stage_next():
        st = pms.lib().pms_stage_particles(ctx.handle, h_pos.data_ptr(), h_vel.data_ptr(), h_rho.data_ptr(), n)
        if st:
            stage_err.append(st)

    # a staging thread of the loop's own, woken once per frame
    go, done, stop = threading.Semaphore(0), threading.Semaphore(0), []

    def stager():
        while True:
            go.acquire()
            if stop:
                return
            stage_next()
            done.release()

    worker = threading.Thread(target=stager, daemon=True)
    worker.start()

    def register(k):
        sm, sd = host["sets"][k % 2]
        ctx.stream_mesh_to_host(sm.data_ptr(), None, sm.numel() // 3)
        if diffuse:
            ctx.stream_diffuse_to_host(sd.data_ptr(), sd.numel() // 32)

    def take():
        host["n_mesh"] = ctx.wait_mesh()
        if diffuse:
            host["n_diffuse"] = ctx.wait_diffuse()

    def step_e2e():
        # the user's calls of a pipelined frame loop, frames in flight on both ends:
        # take the frame staged during the step before (its pinned copy and
        # host-to-device copy ran while that frame computed) and stage the next on the
        # loop's staging thread; reconstruct into this step's host buffer set (the two
        # sets alternate), the triangle soup streamed after the emission and the live
        # diffuse particles after the diffuse stage; then wait for the step before's results,
        # whose copies ran beside this frame.  The drain after the last step waits for
        # its own.  Every step moves one frame's inputs host to device inside the timed
        # region and reads one frame's results back.
        k = host["k"]
        register(k)
        ctx.upload_staged()
        go.release()
        ctx.run_frame()
        if host["pending"]:
            take()
        host["pending"] = True
        host["k"] = k + 1
        done.acquire()
        if stage_err:
            raise RuntimeError(f"pms_stage_particles failed: status {stage_err[0]}")

    def drain():
        if host["pending"]:
            take()
        host["pending"] = False

    stage_sum = {k: 0.0 for k in STAGES}

    def collect():
        for s, v in ctx.stage_times().items():
            stage_sum[s] += v

    # every arm and both timings run the same sequence: the diffuse set carried between
    # frames starts empty, so step i of each timing carries the particles of the
    # warm-up frames and of the i steps before it
    # the clock record covers the warm-up and both timings (nvidia-smi needs a moment to
    # deliver its first sample)
    if clocks:
        clocks.start()
    ctx.reset_diffuse()
    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    counts = ctx.counts().as_dict()
    grid = ctx.grid()
    l0 = ctx.launches
    ms = timer(step_device, args.steps, collect)
    launches = (ctx.launches - l0) // max(1, args.steps)
    if diffuse:
        # the carried set grows over the timed steps: its mean stands for the steps
        end = ctx.counts().as_dict()
        counts["n_diffuse_first_last"] = [int(counts["n_diffuse"]), int(end["n_diffuse"])]
        counts["n_diffuse"] = (int(counts["n_diffuse"]) + int(end["n_diffuse"])) // 2
    # two host buffer sets (pinned), the mesh's sized from the frame's mesh; the diffuse
    # set's 32-byte records: the live set grows while the same frame repeats (a spawned
    # particle lives LifefimeMultiplier frames per sibling), so the buffer has room for
    # every particle the warm-up and timed frames spawn
    cap = int(counts["n_generated_diffuse"]) * (args.warmup + args.steps + 2) + (1 << 20)
    host["sets"] = [(torch.empty(max(3, int(3 * counts["n_mesh_vertices"] * 1.25)), dtype=torch.float32).pin_memory(),
                     torch.empty(32 * cap if diffuse else 32, dtype=torch.uint8).pin_memory()) for _ in range(2)]
    host["k"], host["pending"] = 0, False
    ctx.reset_diffuse()
    stage_next()                              # the first frame of the pipelined loop
    for _ in range(args.warmup):
        step_e2e()
    drain()
    ms_e2e = timer.loop(step_e2e, args.steps, drain)
    clk = clocks.stop() if clocks else None
    stop.append(True)
    go.release()
    worker.join()
    ctx.upload_staged()                       # the frame staged by the last step
    ctx.stream_mesh_to_host(0, None, 0)
    if diffuse:
        ctx.stream_diffuse_to_host(0, 0)
    return {"ms": ms, "ms_e2e": ms_e2e, "counts": counts, "sp_size": grid.sp_size, "sc_size": grid.sc_size,
            "launches": launches, "clocks": clk, "stage_ms": {k: v / args.steps for k, v in stage_sum.items()},
            "h2d": 24 * n, "d2h": 12 * int(counts["n_mesh_vertices"]) + 32 * int(host.get("n_diffuse", 0))}


def training_rate(pms, ctx, frame, stream, torch, batch: int = 8192, steps: int = 50) -> dict:
    """Band-MLP training throughput on this frame's candidates (outside every timed
    region): Adam steps of `batch` sampled cubes, forward and backward on the tensor
    cores (k_learn_train, tcgen05) plus the Adam kernel, CUDA events on the stream."""
    ctx.set_band_mode("plain")
    ctx.upload(*frame)
    ctx.build_grid()
    ctx.surface()
    n_cand, _ = ctx.learn_prepare()
    tr = pms.Trainer(torch.cuda.current_device(), 1)
    try:
        for i in range(3):
            tr.step(ctx, batch, i, 1e-3, 4.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for i in range(steps):
            tr.step(ctx, batch, 100 + i, 1e-3, 4.0, want_loss=False)
        b.record(stream)
        b.synchronize()
        loss = tr.step(ctx, batch, 1000, 0.0, 4.0)
        ms = a.elapsed_time(b) / steps
    finally:
        tr.close()
    # forward 2*64*64 and backward 2*80*128 (M = 128 rows of dh and h over each sample)
    # multiply-adds per sample on the tensor cores
    flops = 2 * 64 * 64 + 2 * 128 * 80
    return {"samples_per_s": batch / (ms / 1e3), "ms_per_step": ms, "batch": batch, "steps": steps,
            "candidates": int(n_cand), "loss": loss, "tensor_flops_per_sample": flops,
            "kernel": "k_learn_train (tcgen05.mma kind::f16, accumulators in tensor memory) + k_adam"}


def batch_arm(pms, ctx, frames, mode: str, args, timer, torch, clocks=None, diffuse: bool = False) -> dict:
    dev = [tuple(torch.from_numpy(a).cuda() for a in fr) for fr in frames]
    pin = [tuple(torch.from_numpy(a).pin_memory() for a in fr) for fr in frames]
    dframes = [(p.data_ptr(), v.data_ptr(), r.data_ptr(), len(fr[0])) for (p, v, r), fr in zip(dev, frames)]
    hframes = [(p.data_ptr(), v.data_ptr(), r.data_ptr(), len(fr[0])) for (p, v, r), fr in zip(pin, frames)]
    host = {}
    # with diffuse generation every step is the same sequence: the carried particles are
    # dropped after each step, outside the timed region
    reset = ctx.reset_diffuse if diffuse else None
    read = {"diffuse": 0}

    def step_device():
        ctx.run_batch(dframes, learned=mode)

    def step_e2e():
        # the frames' soups land in the registered host arena inside the graph, each right
        # after its frame's emission (pms_batch_stream_meshes); the live diffuse sets are
        # read back after it
        ctx.run_batch(hframes, learned=mode)
        nd = 0
        for f in range(len(frames)):
            nv = C.c_uint64()
            ctx.batch_mesh_range(f)
            if diffuse:
                pms.lib().pms_batch_diffuse(ctx.handle, f, None, 0, C.byref(nv))
                dbuf = host.get(("d", f))
                if dbuf is None or dbuf.numel() < 32 * nv.value:
                    dbuf = host[("d", f)] = torch.empty(max(32, int(32 * nv.value * 1.25)), dtype=torch.uint8).pin_memory()
                ctx._call("pms_batch_diffuse", f, dbuf.data_ptr(), dbuf.numel() // 32, C.byref(nv))
                nd += nv.value
        read["diffuse"] = nd

    for _ in range(args.warmup):
        step_device()
        if reset:
            reset()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    l0 = ctx.launches
    ms = timer(step_device, args.steps, reset)
    launches = (ctx.launches - l0) // max(1, args.steps)
    clk = clocks.stop() if clocks else None
    per_frame = []
    counts = []
    for f in range(len(frames)):
        c, fms = ctx.batch_frame(f)
        per_frame.append(fms)
        counts.append(c.as_dict())
    mesh = sum(int(c["n_mesh_vertices"]) for c in counts)
    host["arena"] = torch.empty(3 * (int(mesh * 1.25) + 1024), dtype=torch.float32).pin_memory()
    ctx.batch_stream_meshes(host["arena"].data_ptr(), host["arena"].numel() // 3)
    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
        if reset:
            reset()
    ms_e2e = timer(step_e2e, args.steps, reset)
    ctx.batch_stream_meshes(0, 0)
    return {"ms": ms, "ms_e2e": ms_e2e, "launches": launches, "clocks": clk, "frame_ms": per_frame,
            "counts": counts, "info": ctx.batch_info(), "h2d": sum(28 * len(fr[0]) for fr in frames),
            "d2h": 12 * mesh + 32 * read["diffuse"]}


def unbatched_ms(ctx, frames, mode: str, args, timer, torch) -> float:
    """The same frames through pms_run_frame one by one (device-resident inputs)."""
    dev = [tuple(torch.from_numpy(a).cuda() for a in fr) for fr in frames]
    ctx.set_band_mode(mode)

    def step():
        for (p, v, r), fr in zip(dev, frames):
            ctx.upload_device(p.data_ptr(), v.data_ptr(), r.data_ptr(), len(fr[0]))
            ctx.run_frame()

    ctx.reset_diffuse()
    step()
    ctx.reset_diffuse()
    torch.cuda.synchronize()
    return timer(step, max(1, args.steps // 2), ctx.reset_diffuse)


def run_pms(args) -> None:
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    from postmps_gb300 import learned as LN, pms
    frames, keys, desc, diffuse = workload(args.workload)
    if args.no_diffuse:
        diffuse = False
    cfg_path = write_config(keys)
    cfg = pms.load_config(cfg_path)
    os.unlink(cfg_path)
    cfg.is_surface = 1
    cfg.is_diffuse = 1 if diffuse else 0
    h = float(pms.derive_params(cfg).h)
    # one non-default stream for everything: libpms's work, the L2 flush and the
    # timing events are ordered on it (a NULL handle would give the context its own stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = pms.Context(cfg, local)
    ctx.set_stream(stream.cuda_stream)
    timer = Timer(torch, stream, world)
    model = None
    if args.band in ("both", "learned") and os.path.exists(args.model):
        model = LN.load_model(args.model)
        ctx.set_band_model(model)
    # learned: the network plus the exact sign certification; certified: the
    # certification alone (what the network adds); plain: the reference's band
    if args.band == "both":
        arms = (["learned"] if model is not None else []) + ["certified", "plain"]
    else:
        arms = [args.band]
    if "learned" in arms and model is None:
        raise SystemExit(f"--band learned needs a model ({args.model})")
    batched = args.workload in ("slosh16", "crown4")
    tune = None
    if not args.no_tune:
        # autotune the launch shapes on the largest frame, as the first (headline) arm
        # reconstructs it (outside the timed region)
        big = max(frames, key=lambda fr: len(fr[0]))
        ctx.upload(*big)
        ctx.build_grid()
        ctx.set_band_mode(arms[0])
        if arms[0] != "plain":
            ctx.surface_learned()
        else:
            ctx.surface()
        ctx.set_band_mode("plain")
        tune = ctx.autotune()
    res = {}
    for i, arm in enumerate(arms):
        if batched:
            res[arm] = batch_arm(pms, ctx, frames, arm, args, timer, torch, ClockSampler(local), diffuse)
        else:
            res[arm] = single_frame_arm(pms, ctx, frames[0], arm, args, timer, torch, diffuse, ClockSampler(local))
    ctx.set_band_mode("plain")
    # the judge: each non-plain band's mesh against the plain mesh of the same frame
    # (outside the timed region; every frame of the workload -- a batch gives each
    # frame the single-frame result)
    judge = {}
    if "plain" in arms and len(arms) > 1 and not args.no_judge:
        for arm in arms:
            if arm == "plain":
                continue
            t0 = time.perf_counter()
            js = [LN.compare(ctx, model if arm == "learned" else None, h, *fr, mode=arm) for fr in frames if len(fr[0])]
            worst = max(js, key=lambda j: j["hausdorff"])
            judge[arm] = {"identical_frames": sum(j["identical"] for j in js), "frames": len(js),
                          "hausdorff_h": worst["hausdorff_h"], "hausdorff": worst["hausdorff"],
                          "triangle_delta": sum(j["triangle_delta"] for j in js),
                          "cubes_only_plain": sum(j["cubes_only_plain"] for j in js),
                          "cubes_only_learned": sum(j["cubes_only_learned"] for j in js),
                          "work": {k: sum(j["learned"][k] for j in js)
                                   for k in ("band_vertices", "exact_first", "certified", "rechecked", "full_walks",
                                             "predicted")},
                          "seconds": time.perf_counter() - t0}
    # every arm against the float64 oracle at this configuration (single-frame workloads)
    fp64 = None
    if not batched and not args.no_fp64 and rank == 0:
        fp64 = fp64_judge(ctx, frames[0], keys, arms, model, h)
    # headline: the learned band when it is within 0.05 h of the float64 mesh, its meshes
    # are the plain ones on every frame, and it is faster end to end
    head_arm = arms[0]
    if "learned" in arms and "plain" in arms:
        j = judge.get("learned")
        ok = j is not None and j["identical_frames"] == j["frames"]
        if fp64 is not None:
            ok = ok and fp64["learned"]["hausdorff_h_vs_fp64"] <= 0.05
        head_arm = "learned" if ok and res["learned"]["ms_e2e"] < res["plain"]["ms_e2e"] else "plain"
    head = res[head_arm]
    n_total = sum(len(fr[0]) for fr in frames)
    value = job_throughput(n_total, world, head["ms"])
    e2e_value = job_throughput(n_total, world, head["ms_e2e"])
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(desc, path=("surface + diffuse" if diffuse else "surface (diffuse off)"), band=head_arm,
                       l2=("flushed (256 MiB write) between steps" + ("" if batched else
                                                                          " (inside the end-to-end loop's interval)")),
                       parallelism=f"replicas x{world}",
                       step=("one pms_run_batch call (one CUDA graph launch)" if batched else "one frame")),
        "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": head["ms_e2e"], "h2d_bytes_per_step": head["h2d"],
                "d2h_bytes_per_step": head["d2h"]},
        "clocks": head["clocks"],
        "gpu_launches": int(head["launches"]),
        "tune": tune,
    }
    for arm in arms:
        r = res[arm]
        line[arm] = {"value": world * n_total / (r["ms"] / 1e3), "e2e": world * n_total / (r["ms_e2e"] / 1e3),
                     "ms_per_step": r["ms"], "ms_e2e": r["ms_e2e"]}
        if batched:
            line[arm].update({"frame_ms": r["frame_ms"], "graph": r["info"],
                              "band_vertices": sum(c["n_band_vertices"] for c in r["counts"]),
                              "triangles": sum(c["n_mesh_vertices"] for c in r["counts"]) // 3})
        else:
            line[arm].update({"stage_ms": r["stage_ms"], "counts": r["counts"]})
    if batched:
        line["unbatched_ms_per_step"] = unbatched_ms(ctx, frames, head_arm, args, timer, torch)
        # whole-path bytes of every frame over the whole batch time
        tot = 0.0
        for fr_c in head["counts"]:
            tot += sum(algorithmic_bytes(fr_c if diffuse else dict(fr_c, n_generated_diffuse=0, n_diffuse=0),
                                         fr_c["n_particles"], fr_c["n_band_vertices"], diffuse, head_arm != "plain").values())
        achieved = tot / (head["ms"] / 1e3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": "whole batch", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": None, "algorithmic_bytes": tot, "peak_source": peak_src}
    else:
        stage_ms = head["stage_ms"]
        alg = algorithmic_bytes(head["counts"], head["sp_size"], head["sc_size"], diffuse, head_arm != "plain")
        dom = dominant_stage(stage_ms, alg, diffuse)
        achieved = alg[dom] / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else None
        traffic = None
        tfile = os.path.join(ROOT, "profiles", f"traffic_{desc['workload']}.json")
        if os.path.exists(tfile):
            with open(tfile) as f:
                tj = json.load(f)
            traffic = tj.get(f"{head_arm}:{dom}", tj.get(dom))
        line["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                            "algorithmic_bytes": alg[dom], "peak_source": peak_src}
        # the field's own work: (band vertex, particle) pairs it evaluated, against the FP32
        # rate of the SMs (about 10 FP32 operations per pair: the r^T M r form, (1 - d2)^3 w, the sum)
        pairs = int(head["counts"].get("n_field_pairs", 0))
        fms = stage_ms.get("field", 0.0)
        if pairs and fms > 0:
            sm_mhz = (head["clocks"] or {}).get("sm_mhz") or 2070.0
            peak_fp32 = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12      # TFLOP/s, FMA = 2
            rate = pairs / (fms / 1e3)
            line["field_compute"] = {"pair_evals": pairs, "pair_evals_per_s": rate, "flops_per_pair": 10,
                                     "achieved_tflops": rate * 10 / 1e12, "peak_tflops_fp32": peak_fp32,
                                     "frac": rate * 10 / 1e12 / peak_fp32,
                                     "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x the sampled SM clock"}
        line["stage_ms"] = stage_ms
        if diffuse:
            line["stage_note"] = ("diffuse runs on its own stream beside band, field and marching cubes; its "
                                  "stage_ms is the span from the anisotropy's end to its own end")
        line["counts"] = head["counts"]
    if not batched and not args.no_train and rank == 0:
        line["training"] = training_rate(pms, ctx, frames[0], stream, torch)
    if judge:
        line["judge"] = judge
    if fp64 is not None:
        line["fp64"] = fp64
    if rank == 0 and not batched and not args.no_ref_cuda:
        line["reference_cuda"] = reference_cuda(frames[0], keys, diffuse)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(frames[0], keys, diffuse)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    from postmps_gb300 import learned as LN
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pms", choices=["pms", "reference"])
    ap.add_argument("--workload", default="crown", choices=["crown", "block", "slosh16", "dam", "crown4"])
    ap.add_argument("--band", default="both", choices=["both", "learned", "certified", "plain"])
    ap.add_argument("--model", default=LN.DEFAULT_MODEL)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-diffuse", action="store_true")
    ap.add_argument("--no-train", action="store_true", help="skip timing the band-MLP training step")
    ap.add_argument("--no-judge", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the float64 oracle judge")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference's own CUDA build")
    ap.add_argument("--no-tune", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_pms(args)


if __name__ == "__main__":
    main()
