"""Benchmark: particles/s of the particle-to-surface pipeline on one GB300.

Workload (default): the 2M-particle crown splash -- a 200x200x40 jittered
pool slab (lattice 0.005) plus a seeded 400k-particle ring launched radially
at N(1.5, 0.3) m/s and advected 0.05 s; h = 0.01, scalar-grid cell 0.0025,
iso 0.5, synthetic (seeded) data.  A step is one frame: the inputs are copied
into the context (device to device for `value`, pinned host to device for
`e2e`), then hashing, anisotropy, narrow band, field and marching cubes run;
e2e also reads the mesh back to the host.  L2 is flushed (a 256 MiB write)
between timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl pms|reference]

--impl reference times the reference algorithm's CPU restatement (the float64
oracle, OpenMP over all host cores) on a bounded sample of the same frame:
the reference itself has no CPU implementation of this path and its CUDA
sources do not build with this toolchain.
Multi-GPU runs (torchrun) are frame-level replicas: each rank reconstructs its
own frame, no collective touches the data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
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


def workload(name: str):
    from postmps_gb300 import synth
    if name == "crown":
        pos, vel, rho = synth.crown_splash()
        keys = {"sim.particlespacing": 0.005}
        desc = {"workload": "crown_splash_2M", "particles": int(len(pos)), "h": 0.01, "grid_cell": 0.0025,
                "iso": 0.5, "clamp_ratio": 4}
    elif name == "block":
        pos, vel, rho = synth.water_block(64)
        keys = {}
        desc = {"workload": "water_block_262k", "particles": int(len(pos)), "h": 0.02, "grid_cell": 0.005, "iso": 0.5}
    else:
        raise SystemExit(f"unknown workload {name}")
    return pos, vel, rho, keys, desc


def write_config(keys: dict) -> str:
    from postmps_gb300 import synth
    fd, path = tempfile.mkstemp(suffix=".txt")
    with os.fdopen(fd, "w") as f:
        f.write(synth.config_text(**keys))
    return path


# ---------------------------------------------------------------------------
# algorithmic bytes per stage, from the frame's own counts
# ---------------------------------------------------------------------------
def algorithmic_bytes(c: dict, g, diffuse: bool) -> dict:
    N, Ns, Vs, Cv, M = c["n_particles"], c["n_surface_particles"], c["n_band_vertices"], c["n_valid_cubes"], \
        c["n_mesh_vertices"]
    Ssp, Ssc = g.sp_size, g.sc_size
    P = max(1, -(-int(np.ceil(np.log2(max(Ssp, 2)))) // 8))
    grid = (16 * N + Ssp / 8) + 16 * N * P + (32 * N + (24 * N if diffuse else 0)) + (4 * N + 8 * Ssp)
    aniso = (Ssp / 8 + 8 * Ssp + 4 * Ns) + (16 * N + 68 * Ns) + 20 * N
    band = 2 * Ssc / 8 + (Ssc / 8 + 4 * Vs)
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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


def cpu_baseline(pos, keys: dict, frac: float = 0.25) -> dict:
    """Float64 oracle of the plain path on an x-slab holding `frac` of the frame."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from postmps_gb300 import synth
    O.build()
    p = O.derive_params(O.config_from_keys(synth.keys_of(**keys)))
    xs = np.sort(pos[:, 0])
    cut = xs[int(frac * (len(xs) - 1))]
    sub = np.ascontiguousarray(pos[pos[:, 0] <= cut])
    t = time.perf_counter()
    O.run_surface(p, sub)
    dt = time.perf_counter() - t
    cores = os.cpu_count() or 1
    return {"value": len(sub) / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"x-slab with {len(sub)} of {len(pos)} particles, float64 oracle, surface path, {dt:.2f} s"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pos, vel, rho, keys, desc = workload(args.workload)
    for _ in range(args.warmup):
        cpu_baseline(pos, keys, args.cpu_fraction)
    vals, dts = [], []
    for _ in range(args.steps):
        t = time.perf_counter()
        cb = cpu_baseline(pos, keys, args.cpu_fraction)
        dts.append(time.perf_counter() - t)
        vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(dts)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(desc, sample_fraction=args.cpu_fraction, path="plain surface"),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


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
    from postmps_gb300 import pms
    pos, vel, rho, keys, desc = workload(args.workload)
    cfg_path = write_config(keys)
    cfg = pms.load_config(cfg_path)
    os.unlink(cfg_path)
    cfg.is_surface = 1
    cfg.is_diffuse = 0 if args.no_diffuse else 1
    stream = torch.cuda.current_stream()
    ctx = pms.Context(cfg, local)
    ctx.set_stream(stream.cuda_stream)
    n = len(pos)
    d_pos = torch.from_numpy(pos).cuda()
    d_vel = torch.from_numpy(vel).cuda()
    d_rho = torch.from_numpy(rho).cuda()
    h_pos = torch.from_numpy(pos).pin_memory()
    h_vel = torch.from_numpy(vel).pin_memory()
    h_rho = torch.from_numpy(rho).pin_memory()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step_device():
        ctx.upload_device(d_pos.data_ptr(), d_vel.data_ptr(), d_rho.data_ptr(), n)
        ctx.run_frame()

    mesh_host = {}

    def step_e2e():
        # the user's calls: upload from pinned host memory, reconstruct, read the
        # triangle soup (and the live diffuse particles) back into pinned memory
        ctx._call("pms_upload_particles", h_pos.data_ptr(), h_vel.data_ptr(), h_rho.data_ptr(), n)
        ctx.run_frame()
        import ctypes as C
        nv = C.c_uint64()
        pms.lib().pms_download_mesh(ctx.handle, None, None, 0, C.byref(nv))
        buf = mesh_host.get("mesh")
        if buf is None or buf.numel() < 3 * nv.value:
            buf = mesh_host["mesh"] = torch.empty(max(3, int(3 * nv.value * 1.25)), dtype=torch.float32).pin_memory()
        ctx._call("pms_download_mesh", buf.data_ptr(), None, buf.numel() // 3, C.byref(nv))
        if cfg.is_diffuse:
            mesh_host["diffuse"] = ctx.diffuse_particles(-1)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    counts = ctx.counts().as_dict()
    grid = ctx.grid()
    stage_sum = {k: 0.0 for k in ("grid", "anisotropy", "band", "field", "marching_cubes", "diffuse")}

    def timed(fn, k):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for i in range(k):
            flush.zero_()
            ev[i][0].record(stream)
            fn()
            ev[i][1].record(stream)
            if fn is step_device:
                for s, v in ctx.stage_times().items():
                    stage_sum[s] += v
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / k
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launches
    ms = timed(step_device, args.steps)
    launches = (ctx.launches - l0) // max(1, args.steps)
    clk = clocks.stop()
    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    ms_e2e = timed(step_e2e, args.steps)
    m_vertices = int(counts["n_mesh_vertices"])

    value = world * n / (ms / 1e3)
    e2e_value = world * n / (ms_e2e / 1e3)
    stage_ms = {k: v / args.steps for k, v in stage_sum.items()}
    alg = algorithmic_bytes(counts, grid, diffuse=bool(cfg.is_diffuse))
    dom = max(alg, key=lambda k: stage_ms.get(k, 0.0))
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = alg[dom] / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else None
    traffic = None
    tfile = os.path.join(ROOT, "profiles", f"traffic_{desc['workload']}.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            traffic = json.load(f).get(dom)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(desc, path="surface + diffuse" if cfg.is_diffuse else "surface (diffuse off)", band="plain",
                       l2="flushed (256 MiB write) between steps",
                       parallelism=f"replicas x{world}"),
        "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": ms_e2e, "h2d_bytes_per_step": 28 * n,
                "d2h_bytes_per_step": 12 * m_vertices + 32 * int(counts["n_diffuse"])},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes": alg[dom], "peak_source": peak_src},
        "stage_ms": stage_ms,
        "counts": counts,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pos, keys, args.cpu_fraction)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pms", choices=["pms", "reference"])
    ap.add_argument("--workload", default="crown", choices=["crown", "block"])
    ap.add_argument("--cpu-fraction", type=float, default=0.25)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-diffuse", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_pms(args)


if __name__ == "__main__":
    main()
