"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference ships no tests or fixtures, so the fixtures are produced by
running the reference's own kernels (NeighborSearch_kernel.cuh,
Anisotropic_kernel.cuh, MarchingCube_kernel.cuh, SVD3.cuh, myCuda.cuh) and its
Params.cpp, compiled unmodified for the CPU by ``make -C oracle ref`` (see
oracle/ref_emu/).  Needs the reference tree, named by $PMS_REFERENCE_DIR; the
committed .npz files are what the tests read.

    PMS_REFERENCE_DIR=path/to/PostMPS python tests/golden/make_golden.py [mc]   (mc: the table counts only)
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from postmps_gb300 import synth  # noqa: E402


def drops_and_sheet():
    """A 12^3 block, a thin two-layer sheet above it (flat covariances:
    thin-feature flag) and isolated droplets (fewer than MinNumNeighbors
    neighbours: isotropic kernel)."""
    pos, vel, rho = synth.water_block(12)
    sheet = synth.lattice(14, 14, 2, 0.01, 0.001, seed=11, origin=(-0.01, -0.01, 0.16))
    drops = synth.lattice(3, 3, 1, 0.05, 0.004, seed=12, origin=(0.0, 0.0, 0.24))
    tiny = synth.lattice(2, 2, 2, 0.009, 0.0005, seed=13, origin=(0.2, 0.2, 0.05))
    p = np.concatenate([pos, sheet, drops, tiny]).astype(np.float32)
    v = (synth.uniform(14, 0, 3 * len(p)).reshape(-1, 3) - 0.5).astype(np.float32)
    return p, v, np.full(len(p), 1000.0, np.float32)


CASES = {
    # name: (particles, config overrides)
    "block10": (lambda: synth.water_block(10), {}),
    "block16": (lambda: synth.water_block(16), {}),
    "drops_sheet": (drops_and_sheet, {}),
    "block12_ratio4": (lambda: synth.water_block(12), {"surface.smoothingradiusratio": 4}),
    "block12_iso03_scale3": (lambda: synth.water_block(12),
                             {"surface.isovalue": 0.3, "domain.sclargridsizescale": 3}),
}


def tables_digest() -> str:
    e, t, nv, ev = O.ref_mc_tables()
    h = hashlib.sha256()
    for a in (e, t, nv, ev):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make(name: str) -> str:
    gen, over = CASES[name]
    pos, vel, rho = gen()
    text = synth.config_text(**over)
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        cfg_path = f.name
    try:
        R = O.ref_surface_run(cfg_path, pos, vel, rho)
    finally:
        os.unlink(cfg_path)
    assert R["rc"] == 0, (name, R["rc"])
    sl = R["surf_list"]
    out = dict(
        config=np.array(text), pos=pos, vel=vel, rho_in=rho,
        min_pos=R["min_pos"], max_pos=R["max_pos"], scmin_pos=R["scmin_pos"], scmax_pos=R["scmax_pos"],
        spres=R["spres"], scres=R["scres"], h=np.float32(R["h"]), h_inv=np.float32(R["h_inv"]),
        iso=np.float32(R["iso"]), keys_sorted=R["keys_sorted"], perm=R["perm"], cell_start=R["cell_start"],
        cell_end=R["cell_end"], surf_count=R["surf_count"], surf_list=sl, rho=R["rho"], mean=R["mean"], G=R["G"],
        nrm=R["nrm"][sl], flag=(R["flag"][sl] != 0).astype(np.uint8), band_list=R["band_list"], field=R["field"],
        cube_flag=R["cube_flag"], nvert=R["nvert"], vpos=R["vpos"], vnrm=R["vnrm"], sval=R["sval"],
        n_surface=np.uint32(R["n_surface"]), n_band=np.uint32(R["n_band"]), n_valid=np.uint32(R["n_valid"]),
        n_mesh=np.uint32(R["n_mesh"]), mc_tables_sha256=np.array(tables_digest()),
    )
    path = os.path.join(HERE, f"surface_{name}.npz")
    np.savez_compressed(path, **out)
    return path


DIFFUSE_SEED = 4


def diffuse_frames():
    """Two frames of a 14^3 block stirred with random velocities (sigma 2.5 m/s):
    frame 1 is frame 0 advected by v * 0.02 s, and carries frame 0's diffuse
    particles.  Diffuse keys as the reference's bin/config.txt."""
    pos0, _, rho = synth.water_block(14)
    vel = (synth.normal(21, 0, 3 * len(pos0)).reshape(-1, 3) * 2.5).astype(np.float32)
    pos1 = (pos0 + 0.02 * vel).astype(np.float32)
    return [(pos0, vel, rho), (pos1, vel, rho)]


def make_diffuse() -> str:
    text = synth.config_text(**{"config.isdiffusegeneration": "true"})
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        cfg_path = f.name
    out = {"config": np.array(text), "seed": np.uint64(DIFFUSE_SEED)}
    old = None
    try:
        for fr, (pos, vel, rho) in enumerate(diffuse_frames()):
            R = O.ref_diffuse_frame(cfg_path, pos, vel, rho, True, old, DIFFUSE_SEED, fr)
            assert R["rc"] == 0, R["rc"]
            out[f"f{fr}_pos"], out[f"f{fr}_vel"], out[f"f{fr}_rho"] = pos, vel, rho
            for k in ("perm", "free_list", "nrm", "pot", "num", "gen", "old_after", "live"):
                out[f"f{fr}_{k}"] = R[k]
            out[f"f{fr}_old_in"] = np.zeros((0, 8), np.float32) if old is None else old
            old = R["live"]
    finally:
        os.unlink(cfg_path)
    path = os.path.join(HERE, "diffuse_block14.npz")
    np.savez_compressed(path, **out)
    return path


def make_mc_counts() -> str:
    """The reference's marching-cubes edge flags and vertex counts per case
    (MarchingCubesHelper.cpp), for the check of the tables libpms derives."""
    e, tri, nv, ev = O.ref_mc_tables()
    path = os.path.join(HERE, "mc_tables_counts.npz")
    np.savez_compressed(path, edge_flags=np.asarray(e, np.uint32), num_vertices=np.asarray(nv, np.uint32))
    return path


def main() -> int:
    if not os.environ.get("PMS_REFERENCE_DIR"):
        print("set PMS_REFERENCE_DIR to the reference checkout: the fixtures come from its own kernels",
              file=sys.stderr)
        return 1
    O.build()
    if not O.ref_available():
        print("the reference's kernels did not build from PMS_REFERENCE_DIR: cannot generate fixtures", file=sys.stderr)
        return 1
    p = make_mc_counts()
    print(f"{p}: {os.path.getsize(p) / 1024:.0f} KiB")
    if sys.argv[1:] == ["mc"]:
        return 0
    for name in CASES:
        p = make(name)
        print(f"{p}: {os.path.getsize(p) / 1024:.0f} KiB")
    p = make_diffuse()
    print(f"{p}: {os.path.getsize(p) / 1024:.0f} KiB")
    return 0


if __name__ == "__main__":
    sys.exit(main())
