"""Learned narrow band: training driver, model files, evaluation and the
Hausdorff judge.

The network and its training run on the GPU in libpms (BF16 forward and
backward kernels on the tensor cores, Adam on fp32 master weights); this
module only sequences frames, steps and thresholds.  Labels come from the
plain method: a candidate cube is positive when the plain marching cubes
finds it valid.  The plain method also stays the judge: a learned mesh is
compared with the plain mesh of the same frame by triangle-count delta and by
the Hausdorff distance between the two triangle soups (in units of h).

Usage (one GPU):
    python -m postmps_gb300.learned train --out postmps_gb300/models/band_crown.pmsband
    python -m postmps_gb300.learned eval --model postmps_gb300/models/band_crown.pmsband
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import tempfile
import time

import numpy as np

from . import pms, synth

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "models", "band_crown.pmsband")
TRAIN_SEEDS = range(100, 150)
HELD_OUT_SEEDS = range(200, 210)


# ---------------------------------------------------------------------------
# model files
# ---------------------------------------------------------------------------
def save_model(path: str, model: "pms.BandModel", meta: dict | None = None) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    pms.save_band_model(path, model, json.dumps(meta or {}))


def load_model(path: str = DEFAULT_MODEL) -> "pms.BandModel":
    return pms.load_band_model(path)


def model_meta(path: str = DEFAULT_MODEL) -> dict:
    with open(path, "rb") as f:
        raw = f.read()
    off = 16 + C.sizeof(pms.BandModel)
    n = int.from_bytes(raw[off:off + 4], "little")
    return json.loads(raw[off + 4: off + 4 + n].decode() or "{}")


# ---------------------------------------------------------------------------
# frames
# ---------------------------------------------------------------------------
def crown_config(spacing: float = 0.005) -> "pms.Config":
    fd, path = tempfile.mkstemp(suffix=".txt")
    with os.fdopen(fd, "w") as f:
        f.write(synth.config_text(**{"sim.particlespacing": spacing}))
    try:
        return pms.load_config(path)
    finally:
        os.unlink(path)


def plain_frame(ctx: "pms.Context", pos, vel=None, rho=None) -> None:
    ctx.upload(pos, vel, rho)
    ctx.build_grid()
    ctx.surface()


# ---------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------
def train(seeds=TRAIN_SEEDS, steps_per_frame: int = 60, batch: int = 8192, lr: float = 2e-3, pos_weight: float = 4.0,
          scale: float = 1.0, recall: float = 0.995, threshold_frames: int = 5, device: int = 0, seed: int = 1,
          log=print) -> tuple["pms.BandModel", dict]:
    """Trains the band MLP on crown frames and picks the logit threshold that
    keeps `recall` of the plain method's valid cubes on the last frames."""
    seeds = list(seeds)
    cfg = crown_config()
    trainer = pms.Trainer(device, seed)
    total = steps_per_frame * len(seeds)
    step = 0
    labels = 0
    hist = []
    t0 = time.time()
    with pms.Context(cfg, device) as ctx:
        keep = []
        for fi, s in enumerate(seeds):
            pos, vel, rho = synth.crown_variant(s, scale=scale)
            plain_frame(ctx, pos, vel, rho)
            nc, nvalid = ctx.learn_prepare()
            labels += nc
            losses = []
            for k in range(steps_per_frame):
                lr_k = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(total, 1)))
                losses.append(trainer.step(ctx, batch, (s << 20) + k, lr_k, pos_weight))
                step += 1
            hist.append(float(np.mean(losses)))
            log(f"frame {fi + 1}/{len(seeds)} seed {s}: {len(pos)} particles, {nc} candidates, {nvalid} valid cubes, "
                f"loss {hist[-1]:.4f} ({time.time() - t0:.0f} s)")
            if fi >= len(seeds) - threshold_frames:
                keep.append(s)
        # threshold: the (1 - recall) quantile of the positives' logits on the last frames
        model = trainer.model(0.0)
        ctx.set_band_model(model)
        pos_logits = []
        for s in keep:
            pos, vel, rho = synth.crown_variant(s, scale=scale)
            plain_frame(ctx, pos, vel, rho)
            ctx.learn_prepare()
            c = ctx.learn_candidates(logits=True)
            pos_logits.append(c["logit"][c["label"] == 1])
        pl = np.concatenate(pos_logits) if pos_logits else np.zeros(1, np.float32)
        thr = float(np.quantile(pl, 1.0 - recall)) if len(pl) else 0.0
    model.threshold = thr
    meta = {"seeds": [seeds[0], seeds[-1]], "frames": len(seeds), "labels": int(labels), "steps": step, "batch": batch,
            "lr": lr, "pos_weight": pos_weight, "recall_target": recall, "threshold": thr, "scale": scale,
            "loss_first": hist[0] if hist else None, "loss_last": hist[-1] if hist else None,
            "seconds": time.time() - t0}
    trainer.close()
    return model, meta


# ---------------------------------------------------------------------------
# evaluation and the judge
# ---------------------------------------------------------------------------
def cube_vertex_ranges(ctx: "pms.Context"):
    """Valid cubes (origin ids, ascending) and the mesh vertex range of each."""
    band = ctx.debug("band_list")
    nvert = ctx.debug("cube_nvert").astype(np.int64)
    off = np.concatenate([[0], np.cumsum(nvert)])
    sel = nvert > 0
    return band[sel], off[:-1][sel], nvert[sel]


def _soup_vertices(mesh: np.ndarray, starts, counts) -> np.ndarray:
    if len(starts) == 0:
        return np.zeros((0, 3), np.float32)
    counts = np.asarray(counts, np.int64)
    first = np.repeat(np.asarray(starts, np.int64), counts)
    within = np.arange(int(counts.sum())) - np.repeat(np.cumsum(counts) - counts, counts)
    return mesh[first + within]


def hausdorff(mesh_a: np.ndarray, cubes_a, mesh_b: np.ndarray, cubes_b) -> dict:
    """Symmetric vertex Hausdorff distance between two triangle soups made by
    the same per-cube triangulation of the same field: triangles of a cube in
    both sets are identical, so only cubes in one set alone contribute; their
    vertices are matched to the nearest vertex of the other soup."""
    from scipy.spatial import cKDTree  # host-side judge only
    ids_a, sa, ca = cubes_a
    ids_b, sb, cb = cubes_b
    only_a = ~np.isin(ids_a, ids_b)
    only_b = ~np.isin(ids_b, ids_a)
    out = {"cubes_only_plain": int(only_a.sum()), "cubes_only_learned": int(only_b.sum()), "a_to_b": 0.0, "b_to_a": 0.0}
    qa = _soup_vertices(mesh_a, sa[only_a], ca[only_a])
    qb = _soup_vertices(mesh_b, sb[only_b], cb[only_b])
    if len(qa):
        out["a_to_b"] = float(cKDTree(mesh_b).query(qa)[0].max()) if len(mesh_b) else float("inf")
    if len(qb):
        out["b_to_a"] = float(cKDTree(mesh_a).query(qb)[0].max()) if len(mesh_a) else float("inf")
    out["hausdorff"] = max(out["a_to_b"], out["b_to_a"])
    return out


def band_stats(c: "pms.Counts") -> dict:
    """Work of a learned or certified band: full field walks (exact values) and
    sign certificates (walks stopped above iso)."""
    return {"band_vertices": c.n_band_vertices, "valid_cubes": c.n_valid_cubes, "triangles": c.n_mesh_vertices // 3,
            "candidates": c.n_band_candidates, "predicted": c.n_band_predicted, "exact_first": c.n_band_exact,
            "certified": c.n_band_certified, "rechecked": c.n_band_rechecked,
            "full_walks": c.n_band_vertices - c.n_band_certified + c.n_band_rechecked}


def compare(ctx: "pms.Context", model: "pms.BandModel", h: float, pos, vel=None, rho=None,
            mode: str = "learned") -> dict:
    """Plain and learned (or certified) surface of one frame on one context:
    counts, stage times, whether the two triangle soups are identical, triangle
    delta and Hausdorff distance (also in units of h)."""
    if model is not None:
        ctx.set_band_model(model)
    plain_frame(ctx, pos, vel, rho)
    tp = ctx.stage_times()
    cp = ctx.counts()
    mesh_p, _ = ctx.mesh(normals=False)
    cubes_p = cube_vertex_ranges(ctx)
    ctx.set_band_mode(mode)
    try:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface_learned()
    finally:
        ctx.set_band_mode("plain")
    tl = ctx.stage_times()
    cl = ctx.counts()
    mesh_l, _ = ctx.mesh(normals=False)
    cubes_l = cube_vertex_ranges(ctx)
    hd = hausdorff(mesh_p, cubes_p, mesh_l, cubes_l)
    res = {"particles": int(len(pos)), "plain": {"band_vertices": cp.n_band_vertices, "valid_cubes": cp.n_valid_cubes,
                                                 "triangles": cp.n_mesh_vertices // 3, "ms": tp},
           "learned": dict(band_stats(cl), ms=tl), "mode": mode,
           "identical": bool(mesh_p.shape == mesh_l.shape and np.array_equal(mesh_p, mesh_l)),
           "triangle_delta": int(cl.n_mesh_vertices // 3) - int(cp.n_mesh_vertices // 3)}
    res.update(hd)
    res["hausdorff_h"] = hd["hausdorff"] / h
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--frames", type=int, default=50)
    t.add_argument("--steps", type=int, default=60)
    t.add_argument("--batch", type=int, default=8192)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--pos-weight", type=float, default=4.0)
    t.add_argument("--recall", type=float, default=0.995)
    t.add_argument("--scale", type=float, default=1.0)
    e = sub.add_parser("eval")
    e.add_argument("--model", default=DEFAULT_MODEL)
    e.add_argument("--frames", type=int, default=10)
    e.add_argument("--scale", type=float, default=1.0)
    e.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    if a.cmd == "train":
        seeds = list(TRAIN_SEEDS)[: a.frames]
        model, meta = train(seeds, a.steps, a.batch, a.lr, a.pos_weight, a.scale, a.recall)
        save_model(a.out, model, meta)
        print(json.dumps(meta))
        return 0
    model = load_model(a.model)
    cfg = crown_config()
    h = float(pms.derive_params(cfg).h)
    rows = []
    with pms.Context(cfg, 0) as ctx:
        for s in list(HELD_OUT_SEEDS)[: a.frames]:
            pos, vel, rho = synth.crown_variant(s, scale=a.scale)
            r = compare(ctx, model, h, pos, vel, rho)
            r["seed"] = s
            rows.append(r)
            print(json.dumps(r))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rows, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
