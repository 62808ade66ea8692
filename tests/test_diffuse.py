"""Diffuse (spray/foam/bubble) particles.

CPU: the oracle is pinned to fixtures made by the reference's own diffuse
kernels (tests/golden/make_golden.py, two frames, spawn uniforms injected):
  free-surface list                exact
  spawn counts from the reference's clamped potentials      exact
  spawned particles (position, TTL, type) from its counts   exact; velocity 1e-5
  advection of the previous frame's particles               exact
  clamped potentials (float64 vs its float32)               1e-3 absolute
GPU (through the C ABI), same frames:
  free-surface count                exact
  spawn counts from the GPU's own clamped potentials        exact (oracle)
  spawned particles from the GPU's counts                   exact position/TTL/type, velocity 1e-5
  advected particles from the GPU's previous live set       exact
  potentials vs the reference fixtures                      1e-3 absolute
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN

GPATH = os.path.join(GOLDEN, "diffuse_block14.npz")


def golden():
    z = np.load(GPATH)
    d = {k: z[k] for k in z.files}
    d["config"] = str(d["config"])
    return d


def sorted_frame(oracle, p, pos):
    g = oracle.grid_from_positions(p, pos)
    keys, perm, sk, start, end = oracle.hash_sort(p, g, pos)
    surf, scan, slist = oracle.surface_particles(g, start, end)
    return g, perm, start, end, slist


@pytest.mark.parametrize("frame", [0, 1])
def test_diffuse_oracle_matches_reference(oracle, frame):
    d = golden()
    p = oracle.derive_params(oracle.config_from_keys(oracle.parse_ini(d["config"])))
    pos, vel = d[f"f{frame}_pos"], d[f"f{frame}_vel"]
    g, perm, start, end, slist = sorted_frame(oracle, p, pos)
    np.testing.assert_array_equal(perm, d[f"f{frame}_perm"])
    np.testing.assert_array_equal(slist, d[f"f{frame}_free_list"])
    spos, svel = pos[perm], vel[perm]
    res = oracle.diffuse_frame(p, g, spos, svel, start, end, slist, np.zeros_like(spos, np.float64),
                               int(d["seed"]), frame, old=d[f"f{frame}_old_in"], nrm_for_crests=d[f"f{frame}_nrm"],
                               pot_clamped=d[f"f{frame}_pot"])
    np.testing.assert_array_equal(res["num"], d[f"f{frame}_num"])
    gen, rgen = res["gen"], d[f"f{frame}_gen"]
    assert gen.shape == rgen.shape
    np.testing.assert_array_equal(gen[:, [0, 1, 2, 6, 7]], rgen[:, [0, 1, 2, 6, 7]])
    assert float(np.abs(gen[:, 3:6] - rgen[:, 3:6]).max(initial=0)) <= 1e-5 * max(1.0, float(np.abs(rgen[:, 3:6]).max(initial=0)))
    np.testing.assert_array_equal(res["old_after"], d[f"f{frame}_old_after"])
    # float64 potentials against the reference's float32 ones (clamped to [0, 1])
    assert float(np.abs(res["pot"] - d[f"f{frame}_pot"]).max()) < 1e-3


def run_gpu_frames(pms, tmp_config, d, frames=(0, 1)):
    cfg = pms.load_config(tmp_config(d["config"]))
    cfg.rng_seed = int(d["seed"])
    out = []
    with pms.Context(cfg, 0) as ctx:
        for fr in frames:
            ctx.upload(d[f"f{fr}_pos"], d[f"f{fr}_vel"], d[f"f{fr}_rho"])
            ctx.run_frame()
            c = ctx.counts().as_dict()
            r = {"counts": c, "pot": ctx.debug("diffuse_potential"), "num": ctx.debug("diffuse_count"),
                 "nrm": ctx.debug("free_normal"), "perm": ctx.debug("perm"), "live": ctx.diffuse_particles(-1),
                 "launches": ctx.launches}
            out.append(r)
    return out


def live_records(live: dict) -> np.ndarray:
    return np.concatenate([live["pos"], live["vel"], live["ttl"][:, None].astype(np.float32),
                           live["type"][:, None].astype(np.float32)], 1)


@pytest.mark.gpu
def test_diffuse_gpu_two_frames(pms_lib, oracle, tmp_config):
    d = golden()
    gpu = run_gpu_frames(pms_lib, tmp_config, d)
    check_gpu_frames(oracle, d, gpu, reference=True)


@pytest.mark.gpu
def test_diffuse_gpu_crown_spawns(pms_lib, oracle, tmp_config):
    """A small crown splash (83,200 particles, a 40k-particle ring) with the crown
    workload's diffuse keys: the ring spawns spray, foam and bubbles, and two
    frames of the GPU chain match the oracle (counts exact from the GPU's clamped
    potentials, spawned and advected particles exact, velocities 1e-5)."""
    from postmps_gb300 import synth
    pos, vel, rho = synth.crown_splash(n_slab=(60, 60, 12), n_ring=40000, radius=0.09)
    dt = 0.004
    d = {"config": synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"}), "seed": 7,
         "f0_pos": pos, "f0_vel": vel, "f0_rho": rho,
         "f1_pos": (pos + dt * vel).astype(np.float32), "f1_vel": vel, "f1_rho": rho}
    gpu = run_gpu_frames(pms_lib, tmp_config, d)
    assert gpu[0]["counts"]["n_generated_diffuse"] > 1000, gpu[0]["counts"]
    assert min(gpu[1]["counts"][k] for k in ("n_spray", "n_foam", "n_bubble")) > 0, gpu[1]["counts"]
    check_gpu_frames(oracle, d, gpu, reference=False)


def check_gpu_frames(oracle, d, gpu, reference: bool):
    p = oracle.derive_params(oracle.config_from_keys(oracle.parse_ini(d["config"])))
    prev_live = np.zeros((0, 8), np.float32)
    for fr, r in enumerate(gpu):
        pos, vel = d[f"f{fr}_pos"], d[f"f{fr}_vel"]
        g, perm, start, end, slist = sorted_frame(oracle, p, pos)
        np.testing.assert_array_equal(r["perm"], perm)
        assert r["counts"]["n_free_surface"] == len(slist)
        if reference:
            assert len(slist) == len(d[f"f{fr}_free_list"])
            # potentials against the reference (float32 vs float32, different summation order)
            # where they are used: a particle whose clamped kinetic energy is 0 spawns
            # nothing, and its trapped-air and wave-crest walks are skipped (left 0)
            ref_pot = d[f"f{fr}_pot"]
            assert float(np.abs(r["pot"][:, 2] - ref_pot[:, 2]).max(initial=0)) < 1e-5
            moving = (r["pot"][:, 2] > 0) & (ref_pot[:, 2] > 0)
            assert float(np.abs(r["pot"][moving] - ref_pot[moving]).max(initial=0)) < 1e-3
            assert not r["pot"][r["pot"][:, 2] == 0][:, :2].any()
        # counts: exact from the GPU's own clamped potentials
        spos, svel = pos[perm], vel[perm]
        res = oracle.diffuse_frame(p, g, spos, svel, start, end, slist, np.zeros_like(spos, np.float64),
                                   int(d["seed"]), fr, old=prev_live, nrm_for_crests=r["nrm"], pot_clamped=r["pot"])
        np.testing.assert_array_equal(r["num"], res["num"])
        if reference:
            assert np.mean(r["num"] == d[f"f{fr}_num"]) > 0.99
        assert r["counts"]["n_generated_diffuse"] == int(np.clip(res["num"], 0, None).sum())
        # live particles: generated (from the GPU's counts) then advected old ones, type 3 dropped
        live = live_records(r["live"])
        want = res["live"]
        assert live.shape == want.shape, (live.shape, want.shape)
        np.testing.assert_array_equal(live[:, [0, 1, 2, 6, 7]], want[:, [0, 1, 2, 6, 7]])
        assert float(np.abs(live[:, 3:6] - want[:, 3:6]).max(initial=0)) <= 1e-5 * max(1.0, float(np.abs(want[:, 3:6]).max(initial=0)))
        assert r["counts"]["n_diffuse"] == len(live)
        t = want[:, 7].astype(int)
        assert (r["counts"]["n_spray"], r["counts"]["n_foam"], r["counts"]["n_bubble"]) == \
            (int((t == 0).sum()), int((t == 1).sum()), int((t == 2).sum()))
        prev_live = live


@pytest.mark.gpu
def test_diffuse_files_written(pms_lib, tmp_path):
    from postmps_gb300 import synth
    d = golden()
    frames = tmp_path / "frames"
    frames.mkdir()
    for fr in (0, 1):
        pms_lib.write_vtk(str(frames / f"PartFluid_{fr:04d}.vtk"), d[f"f{fr}_pos"], d[f"f{fr}_vel"], d[f"f{fr}_rho"])
    text = synth.config_text(**{"config.isdiffusegeneration": "true", "config.framefrom": 0, "config.frameto": 1,
                                "config.fluidpath": str(frames), "config.surfacepath": str(tmp_path),
                                "config.diffusepath": str(tmp_path), "config.surfaceprefix": "PartSurface_"})
    cfg = tmp_path / "config.txt"
    cfg.write_text(text)
    pms_lib.run_config(str(cfg))
    for fr in (0, 1):
        assert (tmp_path / f"PartSurface_{fr:04d}.ply").exists()
        for pre in ("PartSpary_", "PartFoam_", "PartBubble_"):
            p = tmp_path / f"{pre}{fr:04d}.vtk"
            assert p.exists()
            pos, vel, _ = pms_lib.read_vtk(str(p))
            assert pos.shape[1] == 3


@pytest.mark.gpu
def test_streamed_diffuse_particles_equal_downloaded(pms_lib, tmp_config):
    """pms_stream_diffuse_to_host: each frame's live set lands in the registered
    host buffer, record for record what pms_download_diffuse returns, and the
    next frame (whose update moves those particles) waits for the copy."""
    import ctypes as C
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.crown_splash(n_slab=(60, 60, 12), n_ring=40000, radius=0.09)
    cfg = pms.load_config(tmp_config(synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"})))
    cap = 1 << 18
    buf = (C.c_uint8 * (32 * cap))()
    rec = np.frombuffer(buf, dtype=np.dtype([("pos", np.float32, 3), ("ttl", np.int32), ("vel", np.float32, 3),
                                             ("type", np.int32)]))
    with pms.Context(cfg, 0) as ctx:
        ctx.stream_diffuse_to_host(C.addressof(buf), cap)
        for fr in range(3):
            p = (pos + np.float32(0.004 * fr) * vel).astype(np.float32)
            ctx.upload(p, vel, rho)
            ctx.run_frame()
            n = ctx.wait_diffuse()
            live = ctx.diffuse_particles(-1)
            assert n == len(live["pos"]) > 0
            np.testing.assert_array_equal(rec["pos"][:n], live["pos"])
            np.testing.assert_array_equal(rec["vel"][:n], live["vel"])
            np.testing.assert_array_equal(rec["ttl"][:n], live["ttl"])
            np.testing.assert_array_equal(rec["type"][:n], live["type"])
        # a reset starts the sequence again: the first frame's live set comes back
        ctx.reset_diffuse()
        first = []
        for fr in range(2):
            ctx.upload((pos + np.float32(0.004 * fr) * vel).astype(np.float32), vel, rho)
            ctx.run_frame()
            first.append(rec[: ctx.wait_diffuse()].copy())
        with pms.Context(cfg, 0) as fresh:
            for fr in range(2):
                fresh.upload((pos + np.float32(0.004 * fr) * vel).astype(np.float32), vel, rho)
                fresh.run_frame()
                live = fresh.diffuse_particles(-1)
                np.testing.assert_array_equal(first[fr]["pos"], live["pos"])
                np.testing.assert_array_equal(first[fr]["ttl"], live["ttl"])
        # too small a buffer: the count comes back with PMS_ERR_CAPACITY
        ctx.stream_diffuse_to_host(C.addressof(buf), 1)
        ctx.upload(pos, vel, rho)
        ctx.run_frame()
        with pytest.raises(pms.PmsError) as ei:
            ctx.wait_diffuse()
        assert ei.value.status == 4
        ctx.stream_diffuse_to_host(0, 0)


@pytest.mark.gpu
def test_frames_in_flight_equal_waited_frames(pms_lib, tmp_config):
    """Streamed outputs with frames in flight: alternating two host buffer sets,
    frame k+1 runs before frame k's mesh and diffuse particles are waited for,
    and each wait returns the oldest frame's results, equal to those of a
    context that waits after every frame.  One buffer set with two frames
    unwaited keeps only the newest."""
    import ctypes as C
    import torch
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.crown_splash(n_slab=(60, 60, 12), n_ring=40000, radius=0.09)
    cfg = pms.load_config(tmp_config(synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"})))
    frames = [((pos + np.float32(0.004 * f) * vel).astype(np.float32), vel, rho) for f in range(4)]
    cap_v, cap_d = 8_000_000, 1 << 19
    mk = lambda: (torch.empty(3 * cap_v, dtype=torch.float32).pin_memory(),
                  torch.empty(32 * cap_d, dtype=torch.uint8).pin_memory())
    sets = [mk(), mk()]

    def register(ctx, s):
        ctx.stream_mesh_to_host(s[0].data_ptr(), None, cap_v)
        ctx.stream_diffuse_to_host(s[1].data_ptr(), cap_d)

    def take(ctx, s):
        n, m = ctx.wait_mesh(), ctx.wait_diffuse()
        return s[0].numpy()[: 3 * n].copy(), s[1].numpy()[: 32 * m].copy()

    with pms.Context(cfg, 0) as ctx:
        register(ctx, sets[0])
        waited = []
        for fr in frames:
            ctx.upload(*fr)
            ctx.run_frame()
            waited.append(take(ctx, sets[0]))
    with pms.Context(cfg, 0) as ctx:
        got = []
        for k, fr in enumerate(frames):
            register(ctx, sets[k % 2])
            ctx.upload(*fr)
            ctx.run_frame()
            if k:
                got.append(take(ctx, sets[(k - 1) % 2]))
        got.append(take(ctx, sets[(len(frames) - 1) % 2]))
        with pytest.raises(pms.PmsError):
            ctx.wait_mesh()
        # one buffer set, two frames unwaited: the second replaces the first
        register(ctx, sets[0])
        for fr in frames[:2]:
            ctx.upload(*fr)
            ctx.run_frame()
        last = take(ctx, sets[0])
        with pytest.raises(pms.PmsError):
            ctx.wait_diffuse()
        ctx.stream_mesh_to_host(0, None, 0)
        ctx.stream_diffuse_to_host(0, 0)
    assert len(got) == len(waited)
    for (m0, d0), (m1, d1) in zip(waited, got):
        assert len(m0) > 0 and len(d0) > 0
        assert np.array_equal(m0, m1)
        assert np.array_equal(d0, d1)
    # the carried diffuse set grew over six frames in that context; the mesh is frame 1's
    assert np.array_equal(last[0], waited[1][0])


@pytest.mark.gpu
def test_overlapped_frame_equals_stage_by_stage(pms_lib, tmp_config):
    """pms_run_frame with surface and diffuse on runs the diffuse stage on a stream
    of its own beside the band, field and marching cubes; calling the stages one
    after the other on the context's stream (pms_build_grid, pms_surface,
    pms_diffuse) gives the same mesh and the same live diffuse particles, bit for
    bit, on a frame that carries particles from the frame before."""
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.crown_splash(n_slab=(60, 60, 12), n_ring=40000, radius=0.09)
    cfg = pms.load_config(tmp_config(synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"})))
    frames = [((pos + np.float32(0.004 * f) * vel).astype(np.float32), vel, rho) for f in range(2)]
    out = []
    for stepwise in (False, True):
        with pms.Context(cfg, 0) as ctx:
            ctx.upload(*frames[0])
            ctx.run_frame()
            ctx.upload(*frames[1])
            if stepwise:
                ctx.build_grid()
                ctx.surface()
                ctx.diffuse()
            else:
                ctx.run_frame()
            live = ctx.diffuse_particles(-1)
            out.append((ctx.mesh(normals=False)[0], live))
    (m0, d0), (m1, d1) = out
    assert len(m0) > 0 and len(d0["pos"]) > 0
    assert np.array_equal(m0, m1)
    for k in ("pos", "vel", "ttl", "type"):
        np.testing.assert_array_equal(d0[k], d1[k])


@pytest.mark.gpu
def test_overlapped_empty_and_single_particle_frames(pms_lib, tmp_config):
    """Empty and one-particle frames through the overlapped frame (surface and
    diffuse on) with both outputs streamed and frames in flight, then a real frame:
    nothing hangs or errors, the empty frame's mesh record comes back with 0 vertices
    and the real frame's outputs are those of a fresh context."""
    import torch
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.crown_splash(n_slab=(40, 40, 10), n_ring=20000, radius=0.07)
    cfg = pms.load_config(tmp_config(synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"})))
    mesh = [torch.empty(3 * 4_000_000, dtype=torch.float32).pin_memory() for _ in range(2)]
    dif = [torch.empty(32 * (1 << 18), dtype=torch.uint8).pin_memory() for _ in range(2)]
    with pms.Context(cfg, 0) as ctx:
        seq = [(np.zeros((0, 3), np.float32), None, None), (np.array([[0.1, 0.2, 0.3]], np.float32), None, None)]
        ns = []
        for k, fr in enumerate(seq):
            ctx.stream_mesh_to_host(mesh[k % 2].data_ptr(), None, 4_000_000)
            ctx.stream_diffuse_to_host(dif[k % 2].data_ptr(), 1 << 18)
            ctx.upload(*fr)
            ctx.run_frame()
        ns.append(ctx.wait_mesh())
        ns.append(ctx.wait_mesh())
        assert ns[0] == 0 and ns[1] % 3 == 0
        ctx.reset_diffuse()
        ctx.stream_mesh_to_host(0, None, 0)
        ctx.stream_diffuse_to_host(0, 0)
        ctx.upload(pos, vel, rho)
        ctx.run_frame()
        m_after = ctx.mesh(normals=False)[0]
        d_after = ctx.diffuse_particles(-1)
    with pms.Context(cfg, 0) as fresh:
        fresh.upload(pos, vel, rho)
        fresh.run_frame()
        assert np.array_equal(m_after, fresh.mesh(normals=False)[0])
        np.testing.assert_array_equal(d_after["pos"], fresh.diffuse_particles(-1)["pos"])
