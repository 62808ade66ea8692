"""Batched frames in one CUDA graph (GPU): every frame of a batch gives the
same counts and the same triangle soup, bit for bit, as the frame run alone;
the graph is captured once and relaunched while the frames' grids stay the
same and captured again when they change; the learned band in a batch equals
the learned band frame by frame.  Also the pipelined output: a mesh streamed
to pinned host memory during the later stages equals the downloaded one."""
from __future__ import annotations

import numpy as np
import pytest


def _frames(k, spacing=0.02):
    from postmps_gb300 import synth
    # smaller tank and coarser spacing: a few 10k particles per frame
    return [synth.sloshing_tank(f, n_frames=k, spacing=spacing, length=1.0, width=0.4, depth_min=0.05, depth_max=0.4)
            for f in range(k)]


def _ctx(pms, spacing, diffuse=False):
    from postmps_gb300 import synth
    import os
    import tempfile
    fd, path = tempfile.mkstemp(suffix=".txt")
    with os.fdopen(fd, "w") as f:
        f.write(synth.config_text(**{"sim.particlespacing": spacing,
                                     "config.isdiffusegeneration": "true" if diffuse else "false"}))
    cfg = pms.load_config(path)
    os.unlink(path)
    return pms.Context(cfg, 0)


def _single(ctx, fr, learned=False):
    ctx.upload(*fr)
    ctx.build_grid()
    if learned:
        ctx.surface_learned()
    else:
        ctx.surface()
    return ctx.counts(), ctx.mesh(normals=False)[0]


@pytest.mark.gpu
def test_batch_equals_single_frames(pms_lib):
    pms = pms_lib
    frames = _frames(5)
    frames.insert(2, (np.zeros((0, 3), np.float32), None, None))     # an empty frame in the middle
    with _ctx(pms, 0.02) as ctx:
        ctx.run_batch(frames)
        got = [(ctx.batch_frame(f), ctx.batch_mesh(f)) for f in range(len(frames))]
        info = ctx.batch_info()
        assert info["captures"] == 1 and info["graph_kernels"] > 10 * len(frames)
        # the same frames again: the graph is relaunched, not captured again
        ctx.run_batch(frames)
        assert ctx.batch_info()["captures"] == 1
        assert np.array_equal(ctx.batch_mesh(1), got[1][1])
        for f, fr in enumerate(frames):
            (cb, ms), mb = got[f]
            if len(fr[0]) == 0:
                assert cb.n_particles == 0 and len(mb) == 0
                continue
            cs, ms_ = _single(ctx, fr)
            assert (cb.n_surface_particles, cb.n_band_vertices, cb.n_valid_cubes, cb.n_mesh_vertices) == \
                   (cs.n_surface_particles, cs.n_band_vertices, cs.n_valid_cubes, cs.n_mesh_vertices)
            assert np.array_equal(mb, ms_), f
            assert ms > 0.0
        # changed frames (and buffers the single runs may have regrown): captured again
        moved = [(fr[0] + np.float32(0.013), fr[1], fr[2]) if len(fr[0]) else fr for fr in frames]
        ctx.run_batch(moved)
        assert ctx.batch_info()["captures"] == 2
        cs, ms_ = _single(ctx, moved[0])
        assert np.array_equal(ctx.batch_mesh(0), ms_)


@pytest.mark.gpu
def test_learned_batch_equals_learned_single_frames(pms_lib):
    pms = pms_lib
    frames = _frames(4)
    with _ctx(pms, 0.02) as ctx:
        # a quickly trained model on the first frame is enough: the certification makes results exact
        ctx.upload(*frames[0])
        ctx.build_grid()
        ctx.surface()
        ctx.learn_prepare()
        t = pms.Trainer(0, 9)
        for k in range(60):
            t.step(ctx, 4096, k, 3e-3, 4.0)
        ctx.set_band_model(t.model(0.0))
        ctx.run_batch(frames, learned=True)
        got = [ctx.batch_mesh(f) for f in range(len(frames))]
        cert = [ctx.batch_frame(f)[0] for f in range(len(frames))]
        for f, fr in enumerate(frames):
            cs, ms_ = _single(ctx, fr, learned=True)
            assert np.array_equal(got[f], ms_), f
            assert (cert[f].n_band_exact, cert[f].n_band_certified, cert[f].n_band_rechecked) == \
                   (cs.n_band_exact, cs.n_band_certified, cs.n_band_rechecked), f
            # ... and equals the plain band's soup
            cp, mp = _single(ctx, fr, learned=False)
            assert np.array_equal(got[f], mp), f
        t.close()


@pytest.mark.gpu
def test_autotune_keeps_results_and_shapes_agree(pms_lib):
    """Every launch shape gives the same field; tuning leaves the frame's results as they were."""
    pms = pms_lib
    frames = _frames(2)
    with _ctx(pms, 0.02) as ctx:
        ctx.upload(*frames[1])
        ctx.build_grid()
        ctx.surface()
        ref_field = ctx.debug("field").copy()
        ref_counts = ctx.counts().as_dict()
        ref_mesh = ctx.mesh(normals=False)[0]
        t = ctx.autotune()
        assert t["field_threads"] in (64, 128, 256) and t["field_waves"] in (1, 2, 4, 8) and t["field_vpt"] in (1, 2, 4)
        assert t["density_threads"] in (64, 128, 256) and t["moments_threads"] in (64, 128, 256)
        assert t["field_ms"] > 0 and t["anisotropy_ms"] > 0
        assert np.array_equal(ctx.debug("field"), ref_field)
        assert ctx.counts().as_dict() == ref_counts
        for shape in ({"field_threads": 64, "field_waves": 1, "density_threads": 256, "moments_threads": 64, "field_vpt": 1},
                      {"field_threads": 256, "field_waves": 8, "density_threads": 64, "moments_threads": 256, "field_vpt": 4},
                      {"field_threads": 128, "field_waves": 2, "density_threads": 128, "moments_threads": 128, "field_vpt": 2}):
            ctx.set_tune(shape)
            cs, mesh = _single(ctx, frames[1])
            assert np.array_equal(mesh, ref_mesh)
            assert np.array_equal(ctx.debug("field"), ref_field), shape
        with pytest.raises(pms.PmsError):
            ctx.set_tune({"field_threads": 96, "field_waves": 1, "density_threads": 64, "moments_threads": 64})


@pytest.mark.gpu
def test_normals_on_demand_equal_streamed_normals(pms_lib):
    """Without a streamed normal buffer the marching cubes write positions only;
    the first download that asks for normals runs the emission again with them.
    Positions before and after, and the normals, equal those of a frame whose
    streamed mesh carried normals."""
    import torch
    pms = pms_lib
    frames = _frames(2)
    with _ctx(pms, 0.02) as ctx:
        buf = torch.empty(3 * 2_000_000, dtype=torch.float32).pin_memory()
        nrm = torch.empty(3 * 2_000_000, dtype=torch.float32).pin_memory()
        ref = []
        ctx.stream_mesh_to_host(buf.data_ptr(), nrm.data_ptr(), buf.numel() // 3)
        for fr in frames:
            ctx.upload(*fr)
            ctx.run_frame()
            n = ctx.wait_mesh()
            ref.append((buf.numpy()[: 3 * n].reshape(-1, 3).copy(), nrm.numpy()[: 3 * n].reshape(-1, 3).copy()))
        ctx.stream_mesh_to_host(0, None, 0)
        for fr, (pos_s, nrm_s) in zip(frames, ref):
            ctx.upload(*fr)
            ctx.run_frame()
            pos_only, _ = ctx.mesh(normals=False)
            pos, nrm_d = ctx.mesh(normals=True)
            assert np.array_equal(pos_only, pos_s)
            assert np.array_equal(pos, pos_s)
            assert np.array_equal(nrm_d, nrm_s)


@pytest.mark.gpu
@pytest.mark.parametrize("diffuse", [False, True])
def test_streamed_mesh_equals_download(pms_lib, diffuse):
    """pms_stream_mesh_to_host: the soup that reaches pinned host memory -- copied
    in vertex ranges on the copy stream while the emission continues and, with
    diffuse generation on, while the diffuse stage runs -- equals
    pms_download_mesh's, frame after frame; a buffer that is too small reports
    the count with PMS_ERR_CAPACITY."""
    import torch
    pms = pms_lib
    frames = _frames(3)
    with _ctx(pms, 0.02, diffuse) as ctx:
        buf = torch.empty(3 * 2_000_000, dtype=torch.float32).pin_memory()
        nrm = torch.empty(3 * 2_000_000, dtype=torch.float32).pin_memory()
        ctx.stream_mesh_to_host(buf.data_ptr(), nrm.data_ptr(), buf.numel() // 3)
        for fr in frames:
            ctx.upload(*fr)
            ctx.run_frame()
            n = ctx.wait_mesh()
            pos_ref, nrm_ref = ctx.mesh(normals=True)
            assert n == len(pos_ref) > 0
            assert np.array_equal(buf.numpy()[: 3 * n].reshape(-1, 3), pos_ref)
            assert np.array_equal(nrm.numpy()[: 3 * n].reshape(-1, 3), nrm_ref)
        small = torch.empty(30, dtype=torch.float32).pin_memory()
        ctx.stream_mesh_to_host(small.data_ptr(), None, 10)
        ctx.upload(*frames[0])
        ctx.run_frame()
        with pytest.raises(pms.PmsError):
            ctx.wait_mesh()
        ctx.stream_mesh_to_host(0, None, 0)
        with pytest.raises(pms.PmsError):
            ctx.wait_mesh()


@pytest.mark.gpu
def test_batch_with_diffuse_equals_single_frames(pms_lib, tmp_config):
    """Diffuse generation inside the batch graph: consecutive crown frames (one of them
    smaller) batched give, frame by frame, the live diffuse particles, counts and meshes
    of running them one by one, and leave the context where the single frames leave
    theirs -- a single frame after the batch, and a second batch (the graph relaunched),
    continue the same sequence."""
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.crown_splash(n_slab=(60, 60, 12), n_ring=40000, radius=0.09)
    small = synth.crown_splash(n_slab=(40, 40, 10), n_ring=20000, radius=0.07, seed=9)

    def frame(i):
        if i == 2:
            return small
        return ((pos + np.float32(0.004 * i) * vel).astype(np.float32), vel, rho)

    cfg = pms.load_config(tmp_config(synth.config_text(**synth.CROWN_KEYS, **{"config.isdiffusegeneration": "true"})))
    with pms.Context(cfg, 0) as single, pms.Context(cfg, 0) as batch:
        def run_single(i):
            single.upload(*frame(i))
            single.run_frame()
            live = single.diffuse_particles(-1)
            return live, single.counts().as_dict(), single.mesh(normals=False)[0].copy()

        def check_batch(idx):
            batch.run_batch([frame(i) for i in idx])
            for f, i in enumerate(idx):
                live, c, mesh = run_single(i)
                got = batch.batch_diffuse(f)
                assert len(got) == len(live["pos"]), (i, len(got), len(live["pos"]))
                np.testing.assert_array_equal(got["pos"], live["pos"])
                np.testing.assert_array_equal(got["vel"], live["vel"])
                np.testing.assert_array_equal(got["ttl"], live["ttl"])
                np.testing.assert_array_equal(got["type"], live["type"])
                bc = batch.batch_frame(f)[0].as_dict()
                for key in ("n_generated_diffuse", "n_spawning", "n_diffuse", "n_spray", "n_foam", "n_bubble",
                            "n_free_surface", "n_mesh_vertices"):
                    assert bc[key] == c[key], (i, key, bc[key], c[key])
                np.testing.assert_array_equal(batch.batch_mesh(f), mesh)

        check_batch([0, 1, 2, 3, 4])
        assert batch.batch_frame(4)[0].as_dict()["n_diffuse"] > 0
        # one frame alone on the batched context continues the sequence
        batch.upload(*frame(5))
        batch.run_frame()
        live, _, _ = run_single(5)
        np.testing.assert_array_equal(batch.diffuse_particles(-1)["pos"], live["pos"])
        # a second batch (other grids: captured again) continues it, and the same frames
        # once more relaunch that graph from the carried particles the context now holds
        check_batch([6, 7, 8, 9, 10])
        caps = batch.batch_info()["captures"]
        check_batch([6, 7, 8, 9, 10])
        assert batch.batch_info()["captures"] == caps


@pytest.mark.gpu
def test_batch_meshes_streamed_inside_the_graph(pms_lib):
    """pms_batch_stream_meshes: with a host arena registered, every frame's soup
    lands there inside the graph at its pms_batch_mesh_range offset, equal to
    pms_batch_mesh's; registering captures the graph again; an arena too small
    for the batch reports PMS_ERR_CAPACITY; unregistering returns to downloads."""
    import torch
    pms = pms_lib
    frames = _frames(5)
    frames.insert(2, (np.zeros((0, 3), np.float32), None, None))
    with _ctx(pms, 0.02) as ctx:
        ctx.run_batch(frames)
        ref = [ctx.batch_mesh(f) for f in range(len(frames))]
        total = sum(len(m) for m in ref)
        arena = torch.empty(3 * (total + 1000), dtype=torch.float32).pin_memory()
        ctx.batch_stream_meshes(arena.data_ptr(), total + 1000)
        caps = ctx.batch_info()["captures"]
        for rep in range(2):
            arena.zero_()
            ctx.run_batch(frames)
            assert ctx.batch_info()["captures"] == caps + 1      # captured once for the registration
            host = arena.numpy().reshape(-1, 3)
            for f in range(len(frames)):
                first, n = ctx.batch_mesh_range(f)
                assert n == len(ref[f])
                assert np.array_equal(host[first:first + n], ref[f]), (rep, f)
        small = torch.empty(3 * (total // 2), dtype=torch.float32).pin_memory()
        ctx.batch_stream_meshes(small.data_ptr(), total // 2)
        with pytest.raises(pms.PmsError) as ei:
            ctx.run_batch(frames)
        assert ei.value.status == 4
        ctx.batch_stream_meshes(0, 0)
        ctx.run_batch(frames)
        assert np.array_equal(ctx.batch_mesh(3), ref[3])
