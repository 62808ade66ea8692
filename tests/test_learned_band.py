"""Learned narrow band.

CPU (oracle/learn_oracle.py, the checker): bf16 rounding, the oracle's own
gradient against finite differences, features / candidates / border check on
hand-made cases.

GPU (through the C ABI): the tensor-core backward pass against the oracle's
gradient, the forward pass and the feature extraction against the oracle on
a real frame, training lowering the loss, the border-check fallback
recovering the plain mesh from a crippled predictor, and the committed model
on a held-out frame: fewer field evaluations than the plain band at a
Hausdorff distance within 0.05 h of the plain mesh.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import learn_oracle as LO  # noqa: E402


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------
def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.0078125, 1.01171875, -2.5, 3.0e-39, 65504.0], np.float32)
    # 1 + 2^-8 ties to even (1.0); 1 + 3*2^-8 ties up to 1 + 2^-6
    got = LO.bf16_value(LO.bf16_bits(x))
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0078125 and got[3] == 1.015625
    assert got[4] == -2.5 and got[6] == 65536.0
    assert np.all(LO.bf16_round(got) == got)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    B = 64
    x = LO.bf16_round(rng.uniform(0, 2, (B, 64)).astype(np.float32))
    y = (rng.uniform(size=B) < 0.3).astype(np.float64)
    p = rng.normal(0, 0.2, LO.N_PARAMS)
    # bf16-exact parameters so that the forward pass is smooth in the probed directions
    p = LO.bf16_round(p.astype(np.float32)).astype(np.float64)
    loss, g = LO.loss_and_grad(p, x, y, 3.0)
    # probe biases exactly (no bf16 rounding on b1 / b2)
    for idx in [LO.OFF_B1 + 3, LO.OFF_B1 + 40, LO.OFF_B2]:
        e = 1e-4
        q1, q2 = p.copy(), p.copy()
        q1[idx] += e
        q2[idx] -= e
        fd = (LO.loss_and_grad(q1, x, y, 3.0)[0] - LO.loss_and_grad(q2, x, y, 3.0)[0]) / (2 * e)
        assert abs(fd - g[idx]) <= 1e-4 * max(1.0, abs(fd)), (idx, fd, g[idx])
    # W1 and w2 through a directional derivative with bf16 steps (the forward
    # pass rounds them): use the unrounded-dh gradient as the reference
    z, pre, h, w2q = LO.forward(p, x)
    pr = 1.0 / (1.0 + np.exp(-z))
    dz = (pr * (3.0 * y + 1 - y) - 3.0 * y) / B
    dh = np.where(pre > 0, dz[:, None] * w2q[None, :], 0.0)
    exact_w1 = (x.astype(np.float64).T @ dh).reshape(-1)
    assert np.allclose(g[: LO.OFF_B1], exact_w1, rtol=2e-2, atol=1e-3 * np.abs(exact_w1).max())


def test_features_and_candidates_small_grid():
    scres = (9, 9, 9)                       # 8 cubes per axis, coarse vertices 0..5 per axis
    sums = np.zeros((6, 6, 6), np.uint32)
    sums[2, 2, 2] = 3 << 20                 # density 3 * inv_expected at coarse vertex (2, 2, 2)
    inv = np.float32(0.5)
    # even cube (4,4,4): coarse cell 2, patch vertices 1..4: vertex 2 at d = 1
    f = LO.features(sums, scres, inv, [(4 * 9 + 4) * 9 + 4])[0]
    assert f[(1 * 4 + 1) * 4 + 1] == 1.5 and np.count_nonzero(f) == 1
    # odd cube (5,5,5): coarse cell 2, reflected patch 4, 3, 2, 1: vertex 2 at d = 2
    f = LO.features(sums, scres, inv, [(5 * 9 + 5) * 9 + 5])[0]
    assert f[(2 * 4 + 2) * 4 + 2] == 1.5 and np.count_nonzero(f) == 1
    # mixed parity (3,4,4): x reflected (vertices 3, 2, 1, 0: d = 1), y and z even (d = 1)
    f = LO.features(sums, scres, inv, [(4 * 9 + 4) * 9 + 3])[0]
    assert f[(1 * 4 + 1) * 4 + 1] == 1.5
    # every cell's patch holds vertex 2 and empty vertices: all 8^3 cubes are candidates
    assert len(LO.candidates(sums, scres, inv)) == 8 ** 3
    # uniformly full inside; vertices outside the grid read 0: only cells whose patch
    # leaves the grid (coarse cell 0 on some axis) stay mixed
    sums[:] = 2 << 20
    cand = LO.candidates(sums, scres, inv)
    assert len(cand) == 8 ** 3 - 6 ** 3
    assert (4 * 9 + 4) * 9 + 4 not in set(cand.tolist())


def test_density_splat_is_a_partition_of_unity():
    # a lattice at the coarse spacing, offset from the coarse vertices: interior vertices read exactly 1
    sc = 0.005
    g = np.arange(1, 9) * 2 * sc + 0.3 * sc
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    sums = LO.coarse_counts(pos, (0.0, 0.0, 0.0), sc, (24, 24, 24))
    d = LO.density(sums, np.float32(1.0))
    assert np.allclose(d[2:8, 2:8, 2:8], 1.0, atol=4e-6)
    assert d.sum() == pytest.approx(len(pos), rel=1e-5)


def test_border_queue_known_case():
    scres = (6, 6, 6)
    vs = set()
    # cube (1,1,1) fully evaluated, its +x face crossed (corners with x=1 inside)
    for k in range(8):
        vs.add(((1 + (k >> 2)) * 6 + 1 + ((k >> 1) & 1)) * 6 + 1 + (k & 1))
    cid = (1 * 6 + 1) * 6 + 1
    q = LO.border_queue([cid], [0xF0 | 0x01], vs, scres)
    # x = 1 face (mask 0xF0) fully inside: no crossing there; x = 0 face mixed (only bit 0)
    # y / z faces mixed as well
    assert (1 * 6 + 1) * 6 + 0 in q          # -x neighbour
    assert (1 * 6 + 1) * 6 + 2 not in q      # +x face not crossed
    assert len(q) == 5


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _crown_ctx(pms, scale, seed=100):
    from postmps_gb300 import learned, synth
    cfg = learned.crown_config()
    ctx = pms.Context(cfg, 0)
    pos, vel, rho = synth.crown_variant(seed, scale=scale)
    return ctx, cfg, pos, vel, rho


@pytest.mark.gpu
def test_backward_matches_oracle_gradient(pms_lib):
    pms = pms_lib
    rng = np.random.default_rng(7)
    B = 1000                                 # not a multiple of the 128-sample block
    x = LO.bf16_round(rng.uniform(0, 2, (B, 64)).astype(np.float32))
    y = (rng.uniform(size=B) < 0.25).astype(np.uint8)
    p = rng.normal(0, 0.15, LO.N_PARAMS).astype(np.float32)
    t = pms.Trainer(0, 5)
    t.set_params(p)
    g, loss = t.grad(LO.bf16_bits(x).reshape(B, 64), y, 4.0)
    lo, go = LO.loss_and_grad(p.astype(np.float64), x, y.astype(np.float64), 4.0)
    assert abs(loss - lo) <= 1e-4 * max(1.0, abs(lo))
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 5e-3, rel
    for sl in (slice(0, LO.OFF_B1), slice(LO.OFF_B1, LO.OFF_W2), slice(LO.OFF_W2, LO.OFF_B2)):
        r = np.linalg.norm(g[sl] - go[sl]) / max(np.linalg.norm(go[sl]), 1e-12)
        assert r < 1e-2, (sl, r)
    assert abs(g[LO.OFF_B2] - go[LO.OFF_B2]) <= 1e-4 * max(1e-3, abs(go[LO.OFF_B2]))
    t.close()


@pytest.mark.gpu
def test_forward_features_candidates_match_oracle(pms_lib):
    pms = pms_lib
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 0.02)
    with ctx:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface()
        nc, nvalid = ctx.learn_prepare()
        assert nc > 0 and nvalid > 0
        g = ctx.grid()
        prm = pms.derive_params(cfg)
        counts = LO.coarse_counts(ctx.debug("pos_sorted"), list(g.scmin_pos), g.sc_grid_size, list(g.scres))
        inv = LO.inv_expected(g.sc_grid_size, prm.particle_spacing)
        cand = LO.candidates(counts, list(g.scres), inv)
        got = ctx.learn_candidates(logits=False)
        assert np.array_equal(got["cube"], cand)
        # labels are the plain valid cubes
        band, nvert = ctx.debug("band_list"), ctx.debug("cube_nvert")
        valid = set(band[nvert > 0].tolist())
        assert np.array_equal(got["label"], np.array([c in valid for c in cand], np.uint8))
        # features bit-exact
        pick = cand[:: max(1, len(cand) // 3000)]
        xo = LO.features(counts, list(g.scres), inv, pick)
        xg = ctx.learn_features(pick)
        assert np.array_equal(xg, LO.bf16_bits(xo))
        # forward pass: logits of a random model
        rng = np.random.default_rng(11)
        p = rng.normal(0, 0.2, LO.N_PARAMS).astype(np.float32)
        t = pms.Trainer(0, 1)
        t.set_params(p)
        ctx.set_band_model(t.model(0.0))
        got = ctx.learn_candidates(logits=True)
        zo = LO.forward(p.astype(np.float64), LO.features(counts, list(g.scres), inv, got["cube"]))[0]
        assert np.allclose(got["logit"], zo, rtol=1e-4, atol=1e-4 * np.abs(zo).max())
        t.close()


@pytest.mark.gpu
def test_training_lowers_the_loss(pms_lib):
    pms = pms_lib
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 0.05)
    with ctx:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface()
        ctx.learn_prepare()
        t = pms.Trainer(0, 3)
        losses = [t.step(ctx, 4096, k, 3e-3, 4.0) for k in range(150)]
        assert np.mean(losses[-20:]) < 0.75 * np.mean(losses[:5]), (losses[:5], losses[-20:])
        t.close()


@pytest.mark.gpu
def test_border_check_recovers_the_plain_mesh(pms_lib):
    """A predictor that keeps only half of the crossed cubes: the border check
    must flood the rest of every surface it touches.  Only surface pieces
    with no predicted cube at all (small droplets) may stay missing."""
    pms = pms_lib
    from postmps_gb300 import learned
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 0.03)
    h = float(pms.derive_params(cfg).h)
    with ctx:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface()
        ctx.learn_prepare()
        t = pms.Trainer(0, 4)
        for k in range(200):
            t.step(ctx, 4096, 1000 + k, 3e-3, 4.0)
        ctx.set_band_model(t.model(0.0))
        c = ctx.learn_candidates(logits=True)
        pl = c["logit"][c["label"] == 1]
        thr = float(np.quantile(pl, 0.5))                    # keeps about half of the positives
        crippled = t.model(thr)
        r = learned.compare(ctx, crippled, h, pos, vel, rho)
        # plain valid cubes the predictor alone would miss
        missed = r["plain"]["valid_cubes"] - int(np.count_nonzero((c["label"] == 1) & (c["logit"] > thr)))
        assert r["learned"]["fallback_cubes"] > 0 and r["learned"]["fallback_rounds"] > 0
        assert missed > 0.3 * r["plain"]["valid_cubes"]
        assert r["cubes_only_plain"] <= 0.05 * missed, (r, missed)
        assert r["cubes_only_learned"] == 0, r
        t.close()


@pytest.mark.gpu
def test_held_out_frame_has_no_cube_outside_the_plain_band(pms_lib):
    """On a held-out frame the network predicts cubes whose corners the plain
    band does not hold (its truncation leaves a hole there); the plain-band
    membership test of the valid cubes' corners removes those corners, so
    the learned surface has no cube the plain one lacks."""
    pms = pms_lib
    from postmps_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model committed")
    model = learned.load_model()
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 1.0, seed=201)
    h = float(pms.derive_params(cfg).h)
    with ctx:
        r = learned.compare(ctx, model, h, pos, vel, rho)
    assert r["learned"]["removed"] > 0, r
    assert r["cubes_only_learned"] == 0, r
    assert r["hausdorff"] <= 0.05 * h, r


@pytest.mark.gpu
def test_tensor_core_wait_that_gives_up_reports_and_recovers(pms_lib):
    """The band network's wait on the tensor cores is bounded: made to give up at
    once, the frame reports the timeout (no fault, no hang), and with the bound
    restored the same context reconstructs the frame as before."""
    pms = pms_lib
    from postmps_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model committed")
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 0.03, seed=202)
    with ctx:
        ctx.set_band_model(learned.load_model())

        def frame():
            ctx.upload(pos, vel, rho)
            ctx.build_grid()
            ctx.surface_learned()
            return ctx.counts()

        ref = frame()
        ctx.set_wait_limit(0)
        with pytest.raises(pms.PmsError, match="tensor cores"):
            frame()
        ctx.set_wait_limit(-1)
        again = frame()
        assert again.n_valid_cubes == ref.n_valid_cubes > 0
        assert again.n_mesh_vertices == ref.n_mesh_vertices
        # batched frames: every lane's captured launches carry the limit, and the
        # frame reports the timeout too (no silent incomplete band)
        frames = [(pos, vel, rho), (pos, vel, rho)]
        ctx.run_batch(frames, learned=True)
        ok = ctx.batch_frame(0)[0].n_mesh_vertices
        assert ok == ref.n_mesh_vertices
        ctx.set_wait_limit(0)
        with pytest.raises(pms.PmsError, match="tensor cores"):
            ctx.run_batch(frames, learned=True)
        ctx.set_wait_limit(-1)
        ctx.run_batch(frames, learned=True)
        assert ctx.batch_frame(1)[0].n_mesh_vertices == ref.n_mesh_vertices
        with pytest.raises(pms.PmsError):
            ctx.set_wait_limit(0xffffffff)


@pytest.mark.gpu
def test_committed_model_gain_on_held_out_frame(pms_lib):
    pms = pms_lib
    from postmps_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model committed")
    model = learned.load_model()
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, 0.1, seed=200)
    h = float(pms.derive_params(cfg).h)
    with ctx:
        r = learned.compare(ctx, model, h, pos, vel, rho)
    # fewer field evaluations than the plain band, same surface within 0.05 h
    assert r["learned"]["band_vertices"] < 0.8 * r["plain"]["band_vertices"], r
    assert r["hausdorff"] <= 0.05 * h, r
    assert abs(r["triangle_delta"]) <= 0.002 * r["plain"]["triangles"] + 16, r
    assert r["cubes_only_learned"] == 0, r


def test_model_file_round_trip_and_config_key(pms_lib, tmp_path, tmp_config):
    pms = pms_lib
    rng = np.random.default_rng(2)
    m = pms.BandModel.from_arrays({"w1": LO.bf16_bits(rng.normal(0, 1, 4096).astype(np.float32)),
                                   "b1": rng.normal(0, 1, 64), "w2": LO.bf16_bits(rng.normal(0, 1, 64).astype(np.float32)),
                                   "b2": 0.25, "threshold": -1.5})
    path = str(tmp_path / "m.pmsband")
    pms.save_band_model(path, m, '{"frames": 3}')
    m2 = pms.load_band_model(path)
    assert bytes(m) == bytes(m2)
    from postmps_gb300 import learned
    assert learned.model_meta(path) == {"frames": 3}
    bad = tmp_path / "bad.pmsband"
    bad.write_bytes(open(path, "rb").read()[:100])
    with pytest.raises(pms.PmsError):
        pms.load_band_model(str(bad))
    cfg = pms.load_config(tmp_config(f"[Sim]\nMass = 1\n[GB300]\nBandModel = {path}\n"))
    assert cfg.band_model.decode() == path
    cfg = pms.load_config(tmp_config("[Sim]\nMass = 1\n"))
    assert cfg.band_model == b""
