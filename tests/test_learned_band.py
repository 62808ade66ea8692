"""Learned narrow band.

CPU (oracle/learn_oracle.py, the checker): bf16 rounding, the oracle's own
gradient against finite differences, features and candidates on hand-made
cases.

GPU (through the C ABI): the tensor-core backward pass against the oracle's
gradient, the forward pass and the feature extraction against the oracle on
a real frame, training lowering the loss, the sign certification recovering
the plain mesh exactly from a crippled or empty predictor and without any
network, and the committed model on all ten full-size held-out frames: the
plain mesh, vertex for vertex, with fewer full field walks.
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
@pytest.mark.parametrize("keep", [0.5, 0.0])
def test_crippled_predictor_still_gives_the_plain_mesh(pms_lib, keep):
    """A predictor that keeps only half of the crossed cubes, and one that keeps
    none: the sign certification of the rest of the band finds every crossed
    cube, so the learned triangle soup is the plain one, vertex for vertex."""
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
        thr = float(np.quantile(pl, 0.5)) if keep else float(c["logit"].max()) + 1.0
        crippled = t.model(thr)
        r = learned.compare(ctx, crippled, h, pos, vel, rho)
        L = r["learned"]
        assert r["identical"], r
        assert r["cubes_only_plain"] == 0 and r["cubes_only_learned"] == 0 and r["triangle_delta"] == 0, r
        # the certified corners of valid cubes were evaluated exactly afterwards
        assert L["certified"] > 0 and L["rechecked"] > 0, r
        if not keep:
            assert L["predicted"] == 0 and L["exact_first"] == 0, r
        t.close()


@pytest.mark.gpu
def test_certified_band_without_network_gives_the_plain_mesh(pms_lib, tmp_config):
    """The certification alone (no network, every band vertex certified first) on
    the golden cases and the full 262,144-particle block: the triangle soup is
    the plain band's, vertex for vertex, and its cases are the oracle's
    classification of the plain field."""
    pms = pms_lib
    from conftest import golden_cases, load_golden
    from postmps_gb300 import learned, synth
    cases = [load_golden(c) for c in golden_cases()]
    cases.append({"config": synth.config_text(), "pos": synth.water_block(64)[0], "vel": None, "rho_in": None})
    for d in cases:
        cfg = pms.load_config(tmp_config(d["config"]))
        h = float(pms.derive_params(cfg).h)
        with pms.Context(cfg, 0) as ctx:
            r = learned.compare(ctx, None, h, d["pos"], d["vel"], d["rho_in"], mode="certified")
        assert r["identical"] and r["triangle_delta"] == 0, r
        assert r["learned"]["band_vertices"] == r["plain"]["band_vertices"]


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [0.05, 0.3])
def test_certificates_hold_and_exact_values_are_the_plain_ones(pms_lib, scale):
    """Every vertex the certified band left with a placeholder has an exact value
    above iso in the plain band (the certificate is right), the placeholder is
    above iso too, and every other band vertex carries the plain band's value bit
    for bit; the marching-cubes cases agree everywhere."""
    pms = pms_lib
    ctx, cfg, pos, vel, rho = _crown_ctx(pms, scale, seed=205)
    iso = float(pms.derive_params(cfg).iso_value)
    with ctx:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface()
        band_p, field_p, case_p = ctx.debug("band_list"), ctx.debug("field"), ctx.debug("cube_case")
        ctx.set_band_mode("certified")
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        ctx.surface_learned()
        band_c, field_c, case_c = ctx.debug("band_list"), ctx.debug("field"), ctx.debug("cube_case")
        cert = ctx.debug("band_certified")
        c = ctx.counts()
    np.testing.assert_array_equal(band_c, band_p)
    np.testing.assert_array_equal(case_c, case_p)
    held = ((cert[band_c >> 5] >> (band_c & 31)) & 1).astype(bool)
    assert held.sum() == c.n_band_certified - c.n_band_rechecked > 0
    assert np.all(field_p[held] > iso) and np.all(field_c[held] > iso)
    np.testing.assert_array_equal(field_c[~held], field_p[~held])


@pytest.mark.gpu
def test_all_held_out_frames_match_the_plain_mesh(pms_lib):
    """The committed model on the ten full-size held-out crown frames (seeds
    200-209, 1.3-1.75M particles, never trained on): every learned triangle soup
    is the plain one (no missed cube, no extra cube, Hausdorff 0), including the
    isolated single-vertex sign islands the network does not predict."""
    pms = pms_lib
    from postmps_gb300 import learned, synth
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model committed")
    model = learned.load_model()
    cfg = learned.crown_config()
    h = float(pms.derive_params(cfg).h)
    rows = []
    with pms.Context(cfg, 0) as ctx:
        for seed in learned.HELD_OUT_SEEDS:
            pos, vel, rho = synth.crown_variant(seed)
            r = learned.compare(ctx, model, h, pos, vel, rho)
            rows.append((seed, r["identical"], r["cubes_only_plain"], r["cubes_only_learned"], r["hausdorff_h"]))
    bad = [row for row in rows if not row[1] or row[2] or row[3] or row[4] > 0.0]
    assert not bad, rows


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
    # fewer full field walks than the plain band, the same surface
    assert r["learned"]["full_walks"] < 0.8 * r["plain"]["band_vertices"], r
    assert r["identical"], r


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
