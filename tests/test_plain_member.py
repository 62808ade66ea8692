"""The learned band's plain-band membership test, restated on the CPU and pinned
against the reference's own band (golden fixtures).  CPU only.

The GPU test (k_band.cu, in_plain_band) decides per vertex u whether some
surface particle marks u, u - 1, u - rx or u - rx*ry (the dilation in linear
order), with k_band_mark's AABB, direction and index-box tests, looking only at
the surface particles of the particle cells within h of the vertex.  Here the
same per-vertex rule, in float32 with the same roundings, must give exactly the
reference's band vertices, and every particle that marks a vertex must lie
inside that vertex's cell window with a margin (so the window the kernel scans
cannot miss it).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, load_golden

F = np.float32


def setup(oracle, d):
    keys = oracle.parse_ini(d["config"])
    p = oracle.derive_params(oracle.config_from_keys(keys))
    g = oracle.grid_from_positions(p, d["pos"])
    return p, g


def b0_by_vertex(g, h: float, sp: np.ndarray, nrm: np.ndarray, flag: np.ndarray):
    """B0 evaluated vertex by vertex (one z slab at a time), and the largest
    amount by which a marking particle's cell comes near the edge of the
    vertex's cell window (negative: outside)."""
    rx, ry, rz = (int(v) for v in g.scres)
    cs = F(g.sc_grid_size)
    scmin = np.array(g.scmin_pos[:], F)
    h32 = F(h)
    ext = int(np.ceil(F(h32 / cs)))
    res = np.array([rx, ry, rz])
    # particle side: AABB bounds, index box, particle cell (float32 like the kernels)
    aa = (sp - h32).astype(F)
    bb = (sp + h32).astype(F)
    c = np.trunc(((sp - scmin).astype(F) / cs).astype(F)).astype(np.int64)
    lo = np.clip(c - ext, 0, res - 1)
    hi = np.clip(c + ext, 0, res - 1)
    mn = np.array(g.min_pos[:], F)
    spc = F(g.sp_grid_size)
    pcell = np.floor(((sp - mn).astype(F) / spc).astype(F)).astype(np.int64)
    # the kernel's window reaches h / cell + 0.01 cells; asking for 0.009 leaves
    # room for its float32 rounding
    r_cells = float(h) / float(spc) + 0.009
    # vertex side
    ix = np.arange(rx)
    iy = np.arange(ry)
    vx = ((ix.astype(F) * cs).astype(F) + scmin[0]).astype(F)
    vy = ((iy.astype(F) * cs).astype(F) + scmin[1]).astype(F)
    b0 = np.zeros(rx * ry * rz, bool)
    worst = np.inf
    X, Y = np.meshgrid(ix, iy, indexing="xy")
    VX, VY = np.meshgrid(vx, vy, indexing="xy")
    X, Y, VX, VY = X.ravel(), Y.ravel(), VX.ravel(), VY.ravel()
    for z in range(rz):
        vz = F(F(F(z) * cs) + scmin[2])
        sel = np.flatnonzero((aa[:, 2] <= vz) & (vz <= bb[:, 2]) & (lo[:, 2] <= z) & (z <= hi[:, 2]))
        if len(sel) == 0:
            continue
        P, N, A, B, L, H = sp[sel], nrm[sel], aa[sel], bb[sel], lo[sel], hi[sel]
        inside = ((VX[:, None] >= A[None, :, 0]) & (VX[:, None] <= B[None, :, 0]) &
                  (VY[:, None] >= A[None, :, 1]) & (VY[:, None] <= B[None, :, 1]) &
                  (X[:, None] >= L[None, :, 0]) & (X[:, None] <= H[None, :, 0]) &
                  (Y[:, None] >= L[None, :, 1]) & (Y[:, None] <= H[None, :, 1]))
        d0 = (VX[:, None] - P[None, :, 0]).astype(F)
        d1 = (VY[:, None] - P[None, :, 1]).astype(F)
        d2 = (vz - P[None, :, 2]).astype(F)
        dot = (((N[None, :, 0] * d0).astype(F) + (N[None, :, 1] * d1).astype(F)).astype(F) +
               (N[None, :, 2] * d2).astype(F)).astype(F)
        marks = inside & ((flag[sel] != 0)[None, :] | (dot > 0))
        b0[z * rx * ry + np.arange(rx * ry)] = marks.any(axis=1)
        # window margins of the marking pairs, in particle cells, float64
        vi, pj = np.nonzero(marks)
        if len(vi):
            u = np.stack([(VX[vi] - mn[0]) / float(spc), (VY[vi] - mn[1]) / float(spc),
                          np.full(len(vi), (float(vz) - float(mn[2])) / float(spc))], 1)
            pc = pcell[sel][pj]
            lo_w = np.floor(u - r_cells)
            hi_w = np.floor(u + r_cells)
            worst = min(worst, float(np.min(np.minimum(pc - lo_w, hi_w - pc))))
    return b0, worst


@pytest.mark.parametrize("case", golden_cases())
def test_vertex_side_rule_gives_the_reference_band(oracle, case):
    d = load_golden(case)
    if "band_list" not in d:
        pytest.skip("no band in this fixture")
    p, g = setup(oracle, d)
    sp = np.ascontiguousarray(d["pos"][d["perm"]], F)[d["surf_list"]]
    b0, worst = b0_by_vertex(g, float(p.h), sp, np.asarray(d["nrm"], F), np.asarray(d["flag"]))
    rx, ry = int(g.scres[0]), int(g.scres[1])
    band = b0.copy()
    for s in (1, rx, rx * ry):                     # the dilation in linear order, row wrap included
        band[s:] |= b0[:-s]
    np.testing.assert_array_equal(np.flatnonzero(band), d["band_list"])
    # every marking particle's cell lies inside the vertex's window, not on its edge
    assert worst >= 0, worst
