"""The scratch-free prefix sum, pms_exclusive_scan_u32_noalloc, called through
the C ABI.

Some hosts cannot let the library allocate: a simulation or renderer that owns
all device memory through its own pool, or a frame loop that cannot take
cudaMalloc's implicit device synchronisation.  This entry point takes device
inputs and outputs only and uses a fixed 16 KiB file-scope scratch array.  The
test (which allocates its own buffers with torch) checks two calls in a row --
the second reuses the scratch left by the first -- against the existing path:
the cell starts that pms_build_grid computes with the library's allocating scan,
and numpy.  Integer results, compared exactly.  The file sorts last so that a
failing run stops after every other test has run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan(pms, torch, values: np.ndarray, stream=None):
    L = pms.lib()
    f = L.pms_exclusive_scan_u32_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    d_in = torch.from_numpy(values.astype(np.int32)).cuda()
    d_out = torch.empty_like(d_in)
    d_tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = f(d_in.data_ptr(), d_out.data_ptr(), len(values), d_tot.data_ptr(), stream)
    assert st == 0, pms.STATUS.get(st, st)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint32), int(d_tot.cpu().numpy().view(np.uint32)[0])


def test_no_alloc_scan_matches_the_allocating_path(pms_lib, tmp_config):
    torch = pytest.importorskip("torch")
    from postmps_gb300 import synth
    pms = pms_lib
    pos, vel, rho = synth.water_block(24)
    cfg = pms.load_config(tmp_config(synth.config_text()))
    with pms.Context(cfg, 0) as ctx:
        ctx.upload(pos, vel, rho)
        ctx.build_grid()
        start = ctx.debug("cell_start")
        end = ctx.debug("cell_end")
    counts = (end - start).astype(np.uint32)
    occupied = counts > 0

    # first call: the cell-count histogram of the frame
    got, total = _scan(pms, torch, counts)
    np.testing.assert_array_equal(got[occupied], start[occupied])   # the library's own cell starts
    assert total == len(pos)
    np.testing.assert_array_equal(got, np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32))

    # second call right after: different input and size, same scratch
    rng = np.random.default_rng(7)
    vals = rng.integers(0, 1000, size=5_000_003).astype(np.uint32)
    got2, total2 = _scan(pms, torch, vals)
    want2 = np.concatenate([[0], np.cumsum(vals.astype(np.uint64))[:-1]]).astype(np.uint32)
    np.testing.assert_array_equal(got2, want2)
    assert total2 == int(vals.astype(np.uint64).sum() & 0xFFFFFFFF)


def test_no_alloc_scan_limits(pms_lib):
    torch = pytest.importorskip("torch")
    L = pms_lib.lib()
    f = L.pms_exclusive_scan_u32_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    assert f(None, None, 33_554_433, None, None) == 4            # above the stated maximum
    assert f(None, None, 10, None, None) == 1                     # null arrays
    d_tot = torch.full((1,), 99, dtype=torch.int32, device="cuda")
    assert f(None, None, 0, d_tot.data_ptr(), None) == 0         # empty input: total 0
    torch.cuda.synchronize()
    assert int(d_tot.item()) == 0
