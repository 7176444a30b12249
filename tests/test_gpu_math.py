"""GPU: the library's own transcendentals agree bit for bit with the oracle's."""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _inputs(fn):
    rng = np.random.default_rng(1)
    if fn in ("exp2_fma", "exp2_fma_full"):
        # every 241st binary32 value of [-127, 1] (the short path's range and its edges)
        lo, hi = np.float32(-127.0).view(np.uint32), np.float32(1.0).view(np.uint32)
        neg = np.arange(0x80000000, lo + 1, 241, dtype=np.uint64).astype(np.uint32).view(np.float32)
        pos = np.arange(0, hi + 1, 241, dtype=np.uint64).astype(np.uint32).view(np.float32)
        x = np.concatenate([neg, pos, rng.uniform(-160, 130, 200000).astype(np.float32),
                            np.array([0.0, -0.0, -126.0, -125.5, -126.5, 1e-45, -1e-45, 127.5, -150.5, np.inf,
                                      -np.inf, np.nan], np.float32)])
    elif fn in ("exp2", "exp"):
        x = np.concatenate([rng.uniform(-160, 130, 200000), rng.uniform(-2, 2, 200000),
                            [0.0, -0.0, 1.0, -1.0, 127.49, 127.5, 127.99, -126.0, -126.5, -149.5, -150.0, -151.0,
                             np.inf, -np.inf, np.nan]])
    elif fn == "log2":
        x = np.concatenate([np.exp(rng.uniform(-100, 88, 200000)), rng.uniform(0, 4, 200000),
                            [0.0, -0.0, 1.0, 2.0, 0.5, 1e-45, 1e-40, 1.17549435e-38, np.inf, -1.0, np.nan]])
    elif fn == "f16_pair":
        # around the half range's edges, its subnormals and rounding ties, and specials
        x = np.concatenate([rng.uniform(-7e4, 7e4, 200000), np.exp(rng.uniform(-20, 11.2, 200000)),
                            np.arange(65480, 65540, 0.25), np.arange(-1e-4, 1e-4, 3e-8),
                            [0.0, -0.0, 65504.0, 65519.996, 65520.0, 1e30, 5.96e-8, 2.98e-8, 2.99e-8,
                             np.inf, -np.inf, np.nan, 1.0009765625, 1.00048828125]])
    else:
        x = np.concatenate([rng.uniform(-50, 50, 200000), rng.uniform(-7, 7, 200000),
                            [0.0, -0.0, np.pi / 4, np.pi / 2, np.pi, 65536.0, 65537.0, np.inf, np.nan]])
    return x.astype(np.float32)


@pytest.mark.parametrize("fn", ["exp2", "exp", "log2", "sin", "cos", "exp2_fma", "exp2_fma_full", "f16_pair"])
def test_own_math_bit_exact(fn):
    import torch

    x = _inputs(fn)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    lib = vg.lib()
    fid = po.MATH[fn]
    rc = lib.vlt_diag_math(fid, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), x.size, None)
    assert rc == 0
    got = yd.cpu().numpy()
    exp = po.math(fn, x)
    gb, eb = got.view(np.uint32), exp.view(np.uint32)
    nan = np.isnan(got) & np.isnan(exp)
    bad = np.nonzero((gb != eb) & ~nan)[0]
    assert bad.size == 0, "%s: %d mismatches, first x=%r gpu=%r oracle=%r" % (
        fn, bad.size, x[bad[0]], got[bad[0]], exp[bad[0]])
