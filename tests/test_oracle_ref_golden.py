"""The oracle's per-pass functions against the reference's own shaders, through the
committed fixtures (tests/golden/ref_passes.npz: inputs and the outputs of the
reference's HLSL compiled as C++, made by tests/golden/make_ref_golden.py). Runs
without the reference tree."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import call_with_args, ref_golden_cases

CASES = ref_golden_cases()


@pytest.mark.parametrize("k", range(len(CASES)), ids=["%s-%d" % (c[0], i) for i, c in enumerate(CASES)])
def test_oracle_pass_matches_reference_shader(k):
    name, args, expect = CASES[k]
    arrays = []  # (kind, host array) per array argument, in order

    def arr(kind, v):
        a = np.array(v, copy=True)
        arrays.append((kind, a))
        return C.c_void_p(a.ctypes.data)

    call, keep = call_with_args(None, args, arr, po._ffi.FrameParams, po._ffi.Params)
    getattr(po.lib(), "vlto_" + name)(*call)
    got = [a for kind, a in arrays if kind != "in"]
    assert len(got) == len(expect)
    for i, (g, e) in enumerate(zip(got, expect)):
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, "%s output %d: %d bytes differ from the reference shader, first at %d" % (
            name, i, bad.size, bad[0])
