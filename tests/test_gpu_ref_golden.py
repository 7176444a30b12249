"""The product's per-pass kernels against the reference's own shaders, directly.

tests/golden/ref_passes.npz holds inputs and the outputs of the reference's HLSL
compiled as C++ (tests/golden/make_ref_golden.py, oracle/ref_build.py) for every
per-pass entry point, on the state of a reference-preset view after 4 frames at
37x23 (partial groups at the edges). Each case runs through the C ABI on the GPU and
every output byte must equal the reference shader's. This ties the kernels to the
reference's text without going through the oracle restatement.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import call_with_args, ref_golden_cases

pytestmark = pytest.mark.gpu

CASES = ref_golden_cases()


def product_args(name, args):
    """The product's entry points take the same arguments as the reference-form
    oracle's, without the colour form and stride of the post passes, with caller
    scratch for the query selection, and a trailing stream."""
    args = list(args)
    if name in ("final_lighting", "temporal_aa"):
        assert args[0] == ("i32", 0)
        args = args[1:]
        if name == "final_lighting":
            assert args[7] == ("i32", 1)
            args = args[:7] + args[8:]
    if name == "hg_query_select":
        args.append(("scratch", None))
    return args + [("none", None)]


@pytest.mark.parametrize("k", range(len(CASES)), ids=["%s-%d" % (c[0], i) for i, c in enumerate(CASES)])
def test_kernel_matches_reference_shader(k):
    import torch

    name, args, expect = CASES[k]
    lib = vg.lib()
    args = product_args(name, args)
    dev = []  # (kind, tensor)

    def arr(kind, v):
        t = torch.from_numpy(np.array(v, copy=True)).cuda() if v.size else torch.zeros(16, dtype=torch.uint8,
                                                                                       device="cuda")
        dev.append((kind, t))
        return C.c_void_p(t.data_ptr())

    scratch = None
    if name == "hg_query_select":
        nb = lib.vlt_hg_select_scratch_bytes(args[0][1], args[1][1])
        scratch = torch.empty(max(int(nb), 16), dtype=torch.uint8, device="cuda")
        args = [a if a[0] != "scratch" else ("ptr", scratch.data_ptr()) for a in args]
    call, keep = call_with_args(None, [a if a[0] != "ptr" else ("none", None) for a in args], arr,
                                vg._ffi.FrameParams, vg._ffi.Params)
    if scratch is not None:
        call[[i for i, a in enumerate(args) if a[0] == "ptr"][0]] = C.c_void_p(scratch.data_ptr())
    rc = getattr(lib, "vlt_" + name)(*call)
    assert rc == 0, "vlt_%s returned %d" % (name, rc)
    torch.cuda.synchronize()
    got = [t.cpu().numpy() for kind, t in dev if kind != "in"]
    assert len(got) == len(expect)
    for i, (g, e) in enumerate(zip(got, expect)):
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, "vlt_%s output %d: %d bytes differ from the reference shader, first at %d" % (
            name, i, bad.size, bad[0])
