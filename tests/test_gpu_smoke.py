"""The smoke entry point (__graft_entry__.smoke) runs as part of the GPU suite: a few
frames of the reference and FP32 forms through the C ABI, checked against the
oracle."""
import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry_point():
    import __graft_entry__ as g

    g.smoke()
