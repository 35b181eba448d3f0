"""The round-end smoke entry point (one design iteration of the 40x20 cantilever through
the public API, checked against the FP64 oracle) runs as part of the GPU suite."""
import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry_point():
    import __graft_entry__ as g
    g.smoke()
