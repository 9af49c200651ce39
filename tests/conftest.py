import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the product kernels")


@pytest.fixture(scope="session")
def built():
    """Builds the library and the oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def cuda_dev(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def no_traversal_faults(request):
    """Every renderer a GPU test closes (or drops) must report zero traversal
    faults: no node group dropped from a full stack, no walk cut short by the
    node budget. A test that provokes faults on purpose marks its renderer
    with `expect_traversal_faults = True`."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    import gc

    import optix_pt_gb300 as opt
    faults = []
    orig_close = opt.Renderer.close

    def checked_close(self):
        if getattr(self, "_h", None) and not getattr(self, "expect_traversal_faults", False):
            st = self.stats()
            if st["traversalStackOverflows"] or st["traversalBudgetExhausted"]:
                faults.append((st["traversalStackOverflows"], st["traversalBudgetExhausted"]))
        orig_close(self)

    opt.Renderer.close = checked_close
    try:
        yield
        gc.collect()
    finally:
        opt.Renderer.close = orig_close
    assert not faults, "traversal faults (stack overflows, walks cut short): %s" % faults
