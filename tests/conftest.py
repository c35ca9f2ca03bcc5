import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    from oracle_lib import Oracle
    return Oracle("orc")


@pytest.fixture(scope="session")
def ref():
    from oracle_lib import Oracle, ref_available
    if not ref_available():
        pytest.skip("reference build oracle/_ref not present on this host")
    return Oracle("ref")


@pytest.fixture(params=["persistent", "graph", "team"])
def executor(request, cuda):
    """Runs a test with the persistent step executor, with per-step kernel
    launches captured in a CUDA graph (whole-solve launches off for both),
    and with small Krylov solves in one whole-solve launch."""
    from unap_gb300 import capi
    old = capi.set_executor(request.param == "persistent")
    cells = capi.set_team_solve_cells(1 << 20 if request.param == "team" else 0)
    yield request.param
    capi.set_executor(old)
    capi.set_team_solve_cells(cells)


TAIL_MODES = {
    "per-wavefront": (0, 0),            # one kernel per wavefront on every level
    "cluster": (1 << 40, 0),            # every level in the cluster tail, all CTAs
    "one-cta": (1 << 40, 1 << 40),      # every level in the tail, first CTA alone
    "split": (1 << 40, 600),            # cluster levels above 600 rows, one CTA below
}


@pytest.fixture(params=sorted(TAIL_MODES))
def tail_mode(request, cuda):
    """Runs a test under each placement of the AMG V-cycle's coarse levels
    (per-wavefront launches, the cluster tail kernel on all CTAs, on one CTA,
    and split between the two)."""
    from unap_gb300 import capi
    if request.param != "per-wavefront" and capi.tail_cluster_size() < 1:
        pytest.skip("device schedules no thread-block cluster for the tail kernel")
    old = capi.set_tail_rows(*TAIL_MODES[request.param])
    yield request.param
    capi.restore_tail_rows(old)


@pytest.fixture(scope="session")
def cuda():
    """torch with a CUDA device, and the product library loaded."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test on a host without CUDA")
    from unap_gb300 import capi
    capi.load()
    return torch
