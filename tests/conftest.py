import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running statistical check")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as ge
    ge.build()
    return True


@pytest.fixture(scope="session")
def coarse(built):
    """Default channel geometry at 0.4 mm (40 x 40 x 60 nodes), plate/downstream DC bases."""
    import multiq_workbench_gb300 as mq
    g = mq.Geom.with_spacing(0.4)
    return mq.Fields.build(g, bases=[0, 1, 2, 3, 4, 5])
