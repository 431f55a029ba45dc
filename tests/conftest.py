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


@pytest.fixture(scope="session")
def s14_coarse(built):
    """Calibrated (S14 "code") channel geometry at 0.4 mm: the tandem's port grid, coarse."""
    import multiq_workbench_gb300 as mq
    return mq.Fields.build(mq.Geom.s14(h_mm=0.4, n_xy=40))


@pytest.fixture(scope="session")
def tandem_small(s14_coarse):
    """Factory of small tandem models: cube at 2.075 mm, ports on the 0.4 mm S14 grid."""
    import multiq_workbench_gb300 as mq

    def make(n=72, seed=486, mouth_start=True, tones=mq.DEFAULT_TONES, port_fields=None, **kw):
        return mq.TandemModel(tones, n=n, seed=seed, mouth_start=mouth_start, channel=s14_coarse,
                              port_fields=port_fields, cube_h=2.0, **kw)
    return make
