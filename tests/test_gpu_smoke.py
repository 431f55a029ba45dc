import pytest


@pytest.mark.gpu
def test_smoke(built):
    import __graft_entry__ as ge
    ge.smoke()


@pytest.mark.gpu
def test_l2_read_bandwidth_probe(built):
    """The L2 roofline denominator: a resident-buffer read rate above the HBM copy rate and below
    any physical L2 figure; malformed requests are refused."""
    import ctypes as C
    from multiq_workbench_gb300 import _native as N
    g = C.c_double(0.0)
    assert N.lib().mq_measure_l2_read_gbs(0, 32 << 20, 50, C.byref(g)) == 0
    assert 5000.0 < g.value < 100000.0
    assert N.lib().mq_measure_l2_read_gbs(0, 1 << 20, 50, C.byref(g)) == -1      # below 16 MiB
    assert N.lib().mq_measure_l2_read_gbs(0, 32 << 20, 0, C.byref(g)) == -1      # no sweeps
