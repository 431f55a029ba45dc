import pytest


@pytest.mark.gpu
def test_smoke(built):
    import __graft_entry__ as ge
    ge.smoke()
