"""Tandem transport on the GPU: the FP64 kernel against the oracle, bit for bit (track states
and every per-port counter), across resumed advances, both launch modes, per-port grids of
different spacing, and the host's refusals."""
import numpy as np
import pytest

import multiq_workbench_gb300 as mq
from oracle import mqtandem as O

pytestmark = pytest.mark.gpu


def _same_tracks(a, b):
    for k, _ in O.TRACK_FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        if not np.array_equal(x.view(np.uint8), y.view(np.uint8)):
            diff = np.flatnonzero(x != y)
            raise AssertionError(f"{k}: {diff.size} tracks differ, first {diff[:5]}: {x[diff[:5]]} vs {y[diff[:5]]}")


def _run_both(m, chunks, seed, mouth):
    d = O.desc_from(m.desc)
    ref = O.inject(d, seed, mouth, m.tracks.n)
    cnt = np.zeros((9, O.NC), np.uint32)
    s0 = 0
    for k in chunks:
        m.advance(k)
        O.advance(d, ref, s0, k, counts=cnt)
        s0 += k
    return ref, cnt


@pytest.mark.parametrize("mouth", [True, False])
def test_tandem_gpu_matches_oracle_bitwise(tandem_small, mouth):
    m = tandem_small(n=301, seed=486, mouth_start=mouth)
    ref, cnt = _run_both(m, [5000, 7001, 12999], 486, mouth)
    _same_tracks(m.tracks, ref)
    assert np.array_equal(m.counts_array(), cnt)
    assert m.counts_array()[:, 0].sum() > 0   # ports were entered
    m.close()


def test_tandem_gpu_per_port_grids(tandem_small, s14_coarse):
    """Ragged batching by field id: ports on grids of different spacing and shape."""
    other = mq.Fields.build(mq.Geom.s14(h_mm=0.5, n_xy=32))
    ports = [s14_coarse if i % 2 == 0 else other for i in range(9)]
    m = tandem_small(n=200, seed=99, port_fields=ports)
    ref, cnt = _run_both(m, [9000, 9000], 99, True)
    _same_tracks(m.tracks, ref)
    assert np.array_equal(m.counts_array(), cnt)
    m.close()


def test_tandem_gpu_long_run_conservation(tandem_small):
    n = 2048
    m = tandem_small(n=n, seed=2024)
    ref, cnt = _run_both(m, [40000, 40000], 2024, True)
    _same_tracks(m.tracks, ref)
    got = m.counts_array()
    assert np.array_equal(got, cnt)
    f = m.frame()
    assert f.split + f.channel + f.combine + f.detected + f.lost + f.back == n
    assert (got[:, 0] + got[:, 14]).sum() == (got[:, 1] + got[:, 2] + got[:, 15]).sum() + f.channel
    assert got[:, 4].sum() > 0 and got[:, 2].sum() > 0   # from_other and forwarded happen
    m.close()


def test_tandem_gpu_refuses_bad_tracks(tandem_small):
    m = tandem_small(n=8)
    m.tracks.sp[3] = 6
    with pytest.raises(mq.MqError) as e:
        m.advance(10)
    assert e.value.code == -1
    m.tracks.sp[3] = 0
    m.tracks.region[5] = 14
    with pytest.raises(mq.MqError):
        m.advance(10)
    m.tracks.region[5] = 0
    m.advance(10)   # the model is still usable
    m.close()
