"""The device Laplace solver against the host solver: bit-identical potentials (same algorithm,
same operations in the same order), on the channel bases, the cube bases and a plates problem."""
import ctypes as C

import numpy as np
import pytest

import multiq_workbench_gb300 as mq
from multiq_workbench_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _solve(nx, ny, nz, mask, fixed, outer, tol, device):
    phi = np.zeros(nx * ny * nz)
    st = N.mq_solve_stats()
    L = N.lib()
    if device is None:
        rc = L.mq_laplace_solve(nx, ny, nz, mask.ctypes.data, fixed.ctypes.data, outer, tol, 0, phi.ctypes.data, C.byref(st))
    else:
        rc = L.mq_laplace_solve_device(nx, ny, nz, mask.ctypes.data, fixed.ctypes.data, outer, tol, device,
                                       phi.ctypes.data, C.byref(st))
    return rc, phi, st


def test_channel_bases_bitwise(built):
    g = mq.Geom.with_spacing(0.4)
    host = mq.Fields.build(g, cache=False)
    dev = mq.Fields.build(g, cache=False, device=0)
    for a, b in [(host.rf, dev.rf), (host.ac, dev.ac)] + list(zip(host.dc, dev.dc)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert [i.iterations for i in host.info] == [i.iterations for i in dev.info]


def test_channel_rf_basis_bitwise_at_0p1mm(built):
    g = mq.Geom()
    nx, ny, nz = g.dims()
    n = nx * ny * nz
    mask = np.zeros(n, np.uint8)
    fixed = np.zeros(n)
    outer = C.c_double(0.0)
    assert N.lib().mq_geom_basis_problem(C.byref(g.native()), 0, mask.ctypes.data, fixed.ctypes.data, n, C.byref(outer)) == 0
    rc_h, phi_h, st_h = _solve(nx, ny, nz, mask, fixed, outer.value, 1e-7, None)
    rc_d, phi_d, st_d = _solve(nx, ny, nz, mask, fixed, outer.value, 1e-7, 0)
    assert rc_h == rc_d == 0
    assert st_h.iterations == st_d.iterations and st_h.final_residual == st_d.final_residual
    assert np.array_equal(phi_h.view(np.uint64), phi_d.view(np.uint64))


def test_cube_fields_bitwise(built):
    g = mq.CubeGeometry.as_built()
    g.array = True
    gs, h = g.snap(2.0)
    a = mq.CubeFields.build(gs, h, 0.4, 1e-7, cache=False)
    b = mq.CubeFields.build(gs, h, 0.4, 1e-7, cache=False, device=0)
    for x, y in ((a.rf, b.rf), (a.wall, b.wall), (a.ent, b.ent), (a.ext, b.ext)):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_plates_are_linear(built):
    nx, ny, nz = 9, 9, 33
    mask = np.zeros(nx * ny * nz, np.uint8)
    fixed = np.zeros(nx * ny * nz)
    mask[: nx * ny] = 1                      # plate at k = 0, 0 V
    mask[-nx * ny:] = 1                      # plate at k = nz - 1, 1 V
    fixed[-nx * ny:] = 1.0
    # side faces follow the linear profile, so the exact solution is phi = k / (nz - 1)
    k = np.repeat(np.arange(nz), nx * ny)
    j = np.tile(np.repeat(np.arange(ny), nx), nz)
    i = np.tile(np.arange(nx), ny * nz)
    side = (i == 0) | (j == 0) | (i == nx - 1) | (j == ny - 1)
    mask[side] = 1
    fixed[side] = k[side] / (nz - 1)
    rc, phi, st = _solve(nx, ny, nz, mask, fixed, 0.0, 1e-10, 0)
    assert rc == 0 and st.converged
    assert np.max(np.abs(phi - k / (nz - 1))) < 1e-8


def test_device_solver_refusals(built):
    mask = np.zeros(8, np.uint8)
    fixed = np.zeros(8)
    assert _solve(2, 2, 2, mask, fixed, 0.0, 1e-7, 0)[0] == -1    # too small
    n = 5 * 5 * 5
    assert _solve(5, 5, 5, np.zeros(n, np.uint8), np.zeros(n), 0.0, 1e-7, 999)[0] == -6   # no such device
