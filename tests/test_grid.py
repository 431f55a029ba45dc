"""Field-grid set-up: geometry rasteriser, Laplace solver, E field, DC combination, cache."""
import ctypes as C

import numpy as np
import pytest


def test_default_dims_and_layers(built):
    import multiq_workbench_gb300 as mq
    g = mq.Geom()
    assert g.dims() == (160, 160, 242)                       # n_xy 160, nz = 24.2 mm / 0.1 mm
    assert np.allclose(g.layers(), [3.0, 15.0, 16.0, 17.6, 18.6, 21.6, 22.6, 24.2])
    assert g.axis() == 8.0
    assert mq.Geom.with_spacing(0.05).dims() == (320, 320, 484)
    assert mq.Geom.with_spacing(0.4).dims() == (40, 40, 60)


def test_classify_regions(built):
    import multiq_workbench_gb300 as mq
    g = mq.Geom()
    e = g.classify()                                          # (nz, ny, nx)
    a = 80
    assert (e[:31] == 0).all()                                # z <= q1_start: free
    assert e[100, a, a] == 0                                  # axis inside Q1 is free
    kind = (e.astype(int) - 1) // 4
    assert (kind[230][e[230] > 0] == 6).all() and (e[230] > 0).all()   # slab layer: every node is electrode
    plate = e[165]                                            # z = 16.5 mm (plate)
    yy, xx = np.mgrid[0:160, 0:160]
    r = np.hypot(xx - a, yy - a) * 0.1
    assert (plate[r < 3.4] == 0).all() and (plate[r > 3.6] > 0).all()
    # Q1 rods: centre of the LL rod (quadrant 0) at (a - c, a - c + sq) with c = 4.201 mm
    c = 0.323 * 6.35 / 2 + 6.35 / 2
    k = 100
    sq = 0.02 * (15.0 - k * 0.1)
    i, j = int(round((8.0 - c) / 0.1)), int(round((8.0 - c + sq) / 0.1))
    assert e[k, j, i] == 1                                    # code 1 + 4*kind(Q1=0) + quadrant 0


def test_laplace_solver_plates_linear(built):
    """Two parallel plates at 0 and 1 V with a grounded box far away: converges, and the
    discrete solution meets the residual bound."""
    import multiq_workbench_gb300 as mq
    from multiq_workbench_gb300 import _native as N
    nx = ny = 33
    nz = 21
    mask = np.zeros((nz, ny, nx), np.uint8)
    fixed = np.zeros((nz, ny, nx))
    mask[0] = 1
    mask[-1] = 1
    fixed[-1] = 1.0
    mask[:, :, 0] = mask[:, :, -1] = 1
    mask[:, 0, :] = mask[:, -1, :] = 1
    zz = np.arange(nz)[:, None, None] / (nz - 1) * np.ones((nz, ny, nx))
    fixed[:, :, 0] = fixed[:, :, -1] = zz[:, :, 0]
    fixed[:, 0, :] = fixed[:, -1, :] = zz[:, 0, :]
    phi = np.zeros(nx * ny * nz)
    st = N.mq_solve_stats()
    N.check(N.lib().mq_laplace_solve(nx, ny, nz, mask.ctypes.data, fixed.ctypes.data, 0.0, 1e-10, 0, phi.ctypes.data,
                                     C.byref(st)), "solve")
    assert st.converged and st.final_residual <= 1e-10
    assert np.abs(phi.reshape(nz, ny, nx) - zz).max() < 1e-8     # linear in z is the exact solution


def test_channel_basis_residual_and_symmetry(coarse):
    f = coarse
    assert all(i.cached or i.residual <= 1e-7 for i in f.info)
    rf = f.rf.reshape(f.nz, f.ny, f.nx, 4)
    # conductor mask only on electrode nodes; field finite
    assert set(np.unique(rf[..., 3])) <= {0.0, 1.0}
    assert np.isfinite(f.rf).all() and np.isfinite(f.ac).all()


def test_efield_of_linear_potential_is_exact(built):
    from multiq_workbench_gb300 import _native as N
    nx, ny, nz, h = 7, 6, 5, 1e-3
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    phi = (2.0 * i + 3.0 * j - 5.0 * k) * h
    e4 = np.zeros((nx * ny * nz, 4), np.float32)
    N.check(N.lib().mq_efield_central(np.ascontiguousarray(phi.reshape(-1)).ctypes.data, nx, ny, nz, h, e4.ctypes.data), "efield")
    assert np.allclose(e4[:, 0], -2.0) and np.allclose(e4[:, 1], -3.0) and np.allclose(e4[:, 2], 5.0)


def test_dc_combine_matches_float32_formula(coarse):
    f = coarse
    v = [18.0, 24.0, 15.0, 20.0]
    got = f.dc_field(v)
    acc = np.zeros((f.n, 3), np.float32)
    for b in range(4):
        acc = acc + np.float32(v[b]) * f.dc[b][:, :3]
    assert np.array_equal(got[:, :3], acc)


def test_rust_debug_key_of_default_geometry(built):
    import multiq_workbench_gb300 as mq
    s = mq.Geom().rust_debug()
    assert s == ("Geom { de: 6.35, coef: 0.323, q1_start: 3.0, q1_len: 12.0, alpha: 0.02, gap: 1.0, plate: 1.6, hole_d: 7.0, "
                 "q2_len: 3.0, stem_d: 4.6, q2_flare_bug: true, grow: 0.0, tilt_mode: 0, ac_mode: 0, "
                 "mis: [[0.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0]], "
                 "n_xy: 160, h_mm: 0.1 }")
    p = mq.cache_path(mq.Geom(), 0)
    assert p.name.startswith("ch_") and len(p.name) == len("ch_0123456789abcdef.bin")


def test_field_cache_roundtrip(built, tmp_path, monkeypatch):
    import multiq_workbench_gb300 as mq
    monkeypatch.setenv("CHSIM_CACHE_DIR", str(tmp_path))
    g = mq.Geom.with_spacing(0.8)
    a = mq.Fields.build(g, bases=[0, 1, 3])
    files = sorted(p.name for p in tmp_path.iterdir())
    assert len(files) == 3 and all(p.stat().st_size == 8 * a.n for p in tmp_path.iterdir())
    b = mq.Fields.build(g, bases=[0, 1, 3])
    assert all(i.cached for i in b.info)
    assert np.array_equal(a.rf, b.rf) and np.array_equal(a.ac, b.ac) and np.array_equal(a.dc[1], b.dc[1])
