"""ctypes view of ``libmqgb.so`` (declarations in include/mq_grid.h, include/mq_engine.h and
include/mq_tandem.h).

The library is built in-tree by :mod:`multiq_workbench_gb300.build`.  Loading fails
loudly if it is missing: there is no Python or CPU fallback for any engine call.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# MQ_LIB selects another build of the library (the bounds-checked libmqgb_check.so)
_LIB_PATH = Path(os.environ["MQ_LIB"]) if os.environ.get("MQ_LIB") else Path(__file__).resolve().parent / "libmqgb.so"
_lib = None

MQ_OK = 0
MQ_PREC_F64 = 0     # include/mq_engine.h
MQ_PREC_MIXED = 1
MQ_ERRORS = {
    -1: "invalid argument",
    -2: "CUDA runtime error",
    -3: "out of memory",
    -4: "device watchdog expired",
    -5: "RF drive must be shared by a batch",
    -6: "no CUDA device",
    -7: "Laplace solve did not converge",
    -8: "request exceeds a fixed capacity",
}


class MqError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str = ""):
        self.code = code
        msg = f"{what}: {MQ_ERRORS.get(code, 'error')} ({code})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


class mq_geom(C.Structure):
    _fields_ = [
        ("de", C.c_double), ("coef", C.c_double), ("q1_start", C.c_double), ("q1_len", C.c_double),
        ("alpha", C.c_double), ("gap", C.c_double), ("plate", C.c_double), ("hole_d", C.c_double),
        ("q2_len", C.c_double), ("stem_d", C.c_double), ("q2_flare_bug", C.c_int32), ("tilt_mode", C.c_int32),
        ("ac_mode", C.c_int32), ("n_xy", C.c_int32), ("grow", C.c_double), ("h_mm", C.c_double),
        ("mis", C.c_double * 16),
    ]


class mq_solve_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("final_residual", C.c_double), ("seconds", C.c_double)]


class mq_grid_desc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("pad", C.c_int32), ("h", C.c_double),
                ("rf4", C.c_void_p), ("ac4", C.c_void_p), ("dc4", C.c_void_p * 4), ("axis_mm", C.c_double),
                ("layers_mm", C.c_double * 8)]


class mq_species(C.Structure):
    _fields_ = [("mass", C.c_double), ("z", C.c_double), ("ccs_n2", C.c_double)]


class mq_rfac(C.Structure):
    _fields_ = [("v_rf", C.c_double), ("f_rf", C.c_double), ("v_ac", C.c_double), ("f_ac", C.c_double)]


class mq_job(C.Structure):
    _fields_ = [("sp", mq_species), ("drive", mq_rfac), ("n", C.c_uint64), ("seed", C.c_uint64)]


class mq_physics(C.Structure):
    _fields_ = [
        ("legacy_force", C.c_int32), ("legacy_collisions", C.c_int32), ("legacy_fields", C.c_int32),
        ("legacy_injection", C.c_int32), ("legacy_criteria", C.c_int32), ("launch", C.c_int32),
        ("rf_phase0", C.c_int32), ("pad0", C.c_int32),
        ("pressure_pa", C.c_double), ("temp_k", C.c_double), ("dt", C.c_double), ("t_max", C.c_double),
        ("r_inject_mm", C.c_double), ("sigma_mm", C.c_double), ("z_inject_mm", C.c_double),
    ]


class mq_outcome(C.Structure):
    _fields_ = [("n", C.c_uint64), ("crashed", C.c_uint64), ("returned", C.c_uint64), ("transmitted", C.c_uint64),
                ("left", C.c_uint64), ("timeout", C.c_uint64), ("mean_coll", C.c_double), ("mean_time", C.c_double)]


class mq_ions(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("vx", C.c_void_p), ("vy", C.c_void_p),
                ("vz", C.c_void_p), ("ph_rf", C.c_void_p), ("ph_ac", C.c_void_p), ("rng", C.c_void_p),
                ("steps", C.c_void_p), ("ncoll", C.c_void_p), ("leg", C.c_void_p), ("status", C.c_void_p),
                ("jid", C.c_void_p)]


class mq_run_stats(C.Structure):
    _fields_ = [("ion_steps", C.c_uint64), ("kernel_ms", C.c_double), ("launches", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("step_kernel_ms", C.c_double), ("step_kernel_launches", C.c_uint32), ("graph_replays", C.c_uint32),
                ("cell_loads", C.c_uint64), ("ions_queued", C.c_uint64)]


class mq_dev_grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("pad", C.c_int32), ("h", C.c_double),
                ("rf4", C.c_void_p), ("ac4", C.c_void_p), ("dc4", C.c_void_p), ("axis_mm", C.c_double),
                ("layers_mm", C.c_double * 8)]


class mq_tuning(C.Structure):
    _fields_ = [("threads_per_block", C.c_int32), ("blocks_per_sm", C.c_int32), ("chunk", C.c_uint32),
                ("use_graph", C.c_int32), ("prefetch", C.c_int32),
                ("wide_records", C.c_int32), ("sort_cells", C.c_int32)]


class mq_cube_geom(C.Structure):
    _fields_ = [("n", C.c_int32), ("array", C.c_int32)] + [
        (k, C.c_double) for k in ("d", "pitch", "height", "t_pcb", "gap", "stem_r", "clear_r", "l_ext", "ap_r",
                                  "rod_clear_extra", "cap_gap", "cap_r")
    ] + [("ent_axis", C.c_int32), ("ent_side", C.c_int32), ("ent_cell", C.c_int32 * 2),
         ("ext_axis", C.c_int32), ("ext_side", C.c_int32), ("ext_cell", C.c_int32 * 2)]


class mq_tandem_port(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("pad", C.c_int32), ("h", C.c_double), ("rf4", C.c_void_p),
                ("ac4", C.c_void_p), ("dc4", C.c_void_p), ("gate4", C.c_void_p), ("tone_khz", C.c_double),
                ("v_ac", C.c_double)]


class mq_tandem_species(C.Structure):
    _fields_ = [("mass", C.c_double), ("z", C.c_double), ("ccs", C.c_double), ("weight", C.c_double)]


class mq_tandem_desc(C.Structure):
    _fields_ = [("cube", mq_cube_geom), ("cube_dims", C.c_int32 * 3), ("pad0", C.c_int32),
                ("cube_lo_mm", C.c_double * 3), ("cube_h_mm", C.c_double), ("cube_rf4", C.c_void_p),
                ("cube_dc4", C.c_void_p * 2), ("port", mq_tandem_port * 9), ("ch_axis_mm", C.c_double),
                ("ch_q1_start_mm", C.c_double), ("v_rf", C.c_double), ("f_rf", C.c_double),
                ("pressure_pa", C.c_double), ("temp_k", C.c_double), ("dt", C.c_double), ("gate_bias_v", C.c_double),
                ("nspecies", C.c_int32), ("precision", C.c_int32), ("species", mq_tandem_species * 8)]


class mq_tracks(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "rng", "sp", "region", "last")]


class mq_port_counts(C.Structure):
    _fields_ = [("entered", C.c_uint32), ("returned", C.c_uint32), ("forwarded", C.c_uint32),
                ("revisits", C.c_uint32), ("from_other", C.c_uint32), ("retry_from", C.c_uint32 * 9),
                ("reverse_entries", C.c_uint32), ("lost", C.c_uint32), ("by_charge", C.c_uint32 * 5)]


class mq_tandem_stats(C.Structure):
    _fields_ = [("steps_cube", C.c_uint64), ("steps_port", C.c_uint64), ("steps_idle", C.c_uint64),
                ("kernel_ms", C.c_double), ("launches", C.c_uint32), ("pad", C.c_uint32), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("cell_fills_cube", C.c_uint64), ("cell_fills_port", C.c_uint64)]


class mq_tandem_frame_counts(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("split", "channel", "combine", "lost", "back", "detected")]


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"native library missing: {_LIB_PATH} (run multiq_workbench_gb300.build.build())")
        L = C.CDLL(str(_LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


def _declare(L) -> None:
    P = C.POINTER
    L.mq_geom_default.argtypes = [P(mq_geom)]
    L.mq_geom_default.restype = None
    L.mq_geom_dims.argtypes = [P(mq_geom), P(C.c_int32)]
    L.mq_geom_dims.restype = C.c_int32
    L.mq_geom_axis_mm.argtypes = [P(mq_geom)]
    L.mq_geom_axis_mm.restype = C.c_double
    L.mq_geom_layers.argtypes = [P(mq_geom), P(C.c_double)]
    L.mq_geom_layers.restype = None
    L.mq_geom_classify.argtypes = [P(mq_geom), C.c_void_p, C.c_size_t]
    L.mq_geom_classify.restype = C.c_int32
    L.mq_geom_basis_problem.argtypes = [P(mq_geom), C.c_int32, C.c_void_p, C.c_void_p, C.c_size_t, P(C.c_double)]
    L.mq_geom_basis_problem.restype = C.c_int32
    L.mq_laplace_solve.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                   C.c_int32, C.c_void_p, P(mq_solve_stats)]
    L.mq_laplace_solve.restype = C.c_int32
    L.mq_efield_central.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p]
    L.mq_efield_central.restype = C.c_int32
    L.mq_channel_basis.argtypes = [P(mq_geom), C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_void_p, P(mq_solve_stats)]
    L.mq_channel_basis.restype = C.c_int32
    L.mq_channel_basis_ex.argtypes = [P(mq_geom), C.c_int32, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                      P(mq_solve_stats)]
    L.mq_channel_basis_ex.restype = C.c_int32
    L.mq_laplace_solve_device.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                          C.c_int32, C.c_void_p, P(mq_solve_stats)]
    L.mq_laplace_solve_device.restype = C.c_int32
    L.mq_dc_combine.argtypes = [C.c_size_t, C.c_void_p * 4, P(C.c_double), C.c_void_p]
    L.mq_dc_combine.restype = C.c_int32
    if hasattr(L, "mq_engine_create"):
        _declare_engine(L)
    if hasattr(L, "mq_tandem_create"):
        _declare_tandem(L)
    if hasattr(L, "mq_fit_binomial_curve"):
        _declare_fit(L)


class mq_res_fit(C.Structure):
    _fields_ = [("shape", C.c_int32), ("converged", C.c_int32), ("p", C.c_double * 4), ("e", C.c_double * 4),
                ("cov", C.c_double * 16), ("chi2", C.c_double), ("chi2_flat", C.c_double), ("dof", C.c_int64),
                ("scale", C.c_double), ("n_pts", C.c_uint64), ("r", C.c_double), ("r_err", C.c_double),
                ("has_boot", C.c_int32), ("pad", C.c_int32), ("r_boot_mean", C.c_double), ("r_boot_sd", C.c_double),
                ("f0_boot_sd", C.c_double)]


def _declare_fit(L) -> None:
    P = C.POINTER
    vp, sz, d, u64, i32 = C.c_void_p, C.c_size_t, C.c_double, C.c_uint64, C.c_int32
    L.mq_fit_model.argtypes = [i32, vp, d]
    L.mq_fit_model.restype = d
    L.mq_fit_shape_sigma.argtypes = [i32, vp, vp, vp, sz, P(mq_res_fit)]
    L.mq_fit_shape_sigma.restype = i32
    L.mq_fit_binomial_shape.argtypes = [i32, vp, vp, vp, sz, u64, u64, P(mq_res_fit)]
    L.mq_fit_binomial_shape.restype = i32
    L.mq_fit_binomial_curve.argtypes = [vp, vp, vp, sz, u64, u64, P(mq_res_fit)]
    L.mq_fit_binomial_curve.restype = i32
    L.mq_fit_is_significant.argtypes = [P(mq_res_fit), vp, sz]
    L.mq_fit_is_significant.restype = i32
    L.mq_fit_r_mz.argtypes = [d, d, d, d, vp]
    L.mq_fit_r_mz.restype = None
    L.mq_rng_seed.argtypes = [u64]
    L.mq_rng_seed.restype = u64
    L.mq_rng_uniform.argtypes = [P(u64)]
    L.mq_rng_uniform.restype = d
    L.mq_rng_binomial_fill.argtypes = [P(u64), vp, vp, sz, vp]
    L.mq_rng_binomial_fill.restype = None
    L.mq_mathieu_beta.argtypes = [d, d]
    L.mq_mathieu_beta.restype = d
    L.mq_sec_freq_khz.argtypes = [d, d, d, d, d]
    L.mq_sec_freq_khz.restype = d
    L.mq_terrain_tables.argtypes = [i32, i32, i32, d, d, vp, vp * 4, sz, vp, vp, vp, P(sz)]
    L.mq_terrain_tables.restype = i32
    L.mq_terrain_compute.argtypes = [sz, sz, vp, vp, vp, vp, sz, d, vp, d, vp, vp]
    L.mq_terrain_compute.restype = i32
    L.mq_terrain_dfdmz.argtypes = [sz, sz, vp, vp, vp, d, d, d, vp, d]
    L.mq_terrain_dfdmz.restype = d
    L.mq_secular_freq.argtypes = [vp, i32, i32, i32, d, d, d, d, d, d, P(d)]
    L.mq_secular_freq.restype = i32


def _declare_tandem(L) -> None:
    P = C.POINTER
    L.mq_cube_as_built.argtypes = [P(mq_cube_geom)]
    L.mq_cube_as_built.restype = None
    L.mq_cube_snap.argtypes = [P(mq_cube_geom), C.c_double, P(mq_cube_geom), P(C.c_double)]
    L.mq_cube_snap.restype = C.c_int32
    L.mq_cube_classify.argtypes = [P(mq_cube_geom), P(C.c_double), C.c_double, P(C.c_int32)]
    L.mq_cube_classify.restype = C.c_int32
    L.mq_cube_size.argtypes = [P(mq_cube_geom)]
    L.mq_cube_size.restype = C.c_double
    L.mq_cube_post_top_depth.argtypes = [P(mq_cube_geom)]
    L.mq_cube_post_top_depth.restype = C.c_double
    L.mq_cube_nearest_port.argtypes = [P(mq_cube_geom), C.c_double, C.c_double]
    L.mq_cube_nearest_port.restype = C.c_int32
    L.mq_cube_port_axis.argtypes = [P(mq_cube_geom), C.c_int32, P(C.c_double)]
    L.mq_cube_port_axis.restype = C.c_int32
    L.mq_efield_fieldsolve.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p]
    L.mq_efield_fieldsolve.restype = C.c_int32
    L.mq_cube_fields.argtypes = [P(mq_cube_geom), C.c_double, C.c_double, C.c_double, C.c_int32, P(C.c_int32),
                                 P(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, P(mq_solve_stats)]
    L.mq_cube_fields.restype = C.c_int32
    L.mq_cube_fields_ex.argtypes = [P(mq_cube_geom), C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                    P(C.c_int32), P(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    P(mq_solve_stats)]
    L.mq_cube_fields_ex.restype = C.c_int32
    L.mq_cube_dc_combined.argtypes = [C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_void_p]
    L.mq_cube_dc_combined.restype = C.c_int32
    L.mq_tandem_create.argtypes = [P(mq_tandem_desc), C.c_int32, P(C.c_void_p)]
    L.mq_tandem_create.restype = C.c_int32
    L.mq_tandem_destroy.argtypes = [C.c_void_p]
    L.mq_tandem_destroy.restype = None
    L.mq_tandem_last_error.argtypes = [C.c_void_p]
    L.mq_tandem_last_error.restype = C.c_char_p
    L.mq_tandem_layout.argtypes = [P(mq_tandem_desc), P(C.c_double), P(C.c_double), P(C.c_double)]
    L.mq_tandem_layout.restype = C.c_int32
    L.mq_tandem_inject.argtypes = [P(mq_tandem_desc), C.c_uint64, C.c_int32, P(mq_tracks), C.c_size_t]
    L.mq_tandem_inject.restype = C.c_int32
    L.mq_tandem_advance.argtypes = [C.c_void_p, P(mq_tracks), C.c_size_t, C.c_uint64, C.c_uint64, P(mq_port_counts),
                                    P(mq_tandem_stats)]
    L.mq_tandem_advance.restype = C.c_int32
    L.mq_tandem_frame.argtypes = [P(mq_tracks), C.c_size_t, P(mq_tandem_frame_counts)]
    L.mq_tandem_frame.restype = C.c_int32


def _declare_engine(L) -> None:
    P = C.POINTER
    L.mq_engine_create.argtypes = [P(mq_grid_desc), C.c_int32, C.c_int32, P(C.c_void_p)]
    L.mq_engine_create.restype = C.c_int32
    L.mq_engine_destroy.argtypes = [C.c_void_p]
    L.mq_engine_destroy.restype = None
    L.mq_last_error.argtypes = [C.c_void_p]
    L.mq_last_error.restype = C.c_char_p
    L.mq_engine_set_dc.argtypes = [C.c_void_p, P(C.c_double)]
    L.mq_engine_set_dc.restype = C.c_int32
    L.mq_inject.argtypes = [C.c_void_p, P(mq_job), C.c_size_t, P(mq_physics), P(mq_ions), C.c_size_t]
    L.mq_inject.restype = C.c_int32
    L.mq_inject_grid.argtypes = [P(mq_grid_desc), P(mq_job), C.c_size_t, P(mq_physics), P(mq_ions), C.c_size_t]
    L.mq_inject_grid.restype = C.c_int32
    L.mq_run_ions.argtypes = [C.c_void_p, P(mq_job), C.c_size_t, P(mq_physics), P(mq_ions), C.c_size_t,
                              C.c_uint32, P(mq_run_stats)]
    L.mq_run_ions.restype = C.c_int32
    L.mq_run_batch.argtypes = [C.c_void_p, P(mq_job), C.c_size_t, P(C.c_double), P(mq_physics), P(mq_outcome),
                               P(mq_ions), P(mq_run_stats)]
    L.mq_run_batch.restype = C.c_int32
    L.mq_summarize.argtypes = [P(mq_ions), C.c_size_t, C.c_double, C.c_size_t, P(mq_outcome)]
    L.mq_summarize.restype = C.c_int32
    L.mq_fnv1a64.argtypes = [C.c_void_p, C.c_size_t, C.c_uint64]
    L.mq_fnv1a64.restype = C.c_uint64
    L.mq_device_count.argtypes = []
    L.mq_device_count.restype = C.c_int32
    L.mq_measure_l2_read_gbs.argtypes = [C.c_int32, C.c_size_t, C.c_int32, P(C.c_double)]
    L.mq_measure_l2_read_gbs.restype = C.c_int32
    L.mq_engine_get_tuning.argtypes = [C.c_void_p, P(mq_tuning)]
    L.mq_engine_get_tuning.restype = C.c_int32
    L.mq_engine_set_tuning.argtypes = [C.c_void_p, P(mq_tuning)]
    L.mq_engine_set_tuning.restype = C.c_int32
    L.mq_engine_autotune.argtypes = [C.c_void_p, P(mq_job), C.c_size_t, P(C.c_double), P(mq_physics), C.c_uint64,
                                     P(mq_tuning), P(C.c_double)]
    L.mq_engine_autotune.restype = C.c_int32
    L.mq_engine_inject_fault.argtypes = [C.c_void_p, C.c_int32]
    L.mq_engine_inject_fault.restype = C.c_int32
    L.mq_check_status.argtypes = [C.c_int32, C.c_int32, P(C.c_int32), P(C.c_uint32), P(C.c_uint32), P(C.c_uint64),
                                  P(C.c_uint64)]
    L.mq_check_status.restype = C.c_int32
    L.mq_check_selftest.argtypes = [C.c_int32]
    L.mq_check_selftest.restype = C.c_int32
    L.mq_run_ions_device_noalloc.argtypes = [P(mq_dev_grid), P(mq_job), C.c_size_t, P(mq_physics), P(mq_ions), C.c_size_t,
                                             C.c_uint32, C.c_void_p, P(C.c_uint64)]
    L.mq_run_ions_device_noalloc.restype = C.c_int32


def check(code: int, what: str, eng=None) -> None:
    if code != MQ_OK:
        detail = ""
        if eng is not None:
            try:
                detail = (lib().mq_last_error(eng) or b"").decode()
            except Exception:
                detail = ""
        raise MqError(code, what, detail)
