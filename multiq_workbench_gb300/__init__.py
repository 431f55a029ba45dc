"""GB300-native batched ion-trajectory engine (drop-in for the chsim batch path of
filiprumenovski/multiq-workbench).  Public API mirrors chsim: ``Geom``, ``Fields``,
``Species``, ``RfAc``, ``Job``, ``Physics``, ``Outcome``, ``Engine.run_batch``; the tandem
router mirrors trapsim: ``TandemModel``, ``CubeGeometry``, ``CubeFields``; ``scan`` holds chsim's
result cache and adaptive scan, ``check`` its batch self-check; ``sweep`` runs excitation-frequency
sweeps of a species mixture as one batch and ``fit`` turns their counts into R = f0 / FWHM (mqviz
``fit_sweep``); ``multiq_workbench_gb300.validate`` compares the engines at the S14 calibrated
point with chsim's own counts (mqviz ``--validate``; also ``python -m`` runnable)."""
from .grid import Geom, Fields, cache_dir, cache_path
from .channel import (Engine, Species, RfAc, Job, JobTable, Physics, Outcome, Outcomes, IonStates, RunStats, MqError, summarize, inject,
                      device_count, PREC_F64, PREC_MIXED, LAUNCH_DISC, LAUNCH_LEGACY, LAUNCH_GAUSSIAN, STATUS,
                      FAULT_NONE, FAULT_LAUNCH_BUDGET, FAULT_ALLOC, FAULT_LAUNCH)
from . import check, scan, fit, sweep
from .tandem import (TandemModel, TandemPreset, TandemSpecies, CubeGeometry, CubeFields, PortGrid, Tracks, PortCounts,
                     Frame, TandemStats, DEFAULT_TONES)

__all__ = ["Geom", "Fields", "cache_dir", "cache_path", "Engine", "Species", "RfAc", "Job", "JobTable", "Physics", "Outcome", "Outcomes",
           "IonStates", "RunStats", "MqError", "summarize", "inject", "device_count", "PREC_F64", "PREC_MIXED", "LAUNCH_DISC",
           "LAUNCH_LEGACY", "LAUNCH_GAUSSIAN", "STATUS", "FAULT_NONE", "FAULT_LAUNCH_BUDGET", "FAULT_ALLOC", "FAULT_LAUNCH", "TandemModel", "TandemPreset", "TandemSpecies", "CubeGeometry",
           "CubeFields", "PortGrid", "Tracks", "PortCounts", "Frame", "TandemStats", "DEFAULT_TONES"]
