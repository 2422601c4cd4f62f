"""msmodel_gb300 -- GB300-native Foldy-Lax hot path of MSModel.

The compute path is libmsgpu.so (hand-written CUDA for sm_103a behind the C
ABI in include/msgpu.h); this package is the Python host mirror of the
reference's interface over it.
"""
from .api import *  # noqa: F401,F403
from .api import MsgpuError, lib  # noqa: F401

__all__ = [
    "Medium", "fill_medium", "random_doubles", "realisation_sizes", "kplane_args", "kcut_args", "halton_points", "free_green", "dk_free_green",
    "free_green_imag", "bessel_k", "invf", "build_ms_matrix", "build_dk_ms_matrix", "tracelog_lu",
    "tracelog_batch", "dk_log_det_batch", "amplitude_batch", "dk_log_det_ms", "total_cross_section",
    "run_tracelog", "wave_function", "wave_function_batch", "wave_cut", "run_wave_function_cut", "diff_cross_section", "dcs_statistics", "run_differential_cross_section", "solve_aberth_batch", "find_eigenstates", "Job", "init", "random_function", "traceinv_batch", "inverse_iteration_batch", "find_roots_muller", "eigvals_batch", "imag_mu_histogram", "imag_mu_task", "logcut_args", "run_imag_mu_histogram", "chistogram", "run_chistogram", "tune_set", "tune_get", "autotune", "tune_table", "tune_save", "tune_load", "launch_count", "sm_count", "probe_fp64_mma_tflops", "MsgpuError", "lib",
]
