"""GB300-native RK3 duct substep of ekman_bl (RK_DUCT + REM_DIV_CURV)."""
from .params import (EkParams, EkMetrics, EkMgStats, Workload, WORKLOADS, default_params,
                     make_grid, ekman_state, workload_setup, spectral_shape)
from .duct import DuctSolver, EkError, load_library, metrics_from_grid
