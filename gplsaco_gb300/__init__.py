"""GB300-native Focused-ACO batch engine (drop-in for LinHuanli/GPLSACO's
gp_faco_ext solve path).  All compute runs in the CUDA library built from
gplsaco_gb300/csrc; importing this package does not load it until first use.
"""
from .engine import (CountedState, FacoBatchEngine, FixedFacoGpu, FixedFacoSettings, ant_diagnostic, faco_ants, pheromone_step,
                     program_to_c, score_controller_cuda, score_cuda)
from .session import GpuSession

__all__ = ["CountedState", "FacoBatchEngine", "FixedFacoGpu", "FixedFacoSettings", "GpuSession", "ant_diagnostic", "faco_ants", "pheromone_step",
           "program_to_c", "score_controller_cuda", "score_cuda"]
