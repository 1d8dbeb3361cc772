"""GB300-native (sm_103a) separation likelihood for Milkyway@Home.

The compute path is libmwsep_gb300.so (hand-written CUDA kernels behind a C
ABI, include/milkyway_separation_gb300.h); this package holds its sources,
its in-tree build and a Python mirror of the reference client's evaluation
interface.
"""
from .native import (MWSEP_MIXED_F32, MWSEP_PLAIN_DF, MWSEP_PLAIN_F64, MwsepError)  # noqa: F401
from .separation import (AstronomyParameters, Context, EvaluationState, Result,  # noqa: F401
                         Server, StarPoints, evaluate, evaluate_df, evaluate_mixed, integral_f, likelihood_f,
                         stripe_transform,
                         write_separation, invert_matrix, errors_from_hessian, write_errors,
                         StarCatalogue)

__all__ = ["AstronomyParameters", "StarPoints", "EvaluationState", "Context", "Result", "Server",
           "evaluate", "evaluate_df", "evaluate_mixed", "integral_f", "likelihood_f", "stripe_transform", "write_separation", "invert_matrix", "errors_from_hessian", "write_errors",
           "StarCatalogue", "MWSEP_PLAIN_F64", "MWSEP_MIXED_F32", "MWSEP_PLAIN_DF", "MwsepError"]
