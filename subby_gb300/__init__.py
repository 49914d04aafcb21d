"""subby_gb300 — GB300-native (sm_103a) backend for subby's eigensubstitution
hot path: Felsenstein inside pass, outside pass, eigenbasis J(t) count
accumulation (general and F81/JC fast path), per-column LogLike, Counts and
root posteriors, per-branch counts, node and branch posteriors, distance
gradients, irreversible and batched models.  Drop-in for ``subby.jax``'s
entry points (same names, arguments and output layouts), with subby's
front-end (``formats``, ``io``, the command line, ``maf_batch``) on top.
"""
from .types import Tree, DiagModel, IrrevDiagModel, RateModel, AnyDiagModel, AnyModel
from .models import (hky85_diag, jukes_cantor_model, f81_model, diagonalize_rate_matrix,
                     reversible_rate_matrix, random_reversible, irrev_model_from_rate_matrix,
                     diagonalize_irreversible, gamma_rate_categories, scale_model, gy94_model,
                     check_detailed_balance, model_from_rate_matrix, diagonalize_rate_matrix_auto, compute_J,
                     compute_J_complex, compute_J_per_row, compute_J_per_row_complex, compute_sub_matrices,
                     compute_sub_matrices_irrev)
from .api import (LogLike, Counts, BranchCounts, RootProb, MixturePosterior, LogLikeCustomGrad, InsideOutside, Plan,
                  get_plan, clear_plan_cache)
from .padding import GEOM_BINS, pad_to_geom_bin, pad_alignment, pad_tree, pad_tree_and_alignment, unpad_columns
from .ctmc import ExpectedCounts, expected_counts_eigen, expected_counts_eigen_irrev
from . import _lib, formats, io, maf_batch

__all__ = ["BranchCounts", "Tree", "DiagModel", "IrrevDiagModel", "RateModel", "irrev_model_from_rate_matrix",
           "diagonalize_irreversible", "gamma_rate_categories", "scale_model", "gy94_model", "MixturePosterior", "hky85_diag", "jukes_cantor_model", "f81_model",
           "diagonalize_rate_matrix", "reversible_rate_matrix", "random_reversible", "LogLike",
           "Counts", "RootProb", "LogLikeCustomGrad", "InsideOutside", "Plan", "get_plan", "clear_plan_cache",
           "ExpectedCounts", "expected_counts_eigen", "expected_counts_eigen_irrev", "AnyDiagModel", "AnyModel",
           "check_detailed_balance", "model_from_rate_matrix", "diagonalize_rate_matrix_auto", "compute_J",
           "compute_J_complex", "compute_J_per_row", "compute_J_per_row_complex", "compute_sub_matrices",
           "compute_sub_matrices_irrev", "GEOM_BINS", "pad_to_geom_bin", "pad_alignment", "pad_tree", "pad_tree_and_alignment", "unpad_columns"]

__version__ = "0.1.0"


def library_path() -> str:
    return _lib.library_path()
