"""lss -- GB300-native locally-stiff linear solver (Python side).

The solver itself is ``liblss.so`` (hand-written sm_103a CUDA + C++ host
library + the C ABI of include/lss.h); this package loads it, mirrors the
reference's linear-solver interface (``lss.Solver``), builds it in-tree
(``lss.build``) and generates the synthetic workloads (``lss.gen``).
"""
from .solver import (BATCH_RHS, Batch, LssError, Solver, factorize_batched_device, load,  # noqa: F401
                     partition_pattern, row_l1_norms, select_bad_dofs, solve_batched_device,
                     stiff_elimination_tree, postprocess_selection, coarse_space,
                     stiff_elimination_plan)

__all__ = ["Solver", "LssError", "load", "row_l1_norms", "solve_batched_device", "factorize_batched_device",
           "select_bad_dofs", "partition_pattern", "stiff_elimination_tree", "postprocess_selection", "coarse_space", "stiff_elimination_plan", "Batch",
           "BATCH_RHS"]
