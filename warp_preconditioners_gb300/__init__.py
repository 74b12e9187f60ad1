"""GB300-native preconditioned-Krylov path of warp-preconditioners.

Drop-in counterparts of the reference package's operators (same names,
arguments and error messages), backed by hand-written sm_103a CUDA kernels in
libgbpc.so reached through its C ABI (include/gbpc.h):

    FSAI, SparseOperator, SquaredLaplacianOperator, BlockJacobi, BlockILU0,
    BiharmonicSystem, RepeatedFSAI, BlockFSAI, BsrBlockFSAI, MixedHarmonicSystem,
    MatchingSchur, ShiftedBlock

plus ``linear.cg`` / ``linear.cr`` / ``linear.gmres`` / ``linear.preconditioner`` and the
``sparse`` helpers that stand in for warp.optim.linear and warp.sparse.
Vectors and matrices are torch CUDA tensors.
"""

from . import batched, linear, multi, sparse
from .biharmonic import BiharmonicSystem, RepeatedFSAI
from .block_fsai import BlockFSAI, BsrBlockFSAI
from .block_ilu import BlockILU0, BlockJacobi
from .fsai import FSAI
from .linear import LinearOperator, aslinearoperator, cg, cr, gmres, preconditioner
from .mixed import MatchingSchur, MixedHarmonicSystem, ShiftedBlock
from .sparse import BsrMatrix, bsr_copy, bsr_from_triplets, bsr_transposed, from_scipy
from .sparse_operator import SparseOperator
from .squared_laplacian import SquaredLaplacianOperator

__all__ = [
    "FSAI",
    "BiharmonicSystem",
    "RepeatedFSAI",
    "SparseOperator",
    "SquaredLaplacianOperator",
    "BlockJacobi",
    "BlockILU0",
    "BlockFSAI",
    "BsrBlockFSAI",
    "MixedHarmonicSystem",
    "MatchingSchur",
    "ShiftedBlock",
    "LinearOperator",
    "BsrMatrix",
    "aslinearoperator",
    "bsr_copy",
    "bsr_from_triplets",
    "bsr_transposed",
    "cg",
    "cr",
    "gmres",
    "from_scipy",
    "batched",
    "linear",
    "multi",
    "preconditioner",
    "sparse",
]


def library_path():
    """Path of the loaded libgbpc.so (builds it on first use)."""
    from . import _lib

    _lib.load()
    return str(_lib.LIB_PATH)
