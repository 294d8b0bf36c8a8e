"""edgpu -- GB300 (sm_103a) implementation of ExactDiagonalization.jl's sector basis, symmetry
reduction and matrix-free (reduced) Hamiltonian application, behind the reference's API.

The compute path is libedgpu.so (hand-written CUDA); this package is the host-side mirror of the
reference's interface over its C ABI (include/edgpu.h).
"""
from ._lib import (ArgumentError, BoundsError, CudaError, DimensionMismatch, FP64, MIXED, device_count, lib)
from .hilbert import (HilbertSpace, HilbertSpaceSector, Site, State, basespace, bitwidth,
                      quantum_number_sectors)
from .operators import (NullOperator, PureOperator, SumOperator, pauli_matrix, pure_operator, simplify,
                        spin_half_system, term_arrays)
from .representation import (Batch, DirectProductOperation, GlobalBitFlip, HilbertSpaceRepresentation,
                             OperatorRepresentation, ReducedHilbertSpaceRepresentation, SitePermutation,
                             apply_, coupling_grad, dimension, mul_, mul_adjoint_, random_state, represent, search_stats,
                             symmetry_apply, symmetry_reduce, symmetry_unreduce, translation_symops)
from .lanczos import LanczosResult, lanczos, set_krylov_limit
from .autograd import apply_hamiltonian

lib()   # fail loudly at import when libedgpu.so is missing
