"""ndtensors_gb300: the NDTensors contraction hot path on GB300 (sm_103a).

Python host mirror of NDTensors' storage / contraction / factorization
interface, calling libndtensors_gb300.so through its C ABI.  No CPU fallback:
every operation runs in the library's CUDA kernels.
"""
from ._lib import NDError, NoConvergence, PRECISIONS, handle, load, LIB_PATH
from .tensors import BlockSparseTensor, DenseTensor, DiagBlockSparseTensor, blockoffsets
from . import workloads
from . import linalg
from . import autodiff
from .autodiff import contract_autograd, contract_rrule, dense_structure
from .linalg import (CombinerTensor, MatricizePlan, Spectrum, SvdPlan, combine, contract_combiner, eigen, eigs,
                     entropy, matricize, qr, svd, truncate, truncerror, uncombine)
from .contract import (ContractionPlan, contract, contract_, contract_blocksparse, contract_labels,
                       get_plan, permutedims, permutedims_, permutedims_blocksparse)
from . import krylov
from .krylov import HeffOperator, Lanczos, SweepStep, lanczos
from . import hdf5io
from .hdf5io import H5Reader, load_blocksparse, read_blocksparse, save_blocksparse, write_blocksparse

__all__ = [
    "workloads", "NDError", "NoConvergence", "PRECISIONS", "handle", "load", "LIB_PATH",
    "BlockSparseTensor", "DenseTensor", "DiagBlockSparseTensor", "blockoffsets",
    "ContractionPlan", "contract", "contract_", "contract_blocksparse", "contract_labels", "get_plan",
    "permutedims", "permutedims_", "permutedims_blocksparse",
    "linalg", "CombinerTensor", "MatricizePlan", "Spectrum", "SvdPlan", "combine", "contract_combiner", "eigen",
    "eigs", "entropy", "matricize", "qr", "svd", "truncate", "truncerror", "uncombine",
    "autodiff", "contract_autograd", "contract_rrule", "dense_structure",
    "krylov", "HeffOperator", "Lanczos", "SweepStep", "lanczos",
    "hdf5io", "H5Reader", "load_blocksparse", "read_blocksparse", "save_blocksparse", "write_blocksparse",
]
