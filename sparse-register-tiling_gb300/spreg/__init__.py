"""spreg -- sparse-register-tiling SpMM for GB300 (sm_103a).

Pack a pruned weight A once (GPU integer kernels, the reference's SOPTile arena layout) and
multiply it by dense B (register-tiled executor kernels).  The public surfaces mirror the
reference: ``sop_driver`` (SOPModule / SOPTile / make_sop_module / execute_tile) and
``matmul.MatMulSpecialized``; both call libspreg.so through its C ABI (include/spreg.h).
"""
from ._lib import BF16, EPILOGUE_NONE, EPILOGUE_RELU, F16, F32, ZERO_PATTERN_ID, SpregError, SpregLibraryMissing
from .mapping import Mapping
from .matmul import MatMulSpecialized, TileConfig
from .packed import PackedMatrix, execute_batched
from .sop_driver import Acc, SOPModule, SOPTile, make_sop_module, pattern_code, sort_and_encode_patterns

__all__ = [
    "Acc", "BF16", "EPILOGUE_NONE", "EPILOGUE_RELU", "F16", "F32", "Mapping", "MatMulSpecialized", "PackedMatrix",
    "SOPModule", "SOPTile", "SpregError", "SpregLibraryMissing", "TileConfig", "ZERO_PATTERN_ID", "execute_batched",
    "make_sop_module", "pattern_code", "sort_and_encode_patterns",
]
