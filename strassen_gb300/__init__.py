"""strassen_gb300 -- block-sparse GEMM, hybrid Strassen-Winograd recursion and the
RI-K exchange step on GB300 (sm_103a), behind the C ABI of include/bsgpu.h.

Python mirror of the reference's C++ interface (BlockSparseMatrix,
BlockMemoryPool, matmult, matmult_strassen_sparse, the RI-K and 3c->2c
drivers).  Everything runs in libbsgpu.so on the GPU; importing
:mod:`strassen_gb300.api` fails when that library is not built.
"""

__all__ = ["api", "synth"]
