"""siml_gb300 — GB300-native (sm_103a) LINGO multiset-Tanimoto engine with
pySIML's GPU API (GPULingo, the SMILES compiler and rowHistogram101).

The compute path is the native library ``libsiml_gb300.so`` (CUDA kernels
behind a C ABI, include/siml_gb300.h); there is no CPU fallback.
"""
from .GPULingo import GPULingo
from .compiler import SMILEStoMatrices, SMILEStoMultiset, cSMILEStoMatrices, preprocessNumbers

__version__ = "1.5.gb300.0"
__all__ = ["GPULingo", "cSMILEStoMatrices", "SMILEStoMatrices", "SMILEStoMultiset", "preprocessNumbers"]
