"""ctypes binding of libflorence_gb300.so (the C ABI declared in include/florence_gb300.h).

The library is built in-tree by ``florence_gb300.build`` (or ``__graft_entry__.build()``).
There is no fallback: if the library is missing or fails to load, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflorence_gb300.so")

FL_OK = 0
FL_ERR_ARG = 1
FL_ERR_UNSUPPORTED = 2
FL_ERR_CUDA = 3
FL_ERR_MESH = 4
FL_ERR_CAPACITY = 5
FL_FLAG_NONPOSITIVE_J = 1
FL_FLAG_BAD_INDEX = 2
FL_FLAG_TIMEOUT = 4
FL_FLAG_PAIR_RANGE = 8
FL_FLAG_CAPACITY = 16
FL_MATERIAL_NEOHOOKEAN = 1
FL_MATERIAL_MOONEYRIVLIN = 2
FL_MATERIAL_NEARLYINCOMPRESSIBLEMOONEYRIVLIN = 3
FL_MATERIAL_LINEARELASTIC = 10
FL_MATERIAL_ANISOTROPICMOONEYRIVLIN_1 = 11
FL_ARITH_FP64 = 0
FL_ARITH_FLOAT_PAIR = 1
FL_ARITH_TENSOR = 2
FL_ARITH_REFERENCE_TENSOR = 3
FL_PCG_F64 = 64
FL_PCG_F32 = 32
FL_PCG_F64_SPLIT = 6432
FL_NOALLOC_SCRATCH_BYTES = 32 << 20


class FlorenceGB300Error(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _lib.fl_status_string(status).decode() if _lib is not None else str(status)
        super().__init__("%s failed: %s (status %d)" % (what or "florence_gb300", msg, status))


_lib = None

P = ctypes.c_void_p
I64 = ctypes.c_int64
D = ctypes.c_double
INT = ctypes.c_int

_DF_ARGS = [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64, I64, I64, P, P, P, P, P, P, INT, INT, P, P, P, P,
            D, D, D, D, D, D, D, D, D, D, D, P, P, P]


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("florence_gb300 CUDA library not built: %s is missing "
                              "(run `python -m florence_gb300.build` or __graft_entry__.build())" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        L.fl_status_string.argtypes = [INT]
        L.fl_status_string.restype = ctypes.c_char_p
        L.fl_ComputeSparsityPattern_workspace_size.argtypes = [I64, I64, I64]
        L.fl_ComputeSparsityPattern_workspace_size.restype = ctypes.c_size_t
        L.fl_ComputeSparsityPattern.argtypes = [P, I64, I64, I64, I64, P, P, I64, ctypes.POINTER(I64), P, P, P,
                                                ctypes.c_size_t, P]
        L.fl_TetNodeLayout.argtypes = [P, I64, P]
        L.fl_RaiseTetOrder_workspace_size.argtypes = [I64, I64]
        L.fl_RaiseTetOrder_workspace_size.restype = ctypes.c_size_t
        L.fl_RaiseTetOrder.argtypes = [P, I64, P, I64, P, I64, P, I64, ctypes.POINTER(I64), P, P, ctypes.c_size_t, P]
        L.fl_HexNodeLayout.argtypes = [P, I64, P]
        L.fl_RaiseHexOrder_workspace_size.argtypes = [I64, I64]
        L.fl_RaiseHexOrder_workspace_size.restype = ctypes.c_size_t
        L.fl_RaiseHexOrder.argtypes = [P, I64, P, I64, P, I64, P, I64, ctypes.POINTER(I64), P, P, ctypes.c_size_t, P]
        for name in ("fl_GlobalAssemblyDF__NeoHookean_", "fl_GlobalAssemblyDF__MooneyRivlin_",
                     "fl_GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_", "fl_GlobalAssemblyDF__LinearElastic_",
                     "fl_GlobalAssemblyDF__AnisotropicMooneyRivlin_1_"):
            getattr(L, name).argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDF_noalloc.argtypes = [INT] + _DF_ARGS
        L.fl_GlobalAssemblyDF_Blocks.argtypes = [INT, P, P] + _DF_ARGS
        L.fl_ReferenceGeometry.argtypes = [P, P, P, I64, I64, I64, I64, P, P, P]
        L.fl_ElementBlockOffsets.argtypes = [P, I64, I64, I64, P, P, P, P, P]
        L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_101_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_0_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_106_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__IsotropicElectroMechanics_105_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__SteinmannModel_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDPF__Piezoelectric_100_.argtypes = _DF_ARGS
        L.fl_GlobalAssemblyDF_Batched.argtypes = [INT, P, P, P, P, P, I64, I64, I64, I64, I64, P, P, P, P, P, P, P, P,
                                                  P]
        L.fl_SetAssemblyTuning.argtypes = [I64, I64, INT]
        L.fl_SetAssemblyArithmetic.argtypes = [INT]
        L.fl_GetAssemblyArithmetic.argtypes = []
        L.fl_SetTensorCoreTiling.argtypes = [INT, INT]
        L.fl_AssembleExternalTractionForces.argtypes = [P, I64, I64, P, P, P, P, I64, P, P, I64, P, P, P]
        L.fl_AssembleBodyForces.argtypes = [P, I64, I64, P, P, I64, D, I64, P, P, P]
        L.fl_GlobalAssemblyDF_Mixed.argtypes = [INT, P, P, P, P, P, I64, I64, I64, I64, I64, P, P, P, P, P, P, D, D, D,
                                                D, D, P, P, P, P]
        L.fl_GlobalAssemblyExplicit_DF_DPF_.argtypes = [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64, I64, I64, P,
                                                        D, D, D, D, D, D, D, D, D, D, D, P, INT, INT, P, P]
        L.fl_LumpedMass.argtypes = [P, P, P, P, P, I64, I64, I64, I64, I64, I64, D, P, P, P]
        L.fl_ConsistentMass.argtypes = [P, P, P, P, P, I64, I64, I64, I64, I64, I64, D, INT, INT, P, P, I64, P, P, P,
                                        P, P, P, P]
        L.fl_measure_fp64_peak.argtypes = [ctypes.POINTER(D), P]
        L.fl_measure_fp32_peak.argtypes = [ctypes.POINTER(D), P]
        L.fl_TensorCoreSelfTest.argtypes = [P, P, P, P, P]
        L.fl_ReferenceGradients.argtypes = [P, P, P, P, I64, I64, I64, I64, P, P, P, P]
        L.fl_InternalForceF32.argtypes = [P, P, P, P, I64, I64, I64, I64, INT, D, D, P, P, P]
        L.fl_ReferenceGradientsPair.argtypes = [P, P, P, P, I64, I64, I64, I64, P, P, P, P, P]
        L.fl_InternalForcePair.argtypes = [P, P, P, P, P, I64, I64, I64, I64, INT, D, D, P, P, P]
        L.fl_CentralDifferenceUpdate.argtypes = [I64, D, P, INT, P, P, P, P, P, P]
        L.fl_StrainEnergy.argtypes = [P, P, P, P, P, I64, I64, I64, I64, INT, D, D, P, P]
        L.fl_MLP_num_params.argtypes = []
        L.fl_MLP_num_params.restype = I64
        L.fl_MLP_workspace_size.argtypes = [I64]
        L.fl_MLP_workspace_size.restype = ctypes.c_size_t
        L.fl_MLPForward.argtypes = [P, P, I64, P, P, ctypes.c_size_t, P]
        L.fl_MLPGradients.argtypes = [P, P, P, I64, P, P, P, ctypes.c_size_t, P]
        L.fl_MLPAdamStep.argtypes = [P, P, P, P, I64, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     P]
        L.fl_NodalTransfer.argtypes = [I64, P, P, P, P, P, INT, P]
        L.fl_MaskedMatVec.argtypes = [P, P, P, I64, P, P, P, P, P]
        L.fl_MaskedMatVecBlocks.argtypes = [P, P, P, I64, P, P, P, P, P]
        L.fl_MaskedMatVecBlocksF32.argtypes = [P, P, P, I64, P, P, P, P, P]
        L.fl_SplitPairs.argtypes = [I64, P, P, P]
        L.fl_MaskedMatMatBlocksF32.argtypes = [P, P, P, I64, P, P, P, I64, P]
        L.fl_MaskedMatVecBlocksPair.argtypes = [P, P, P, I64, P, P, P, P, P]
        L.fl_BlockJacobiInverse.argtypes = [P, P, P, I64, P, P, P, P]
        L.fl_BlockJacobiApply.argtypes = [I64, P, P, D, P, P, INT, P]
        L.fl_CoarsePCG_workspace_size.argtypes = [I64]
        L.fl_CoarsePCG_workspace_size.restype = ctypes.c_size_t
        L.fl_CoarsePCG.argtypes = [P, P, P, I64, P, P, P, P, D, I64, P, ctypes.c_size_t, P, P, P, P]
        L.fl_SetPCGDeviceLoop.argtypes = [INT]
        L.fl_GetPCGDeviceLoop.argtypes = []
        L.fl_BlockJacobiPCG_workspace_size.argtypes = [I64, I64, INT]
        L.fl_BlockJacobiPCG_workspace_size.restype = ctypes.c_size_t
        L.fl_BlockJacobiPCG.argtypes = [P, P, P, INT, I64, P, P, P, D, I64, P, ctypes.c_size_t,
                                        ctypes.POINTER(I64), ctypes.POINTER(D), P]
        _lib = L
    return _lib


def check(status, what=""):
    if status != FL_OK:
        raise FlorenceGB300Error(status, what)


# every symbol include/florence_gb300.h declares
EXPORTS = ["fl_status_string", "fl_ComputeSparsityPattern_workspace_size", "fl_ComputeSparsityPattern",
           "fl_TetNodeLayout", "fl_RaiseTetOrder_workspace_size", "fl_RaiseTetOrder", "fl_HexNodeLayout",
           "fl_RaiseHexOrder_workspace_size", "fl_RaiseHexOrder",
           "fl_GlobalAssemblyDF__NeoHookean_", "fl_GlobalAssemblyDF__MooneyRivlin_",
           "fl_GlobalAssemblyDF__NearlyIncompressibleMooneyRivlin_", "fl_GlobalAssemblyDF__LinearElastic_",
           "fl_GlobalAssemblyDF__AnisotropicMooneyRivlin_1_", "fl_GlobalAssemblyDF_noalloc",
           "fl_GlobalAssemblyDF_Blocks", "fl_ElementBlockOffsets", "fl_ReferenceGeometry",
           "fl_GlobalAssemblyDPF__IsotropicElectroMechanics_108_", "fl_GlobalAssemblyDPF__IsotropicElectroMechanics_101_",
           "fl_GlobalAssemblyDPF__IsotropicElectroMechanics_0_", "fl_GlobalAssemblyDPF__IsotropicElectroMechanics_106_",
           "fl_GlobalAssemblyDPF__IsotropicElectroMechanics_105_", "fl_GlobalAssemblyDPF__SteinmannModel_",
           "fl_GlobalAssemblyDPF__Piezoelectric_100_",
           "fl_GlobalAssemblyExplicit_DF_DPF_", "fl_LumpedMass", "fl_ConsistentMass", "fl_measure_fp64_peak", "fl_measure_fp32_peak", "fl_TensorCoreSelfTest",
           "fl_BlockJacobiPCG_workspace_size", "fl_BlockJacobiPCG", "fl_SetPCGDeviceLoop", "fl_GetPCGDeviceLoop", "fl_ReferenceGradients", "fl_ReferenceGradientsPair", "fl_InternalForcePair",
           "fl_InternalForceF32", "fl_CentralDifferenceUpdate", "fl_StrainEnergy", "fl_GlobalAssemblyDF_Mixed",
           "fl_GlobalAssemblyDF_Batched", "fl_SetAssemblyTuning", "fl_SetAssemblyArithmetic", "fl_GetAssemblyArithmetic", "fl_SetTensorCoreTiling", "fl_AssembleExternalTractionForces", "fl_AssembleBodyForces", "fl_MLP_num_params", "fl_MLP_workspace_size",
           "fl_MLPForward", "fl_MLPGradients", "fl_MLPAdamStep", "fl_NodalTransfer", "fl_MaskedMatVec", "fl_MaskedMatVecBlocks", "fl_MaskedMatVecBlocksF32", "fl_SplitPairs", "fl_MaskedMatVecBlocksPair", "fl_MaskedMatMatBlocksF32",
           "fl_BlockJacobiInverse", "fl_BlockJacobiApply", "fl_CoarsePCG_workspace_size", "fl_CoarsePCG"]
