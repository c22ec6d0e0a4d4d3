"""GB300-native simulated-bifurcation Ising solver (drop-in for strongshih/Annealing SB/CUDA_GPU).

The solver (SB, plus the reference's SQA and NMFA annealers) is the C ABI in include/sb.h,
implemented by annealing_gb300/libsbsolve.so (CUDA kernels for sm_103a + C++ host code). This package holds the ctypes binding (sb.py), the in-tree
build (_build.py) and the synthetic instance generators (instances.py).
"""
from .sb import (ASB, BSB, DSB, Batch, FIELD_AUTO, FIELD_FP32, FIELD_TC, INIT_REFERENCE, INIT_UNIFORM,
                 OPERAND_AUTO, OPERAND_BF16, OPERAND_BF16X2, OPERAND_FP4, OPERAND_FP6, OPERAND_FP8, OPERAND_FP16X2,
                 Context,
                 NmfaParams,
                 NmfaResult, Params, Plan, Problem, Result, SBError, SQA_RNG_HASH, SQA_RNG_REFERENCE, SqaParams,
                 SqaResult, lib, nmfa_schedule, pump, result_time_to_target, sqa_schedule, success_threshold,
                 time_to_target)

__all__ = ["ASB", "BSB", "DSB", "Batch", "FIELD_AUTO", "FIELD_FP32", "FIELD_TC", "INIT_REFERENCE",
           "INIT_UNIFORM", "OPERAND_AUTO", "OPERAND_BF16", "OPERAND_BF16X2", "OPERAND_FP4", "OPERAND_FP6", "OPERAND_FP8",
           "OPERAND_FP16X2", "Context",
           "NmfaParams", "NmfaResult", "nmfa_schedule", "Params", "Plan", "Problem", "Result", "SBError", "lib",
           "pump", "result_time_to_target", "SQA_RNG_HASH", "SQA_RNG_REFERENCE", "SqaParams", "SqaResult",
           "sqa_schedule", "success_threshold", "time_to_target"]
