// Kernel-argument types and the Algorithms enum of the reference's coupled
// per-block solver, for building the reference kernel outside its interface
// header.
//
// TEST INFRASTRUCTURE ONLY (used by ref_gpu_coupled_entry.cu).
// CoupledSystems_PerBlock_Interface.cuh:33,80-132 declares these next to its
// host-side class, whose host code does not compile against the CUDA 13
// runtime headers (it reads cudaDeviceProp fields that were removed), so the
// declarations are repeated with the reference's field order and types, which
// the kernel's by-value argument layout depends on.
#pragma once

enum Algorithms { RK4, RKCK45 };

struct Struct_ThreadConfiguration {
    int LogicalThreadsPerBlock;
    int NumberOfBlockLaunches;
    int ThreadPaddingPerBlock;
    int BlockSize;
    int GridSize;
    int TotalLogicalThreads;
};
template <class Precision>
struct Struct_GlobalVariables {
    Precision* d_TimeDomain;
    Precision* d_ActualState;
    Precision* d_ActualTime;
    Precision* d_UnitParameters;
    Precision* d_SystemParameters;
    Precision* d_GlobalParameters;
    int* d_IntegerGlobalParameters;
    Precision* d_UnitAccessories;
    int* d_IntegerUnitAccessories;
    Precision* d_SystemAccessories;
    int* d_IntegerSystemAccessories;
    Precision* d_CouplingMatrix;
    Precision* d_CouplingStrength;
    int* d_CouplingIndex;
    int* d_DenseOutputIndex;
    Precision* d_DenseOutputTimeInstances;
    Precision* d_DenseOutputStates;
    Precision* d_RelativeTolerance;
    Precision* d_AbsoluteTolerance;
    Precision* d_EventTolerance;
    int* d_EventDirection;
};
struct Struct_SharedMemoryUsage {
    bool GlobalVariables;
    bool CouplingMatrices;
    int SingleCouplingMatrixSize;
    int IsAdaptive;
};
template <class Precision>
struct Struct_SolverOptions {
    Precision InitialTimeStep;
    int ActiveSystems;
    Precision MaximumTimeStep;
    Precision MinimumTimeStep;
    Precision TimeStepGrowLimit;
    Precision TimeStepShrinkLimit;
    int DenseOutputSaveFrequency;
    Precision DenseOutputMinimumTimeStep;
};
