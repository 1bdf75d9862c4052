// Kernel-argument types and the Algorithms enum of the reference's per-thread
// solver, for building the reference kernel outside its interface header.
//
// TEST INFRASTRUCTURE ONLY (shared by ref_cpu_entry.cpp and ref_gpu_entry.cu).
// SingleSystem_PerThread_Interface.cuh:33,72-115 declares these next to its
// host-side class; that header is not compiled here, so the declarations are
// repeated with the reference's field order and types, which the kernel's
// by-value argument layout depends on.
#pragma once

enum Algorithms { RK4, RKCK45 };

struct Struct_ThreadConfiguration {
    int GridSize;
    int BlockSize;
    int NumberOfActiveThreads;
};
template <class Precision>
struct Struct_GlobalVariables {
    Precision* d_TimeDomain;
    Precision* d_ActualState;
    Precision* d_ActualTime;
    Precision* d_ControlParameters;
    Precision* d_SharedParameters;
    int* d_IntegerSharedParameters;
    Precision* d_Accessories;
    int* d_IntegerAccessories;
    Precision* d_RelativeTolerance;
    Precision* d_AbsoluteTolerance;
    Precision* d_EventTolerance;
    int* d_EventDirection;
    int* d_DenseOutputIndex;
    Precision* d_DenseOutputTimeInstances;
    Precision* d_DenseOutputStates;
};
struct Struct_SharedMemoryUsage {
    int PreferSharedMemory;
    int IsAdaptive;
};
template <class Precision>
struct Struct_SolverOptions {
    Precision InitialTimeStep;
    Precision MaximumTimeStep;
    Precision MinimumTimeStep;
    Precision TimeStepGrowLimit;
    Precision TimeStepShrinkLimit;
    int DenseOutputSaveFrequency;
    Precision DenseOutputMinimumTimeStep;
};

