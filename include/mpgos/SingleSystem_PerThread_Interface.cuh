// Drop-in C++ interface of the GB300 per-thread ensemble solver.
//
// Same names, argument meaning and index layout as the reference's
// SourceCodes/SingleSystem_PerThread_Interface.cuh: enums Algorithms,
// ListOfVariables, ListOfSolverOptions (:33-62), free functions
// ListCUDADevices / SelectDeviceByClosestRevision /
// PrintPropertiesOfSpecificDevice (:67-69), and the class template
// ProblemSolver<NT,SD,NCP,NSP,NISP,NE,NA,NIA,NDO,Algorithm,Precision>
// (:117-208). A user program includes its system definition (the PerThread_*
// hook templates) first and this header second, exactly as with the
// reference, and compiles unchanged:
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -I<repo>/include/mpgos \
//        -I<repo>/include user.cu -L<build> -lmpgos_runtime
//
// Everything below is host code calling the C-ABI of mpgos.h; the kernels are
// the sm_103a templates of csrc/perthread instantiated here for the user's
// hooks and handed to the runtime as a kernel table. Errors print the
// reference-style message and exit(EXIT_FAILURE), as the reference does.
#ifndef SINGLESYSTEM_PERTHREAD_INTERFACE_H
#define SINGLESYSTEM_PERTHREAD_INTERFACE_H

#include <cuda_runtime.h>
#include <stdio.h>

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <typeinfo>
#include <vector>

#include "../mpgos.h"
#include "../../massively-parallel-gpu-ode-solver_gb300/csrc/perthread/kernel.cuh"
#include "dropin_common.h"

enum Algorithms { RK4 = MPGOS_RK4, RKCK45 = MPGOS_RKCK45 };

enum ListOfVariables {
    All = MPGOS_ALL,
    TimeDomain = MPGOS_TIME_DOMAIN,
    ActualState = MPGOS_ACTUAL_STATE,
    ActualTime = MPGOS_ACTUAL_TIME,
    ControlParameters = MPGOS_CONTROL_PARAMETERS,
    SharedParameters = MPGOS_SHARED_PARAMETERS,
    IntegerSharedParameters = MPGOS_INTEGER_SHARED_PARAMETERS,
    Accessories = MPGOS_ACCESSORIES,
    IntegerAccessories = MPGOS_INTEGER_ACCESSORIES,
    DenseOutput = MPGOS_DENSE_OUTPUT,
    DenseIndex = MPGOS_DENSE_INDEX,
    DenseTime = MPGOS_DENSE_TIME,
    DenseState = MPGOS_DENSE_STATE
};

enum ListOfSolverOptions {
    ThreadsPerBlock = MPGOS_THREADS_PER_BLOCK,
    InitialTimeStep = MPGOS_INITIAL_TIME_STEP,
    ActiveNumberOfThreads = MPGOS_ACTIVE_NUMBER_OF_THREADS,
    MaximumTimeStep = MPGOS_MAXIMUM_TIME_STEP,
    MinimumTimeStep = MPGOS_MINIMUM_TIME_STEP,
    TimeStepGrowLimit = MPGOS_TIME_STEP_GROW_LIMIT,
    TimeStepShrinkLimit = MPGOS_TIME_STEP_SHRINK_LIMIT,
    RelativeTolerance = MPGOS_RELATIVE_TOLERANCE,
    AbsoluteTolerance = MPGOS_ABSOLUTE_TOLERANCE,
    EventTolerance = MPGOS_EVENT_TOLERANCE,
    EventDirection = MPGOS_EVENT_DIRECTION,
    DenseOutputMinimumTimeStep = MPGOS_DENSE_OUTPUT_MINIMUM_TIME_STEP,
    DenseOutputSaveFrequency = MPGOS_DENSE_OUTPUT_SAVE_FREQUENCY,
    PreferSharedMemory = MPGOS_PREFER_SHARED_MEMORY
};

inline std::string SolverOptionsToString(ListOfSolverOptions o)
{
    static const char* names[] = {"ThreadsPerBlock", "InitialTimeStep", "ActiveNumberOfThreads", "MaximumTimeStep",
                                  "MinimumTimeStep", "TimeStepGrowLimit", "TimeStepShrinkLimit",
                                  "RelativeTolerance", "AbsoluteTolerance", "EventTolerance", "EventDirection",
                                  "DenseOutputMinimumTimeStep", "DenseOutputSaveFrequency", "PreferSharedMemory"};
    return (o >= 0 && o <= 13) ? names[o] : "Non-existent solver option!";
}

inline std::string VariablesToString(ListOfVariables v)
{
    static const char* names[] = {"All", "TimeDomain", "ActualState", "ActualTime", "ControlParameters",
                                  "SharedParameters", "IntegerSharedParameters", "Accessories",
                                  "IntegerAccessories", "DenseOutput", "DenseIndex", "DenseTime", "DenseState"};
    return (v >= 0 && v <= 12) ? names[v] : "Non-existent variable!";
}

// ---- ProblemSolver (:117-208) ---------------------------------------------------
template <int NT, int SD, int NCP, int NSP, int NISP, int NE, int NA, int NIA, int NDO, Algorithms Algorithm,
          class Precision>
class ProblemSolver {
  public:
    explicit ProblemSolver(int device)
    {
        using Table = mpgos::pt::KernelTable<mpgos::pt::Shape<SD, NCP, NSP, NISP, NE, NA, NIA>,
                                             static_cast<int>(Algorithm), Precision>;
        mpgos::dropin::check(mpgos_pt_create(Table::get("user"), NT, NDO, device, &h_), "ProblemSolver");
        for (int v = 0; v < 64; v++) host_[v] = nullptr;
        const int vars[] = {TimeDomain, ActualState, ActualTime, ControlParameters, SharedParameters,
                            IntegerSharedParameters, Accessories, IntegerAccessories, DenseIndex, DenseTime, DenseState};
        for (int v : vars) mpgos::dropin::check(mpgos_pt_host_buffer(h_, v, &host_[v], nullptr), "ProblemSolver");
    }
    ~ProblemSolver() { mpgos_pt_destroy(h_); }
    ProblemSolver(const ProblemSolver&) = delete;
    ProblemSolver& operator=(const ProblemSolver&) = delete;

    template <typename T> void SolverOption(ListOfSolverOptions option, T value)
    {
        if (option == RelativeTolerance || option == AbsoluteTolerance || option == EventTolerance ||
            option == EventDirection) {
            std::cerr << "ERROR: In solver member function SolverOption!" << std::endl;
            std::cerr << "       Option: " << SolverOptionsToString(option) << std::endl;
            std::cerr << "       This option needs 2 input arguments or not applicable!" << std::endl;
            exit(EXIT_FAILURE);
        }
        mpgos::dropin::check(mpgos_pt_set_option(h_, option, 0, static_cast<double>(value)), "SolverOption");
    }
    template <typename T> void SolverOption(ListOfSolverOptions option, int index, T value)
    {
        const int limit = (option == RelativeTolerance || option == AbsoluteTolerance) ? SD
                          : (option == EventTolerance || option == EventDirection)     ? NE
                                                                                       : -1;
        if (limit < 0) {
            std::cerr << "ERROR: In solver member function SolverOption!" << std::endl;
            std::cerr << "       Option: " << SolverOptionsToString(option) << std::endl;
            std::cerr << "       This option needs 1 input arguments or not applicable!" << std::endl;
            exit(EXIT_FAILURE);
        }
        mpgos::dropin::bound("SolverOption", SolverOptionsToString(option).c_str(), index, 0, limit - 1);
        mpgos::dropin::check(mpgos_pt_set_option(h_, option, index, static_cast<double>(value)), "SolverOption");
    }

    // Unit scope and DenseTime
    template <typename T> void SetHost(int pid, ListOfVariables v, int serial, T value) { ref_unit("SetHost", pid, v, serial, [&](auto& x) { x = static_cast<std::remove_reference_t<decltype(x)>>(value); }); }
    // System scope
    template <typename T> void SetHost(int pid, ListOfVariables v, T value)
    {
        mpgos::dropin::bound("SetHost", "ProblemNumber", pid, 0, NT - 1);
        if (v == ActualTime) {
            static_cast<Precision*>(host_[ActualTime])[pid] = static_cast<Precision>(value);
        } else if (v == DenseIndex) {
            mpgos::dropin::bound("SetHost", "DenseIndex-Value", static_cast<int>(value), 0, NDO - 1);
            static_cast<int*>(host_[DenseIndex])[pid] = static_cast<int>(value);
        } else {
            wrong("SetHost", v);
        }
    }
    // Global scope
    template <typename T> void SetHost(ListOfVariables v, int serial, T value)
    {
        if (v == SharedParameters) {
            mpgos::dropin::bound("SetHost", "SharedParameters", serial, 0, NSP - 1);
            static_cast<Precision*>(host_[SharedParameters])[serial] = static_cast<Precision>(value);
        } else if (v == IntegerSharedParameters) {
            mpgos::dropin::bound("SetHost", "IntegerSharedParameters", serial, 0, NISP - 1);
            static_cast<int*>(host_[IntegerSharedParameters])[serial] = static_cast<int>(value);
        } else {
            wrong("SetHost", v);
        }
    }
    // DenseState
    template <typename T> void SetHost(int pid, ListOfVariables v, int comp, int step, T value)
    {
        dense_state_index("SetHost", pid, v, comp, step);
        static_cast<Precision*>(host_[DenseState])[pid + comp * NT + step * NT * SD] = static_cast<Precision>(value);
    }

    void SynchroniseFromHostToDevice(ListOfVariables v)
    {
        mpgos::dropin::check(mpgos_pt_sync_h2d(h_, v), "SynchroniseFromHostToDevice");
    }
    void SynchroniseFromDeviceToHost(ListOfVariables v)
    {
        mpgos::dropin::check(mpgos_pt_sync_d2h(h_, v), "SynchroniseFromDeviceToHost");
    }

    template <typename T> T GetHost(int pid, ListOfVariables v, int serial)
    {
        T out{};
        ref_unit("GetHost", pid, v, serial, [&](auto& x) { out = static_cast<T>(x); });
        return out;
    }
    template <typename T> T GetHost(int pid, ListOfVariables v)
    {
        mpgos::dropin::bound("GetHost", "ProblemNumber", pid, 0, NT - 1);
        if (v == ActualTime) return static_cast<T>(static_cast<Precision*>(host_[ActualTime])[pid]);
        if (v == DenseIndex) return static_cast<T>(static_cast<int*>(host_[DenseIndex])[pid]);
        wrong("GetHost", v);
        return T{};
    }
    template <typename T> T GetHost(ListOfVariables v, int serial)
    {
        if (v == SharedParameters) {
            mpgos::dropin::bound("GetHost", "SharedParameters", serial, 0, NSP - 1);
            return static_cast<T>(static_cast<Precision*>(host_[SharedParameters])[serial]);
        }
        if (v == IntegerSharedParameters) {
            mpgos::dropin::bound("GetHost", "IntegerSharedParameters", serial, 0, NISP - 1);
            return static_cast<T>(static_cast<int*>(host_[IntegerSharedParameters])[serial]);
        }
        wrong("GetHost", v);
        return T{};
    }
    template <typename T> T GetHost(int pid, ListOfVariables v, int comp, int step)
    {
        dense_state_index("GetHost", pid, v, comp, step);
        return static_cast<T>(static_cast<Precision*>(host_[DenseState])[pid + comp * NT + step * NT * SD]);
    }

    // Print (:1083-1276): same file names and number format.
    void Print(ListOfVariables v)
    {
        namespace pr = mpgos::dropin::print;
        switch (v) {
            case TimeDomain: pr::general("TimeDomainInSolverObject.txt", NT, 2, static_cast<Precision*>(host_[v])); break;
            case ActualState: pr::general("ActualStateInSolverObject.txt", NT, SD, static_cast<Precision*>(host_[v])); break;
            case ActualTime: pr::general("ActualTimeInSolverObject.txt", NT, 1, static_cast<Precision*>(host_[v])); break;
            case ControlParameters: pr::general("ControlParametersInSolverObject.txt", NT, NCP, static_cast<Precision*>(host_[v])); break;
            case SharedParameters: pr::general("SharedParametersInSolverObject.txt", NSP, 1, static_cast<Precision*>(host_[v])); break;
            case IntegerSharedParameters: pr::general("IntegerSharedParametersInSolverObject.txt", NISP, 1, static_cast<int*>(host_[v])); break;
            case Accessories: pr::general("AccessoriesInSolverObject.txt", NT, NA, static_cast<Precision*>(host_[v])); break;
            case IntegerAccessories: pr::general("IntegerAccessoriesInSolverObject.txt", NT, NIA, static_cast<int*>(host_[v])); break;
            default: wrong("Print", v);
        }
    }
    void Print(ListOfVariables v, int tid)
    {
        mpgos::dropin::bound("Print", "Thread", tid, 0, NT - 1);
        if (v != DenseOutput) wrong("Print", v);
        mpgos::dropin::print::perthread_dense(
            "DenseOutput_" + std::to_string(tid) + ".txt", tid, NT, SD, NCP, NSP, NISP, NA, NIA, NDO,
            static_cast<Precision*>(host_[ControlParameters]), static_cast<Precision*>(host_[SharedParameters]),
            static_cast<int*>(host_[IntegerSharedParameters]), static_cast<Precision*>(host_[Accessories]),
            static_cast<int*>(host_[IntegerAccessories]), static_cast<int*>(host_[DenseIndex]),
            static_cast<Precision*>(host_[DenseTime]), static_cast<Precision*>(host_[DenseState]));
    }

    void Solve() { mpgos::dropin::check(mpgos_pt_solve(h_), "Solve"); }
    void SynchroniseDevice() { mpgos::dropin::check(mpgos_pt_sync_device(h_), "SynchroniseDevice"); }
    void InsertSynchronisationPoint() { mpgos::dropin::check(mpgos_pt_insert_sync_point(h_), "InsertSynchronisationPoint"); }
    void SynchroniseSolver() { mpgos::dropin::check(mpgos_pt_sync_solver(h_), "SynchroniseSolver"); }

    // Extensions beyond the reference object.
    mpgos_pt_solver* Handle() { return h_; }
    void SolvePhases(int n) { mpgos::dropin::check(mpgos_pt_solve_phases(h_, n, -1, nullptr), "SolvePhases"); }

  private:
    mpgos_pt_solver* h_ = nullptr;
    void* host_[64];

    [[noreturn]] void wrong(const char* fn, ListOfVariables v)
    {
        std::cerr << "ERROR: In solver member function " << fn << "!" << std::endl;
        std::cerr << "       Option: " << VariablesToString(v) << std::endl;
        std::cerr << "       This option needs different argument configuration or not applicable!" << std::endl;
        exit(EXIT_FAILURE);
    }

    template <class F> void ref_unit(const char* fn, int pid, ListOfVariables v, int serial, F&& f)
    {
        mpgos::dropin::bound(fn, "ProblemNumber", pid, 0, NT - 1);
        const int idx = pid + serial * NT;
        switch (v) {
            case TimeDomain: mpgos::dropin::bound(fn, "TimeDomain", serial, 0, 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case ActualState: mpgos::dropin::bound(fn, "ActualState", serial, 0, SD - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case ControlParameters: mpgos::dropin::bound(fn, "ControlParameters", serial, 0, NCP - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case Accessories: mpgos::dropin::bound(fn, "Accessories", serial, 0, NA - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case IntegerAccessories: mpgos::dropin::bound(fn, "IntegerAccessories", serial, 0, NIA - 1); f(static_cast<int*>(host_[v])[idx]); break;
            case DenseTime: mpgos::dropin::bound(fn, "DenseTime", serial, 0, NDO - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            default: wrong(fn, v);
        }
    }

    void dense_state_index(const char* fn, int pid, ListOfVariables v, int comp, int step)
    {
        mpgos::dropin::bound(fn, "ProblemNumber", pid, 0, NT - 1);
        if (v != DenseState) wrong(fn, v);
        mpgos::dropin::bound(fn, "DenseState/ComponentNumber", comp, 0, SD - 1);
        mpgos::dropin::bound(fn, "DenseState/TimeStepNumber", step, 0, NDO - 1);
    }

};

#endif
