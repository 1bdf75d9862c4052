// Drop-in C++ interface of the GB300 coupled per-block solver.
//
// Same names, argument meaning and index layout as the reference's
// SourceCodes/CoupledSystems_PerBlock_Interface.cuh: enums Algorithms,
// ListOfVariables, ListOfSolverOptions (:33-66), free functions
// ListCUDADevices / SelectDeviceByClosestRevision /
// PrintPropertiesOfSpecificDevice (:73-75), and the class template
// ProblemSolver<NS,UPS,UD,TPB,SPB,NC,CBW,CCI,NUP,NSP,NGP,NiGP,NUA,NiUA,NSA,NiSA,NE,NDO,Algorithm,Precision>
// (:135-248) with its six SetHost / GetHost overloads, SolverOption,
// Synchronise*, Print and Solve. A user program includes its system definition
// (the CoupledSystems_PerBlock_* hook templates) first and this header second,
// exactly as with the reference, and compiles unchanged:
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -I<repo>/include/mpgos \
//        -I<repo>/include user.cu -L<build> -lmpgos_runtime
//
// TPB and SPB (threads and systems per block of the reference's four kernel
// variants) are accepted and ignored: one warp integrates one system here
// (csrc/coupled/coupled_kernel.cuh), so there is no thread padding and the
// unit-scope index of (system s, unit u) is s*UPS + u for every TPB/SPB.
// Errors print the reference-style message and exit(EXIT_FAILURE), as the
// reference does.
#ifndef COUPLEDSYSTEMS_PERBLOCK_INTERFACE_H
#define COUPLEDSYSTEMS_PERBLOCK_INTERFACE_H

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
#include "../../massively-parallel-gpu-ode-solver_gb300/csrc/coupled/coupled_kernel.cuh"
#include "dropin_common.h"

enum Algorithms { RK4 = MPGOS_RK4, RKCK45 = MPGOS_RKCK45 };

enum ListOfVariables {
    All = MPGOS_CB_ALL,
    TimeDomain = MPGOS_CB_TIME_DOMAIN,
    ActualTime = MPGOS_CB_ACTUAL_TIME,
    ActualState = MPGOS_CB_ACTUAL_STATE,
    UnitParameters = MPGOS_CB_UNIT_PARAMETERS,
    SystemParameters = MPGOS_CB_SYSTEM_PARAMETERS,
    GlobalParameters = MPGOS_CB_GLOBAL_PARAMETERS,
    IntegerGlobalParameters = MPGOS_CB_INTEGER_GLOBAL_PARAMETERS,
    UnitAccessories = MPGOS_CB_UNIT_ACCESSORIES,
    IntegerUnitAccessories = MPGOS_CB_INTEGER_UNIT_ACCESSORIES,
    SystemAccessories = MPGOS_CB_SYSTEM_ACCESSORIES,
    IntegerSystemAccessories = MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES,
    CouplingMatrix = MPGOS_CB_COUPLING_MATRIX,
    CouplingStrength = MPGOS_CB_COUPLING_STRENGTH,
    CouplingIndex = MPGOS_CB_COUPLING_INDEX,
    DenseOutput = MPGOS_CB_DENSE_OUTPUT,
    DenseIndex = MPGOS_CB_DENSE_INDEX,
    DenseTime = MPGOS_CB_DENSE_TIME,
    DenseState = MPGOS_CB_DENSE_STATE
};

enum ListOfSolverOptions {
    InitialTimeStep = MPGOS_CB_INITIAL_TIME_STEP,
    ActiveSystems = MPGOS_CB_ACTIVE_SYSTEMS,
    MaximumTimeStep = MPGOS_CB_MAXIMUM_TIME_STEP,
    MinimumTimeStep = MPGOS_CB_MINIMUM_TIME_STEP,
    TimeStepGrowLimit = MPGOS_CB_TIME_STEP_GROW_LIMIT,
    TimeStepShrinkLimit = MPGOS_CB_TIME_STEP_SHRINK_LIMIT,
    RelativeTolerance = MPGOS_CB_RELATIVE_TOLERANCE,
    AbsoluteTolerance = MPGOS_CB_ABSOLUTE_TOLERANCE,
    EventTolerance = MPGOS_CB_EVENT_TOLERANCE,
    EventDirection = MPGOS_CB_EVENT_DIRECTION,
    DenseOutputSaveFrequency = MPGOS_CB_DENSE_OUTPUT_SAVE_FREQUENCY,
    DenseOutputMinimumTimeStep = MPGOS_CB_DENSE_OUTPUT_MINIMUM_TIME_STEP,
    SharedGlobalVariables = MPGOS_CB_SHARED_GLOBAL_VARIABLES,
    SharedCouplingMatrices = MPGOS_CB_SHARED_COUPLING_MATRICES
};

inline std::string SolverOptionsToString(ListOfSolverOptions o)
{
    static const char* names[] = {"InitialTimeStep", "ActiveSystems", "MaximumTimeStep", "MinimumTimeStep",
                                  "TimeStepGrowLimit", "TimeStepShrinkLimit", "RelativeTolerance",
                                  "AbsoluteTolerance", "EventTolerance", "EventDirection",
                                  "DenseOutputSaveFrequency", "DenseOutputMinimumTimeStep", "SharedGlobalVariables",
                                  "SharedCouplingMatrices"};
    return (o >= 0 && o <= 13) ? names[o] : "Non-existent solver option!";
}

inline std::string VariablesToString(ListOfVariables v)
{
    static const char* names[] = {"All", "TimeDomain", "ActualTime", "ActualState", "UnitParameters",
                                  "SystemParameters", "GlobalParameters", "IntegerGlobalParameters",
                                  "UnitAccessories", "IntegerUnitAccessories", "SystemAccessories",
                                  "IntegerSystemAccessories", "CouplingMatrix", "CouplingStrength", "CouplingIndex",
                                  "DenseOutput", "DenseIndex", "DenseTime", "DenseState"};
    return (v >= 0 && v <= 18) ? names[v] : "Non-existent variable!";
}

// ---- ProblemSolver (:135-248) -------------------------------------------------------
template <int NS, int UPS, int UD, int TPB, int SPB, int NC, int CBW, int CCI, int NUP, int NSP, int NGP, int NiGP,
          int NUA, int NiUA, int NSA, int NiSA, int NE, int NDO, Algorithms Algorithm, class Precision>
class ProblemSolver {
    using Shape = mpgos::cb::Shape<UPS, UD, NC, CBW, CCI, NUP, NSP, NGP, NiGP, NUA, NiUA, NSA, NiSA, NE>;
    static constexpr int NU = NS * UPS;
    static constexpr int MAT = Shape::MAT;

  public:
    explicit ProblemSolver(int device)
    {
        using Table = mpgos::cb::KernelTable<Shape, static_cast<int>(Algorithm), Precision>;
        mpgos::dropin::check(mpgos_cb_create(Table::get("user"), NS, NDO, device, &h_), "ProblemSolver");
        for (int v = 0; v < 40; v++) host_[v] = nullptr;
        for (int v = MPGOS_CB_TIME_DOMAIN; v <= MPGOS_CB_DENSE_STATE; v++)
            if (v != MPGOS_CB_DENSE_OUTPUT)
                mpgos::dropin::check(mpgos_cb_host_buffer(h_, v, &host_[v], nullptr), "ProblemSolver");
        full_.assign(static_cast<size_t>(NC) * UPS * UPS, Precision(0));
        // the reference keeps a circular coupling matrix in shared memory
        // (:524-527); here every storage is staged per CTA by default
        mpgos::dropin::check(mpgos_cb_set_option(h_, MPGOS_CB_SHARED_COUPLING_MATRICES, 0, 1.0), "ProblemSolver");
    }
    ~ProblemSolver() { mpgos_cb_destroy(h_); }
    ProblemSolver(const ProblemSolver&) = delete;
    ProblemSolver& operator=(const ProblemSolver&) = delete;

    // SolverOption (:760-860)
    template <typename T> void SolverOption(ListOfSolverOptions option, T value)
    {
        if (option == RelativeTolerance || option == AbsoluteTolerance || option == EventTolerance ||
            option == EventDirection) {
            std::cerr << "ERROR: In solver member function SolverOption!" << std::endl;
            std::cerr << "       Option: " << SolverOptionsToString(option) << std::endl;
            std::cerr << "       This option needs 2 input arguments or not applicable!" << std::endl;
            exit(EXIT_FAILURE);
        }
        mpgos::dropin::check(mpgos_cb_set_option(h_, option, 0, static_cast<double>(value)), "SolverOption");
    }
    template <typename T> void SolverOption(ListOfSolverOptions option, int index, T value)
    {
        const int limit = (option == RelativeTolerance || option == AbsoluteTolerance) ? UD
                          : (option == EventTolerance || option == EventDirection)     ? NE
                                                                                       : -1;
        if (limit < 0) {
            std::cerr << "ERROR: In solver member function SolverOption!" << std::endl;
            std::cerr << "       Option: " << SolverOptionsToString(option) << std::endl;
            std::cerr << "       This option needs 1 input arguments or not applicable!" << std::endl;
            exit(EXIT_FAILURE);
        }
        mpgos::dropin::bound("SolverOption", SolverOptionsToString(option).c_str(), index, 0, limit - 1);
        mpgos::dropin::check(mpgos_cb_set_option(h_, option, index, static_cast<double>(value)), "SolverOption");
    }

    // ---- SetHost (:870-1145) -----------------------------------------------------
    // Unit scope
    template <typename T> void SetHost(int sid, int uid, ListOfVariables v, int serial, T value)
    {
        unit("SetHost", sid, uid, v, serial, [&](auto& x) { x = static_cast<std::remove_reference_t<decltype(x)>>(value); });
    }
    // System scope and dense time
    template <typename T> void SetHost(int sid, ListOfVariables v, int serial, T value)
    {
        system("SetHost", sid, v, serial, [&](auto& x) { x = static_cast<std::remove_reference_t<decltype(x)>>(value); });
    }
    // Global scope
    template <typename T> void SetHost(ListOfVariables v, int serial, T value)
    {
        global("SetHost", v, serial, [&](auto& x) { x = static_cast<std::remove_reference_t<decltype(x)>>(value); });
    }
    // Coupling matrix: full (row, col) form, stored as the plugin's storage holds it (:993-1080)
    template <typename T> void SetHost(int coupling, ListOfVariables v, int row, int col, T value)
    {
        const int idx = matrix_slot("SetHost", coupling, v, row, col);
        full_[static_cast<size_t>(row) + static_cast<size_t>(col) * UPS + static_cast<size_t>(coupling) * UPS * UPS] =
            static_cast<Precision>(value);
        static_cast<Precision*>(host_[CouplingMatrix])[idx] = static_cast<Precision>(value);
    }
    // Dense index and actual time
    template <typename T> void SetHost(int sid, ListOfVariables v, T value)
    {
        mpgos::dropin::bound("SetHost", "SystemNumber", sid, 0, NS - 1);
        if (v == ActualTime)
            static_cast<Precision*>(host_[ActualTime])[sid] = static_cast<Precision>(value);
        else if (v == DenseIndex)
            static_cast<int*>(host_[DenseIndex])[sid] = static_cast<int>(value);
        else
            wrong("SetHost", v);
    }
    // Dense state
    template <typename T> void SetHost(int sid, int uid, ListOfVariables v, int comp, int slot, T value)
    {
        static_cast<Precision*>(host_[DenseState])[dense_state("SetHost", sid, uid, v, comp, slot)] =
            static_cast<Precision>(value);
    }

    void SynchroniseFromHostToDevice(ListOfVariables v)
    {
        mpgos::dropin::check(mpgos_cb_sync_h2d(h_, v), "SynchroniseFromHostToDevice");
    }
    void SynchroniseFromDeviceToHost(ListOfVariables v)
    {
        mpgos::dropin::check(mpgos_cb_sync_d2h(h_, v), "SynchroniseFromDeviceToHost");
    }

    // ---- GetHost (:1280-1530) -----------------------------------------------------
    template <typename T> T GetHost(int sid, int uid, ListOfVariables v, int serial)
    {
        T out{};
        unit("GetHost", sid, uid, v, serial, [&](auto& x) { out = static_cast<T>(x); });
        return out;
    }
    template <typename T> T GetHost(int sid, ListOfVariables v, int serial)
    {
        T out{};
        system("GetHost", sid, v, serial, [&](auto& x) { out = static_cast<T>(x); });
        return out;
    }
    template <typename T> T GetHost(ListOfVariables v, int serial)
    {
        T out{};
        global("GetHost", v, serial, [&](auto& x) { out = static_cast<T>(x); });
        return out;
    }
    template <typename T> T GetHost(int coupling, ListOfVariables v, int row, int col)
    {
        matrix_slot("GetHost", coupling, v, row, col);
        return static_cast<T>(
            full_[static_cast<size_t>(row) + static_cast<size_t>(col) * UPS + static_cast<size_t>(coupling) * UPS * UPS]);
    }
    template <typename T> T GetHost(int sid, ListOfVariables v)
    {
        mpgos::dropin::bound("GetHost", "SystemNumber", sid, 0, NS - 1);
        if (v == ActualTime) return static_cast<T>(static_cast<Precision*>(host_[ActualTime])[sid]);
        if (v == DenseIndex) return static_cast<T>(static_cast<int*>(host_[DenseIndex])[sid]);
        wrong("GetHost", v);
        return T{};
    }
    template <typename T> T GetHost(int sid, int uid, ListOfVariables v, int comp, int slot)
    {
        return static_cast<T>(static_cast<Precision*>(host_[DenseState])[dense_state("GetHost", sid, uid, v, comp, slot)]);
    }

    // ---- Print (:1808-1945): same file names and number format; unit-scope
    // files in the reference's padded logical-thread rows for this TPB/SPB ----
    void Print(ListOfVariables v)
    {
        namespace pr = mpgos::dropin::print;
        auto P_ = [&](ListOfVariables x) { return static_cast<Precision*>(host_[x]); };
        auto I_ = [&](ListOfVariables x) { return static_cast<int*>(host_[x]); };
        switch (v) {
            case TimeDomain: pr::system_scope("TimeDomainInSolverObject.txt", NS, 2, P_(v)); break;
            case ActualTime: pr::system_scope("ActualTimeInSolverObject.txt", NS, 1, P_(v)); break;
            case ActualState: pr::unit_scope("ActualStateInSolverObject.txt", UD, P_(v), NS, UPS, TPB, SPB); break;
            case UnitParameters: pr::unit_scope("UnitParametersInSolverObject.txt", NUP, P_(v), NS, UPS, TPB, SPB); break;
            case SystemParameters: pr::system_scope("SystemParametersInSolverObject.txt", NS, NSP, P_(v)); break;
            case GlobalParameters: pr::system_scope("GlobalParametersInSolverObject.txt", NGP, 1, P_(v)); break;
            case IntegerGlobalParameters: pr::system_scope("IntegerGlobalParametersInSolverObject.txt", NiGP, 1, I_(v)); break;
            case UnitAccessories: pr::unit_scope("UnitAccessoriesInSolverObject.txt", NUA, P_(v), NS, UPS, TPB, SPB); break;
            case IntegerUnitAccessories: pr::unit_scope("IntegerUnitAccessoriesInSolverObject.txt", NiUA, I_(v), NS, UPS, TPB, SPB); break;
            case SystemAccessories: pr::system_scope("SystemAccessoriesInSolverObject.txt", NS, NSA, P_(v)); break;
            case IntegerSystemAccessories: pr::system_scope("IntegerSystemAccessoriesInSolverObject.txt", NS, NiSA, I_(v)); break;
            case CouplingStrength: pr::system_scope("CouplingStrengthInSolverObject.txt", NS, NC, P_(v)); break;
            case CouplingIndex: pr::system_scope("CouplingIndexInSolverObject.txt", NC, 1, I_(v)); break;
            default: wrong("Print", v);
        }
    }
    void Print(ListOfVariables v, int serial)
    {
        if (v == CouplingMatrix) {
            mpgos::dropin::bound("Print", "CouplingMatrix", serial, 0, NC - 1);
            mpgos::dropin::print::system_scope("CouplingMatrixInSolverObject_" + std::to_string(serial) + ".txt", UPS,
                                               UPS, full_.data() + static_cast<size_t>(serial) * UPS * UPS);
        } else if (v == DenseOutput) {
            mpgos::dropin::bound("Print", "DenseOutput", serial, 0, NS - 1);
            mpgos::dropin::print::coupled_dense(
                "DenseOutput_" + std::to_string(serial) + ".txt", serial, NS, UPS, UD, NUP, NUA, NiUA, NSP, NSA, NiSA,
                NGP, NiGP, NDO, static_cast<Precision*>(host_[UnitParameters]),
                static_cast<Precision*>(host_[UnitAccessories]), static_cast<int*>(host_[IntegerUnitAccessories]),
                static_cast<Precision*>(host_[SystemParameters]), static_cast<Precision*>(host_[SystemAccessories]),
                static_cast<int*>(host_[IntegerSystemAccessories]), static_cast<Precision*>(host_[GlobalParameters]),
                static_cast<int*>(host_[IntegerGlobalParameters]), static_cast<int*>(host_[DenseIndex]),
                static_cast<Precision*>(host_[DenseTime]), static_cast<Precision*>(host_[DenseState]));
        } else {
            wrong("Print", v);
        }
    }

    void Solve() { mpgos::dropin::check(mpgos_cb_solve(h_), "Solve"); }
    void SynchroniseDevice()
    {
        InsertSynchronisationPoint();
        SynchroniseSolver();
    }
    void InsertSynchronisationPoint() { mpgos::dropin::check(mpgos_cb_insert_sync_point(h_), "InsertSynchronisationPoint"); }
    void SynchroniseSolver() { mpgos::dropin::check(mpgos_cb_sync_solver(h_), "SynchroniseSolver"); }

    // Extension beyond the reference object.
    mpgos_cb_solver* Handle() { return h_; }

  private:
    mpgos_cb_solver* h_ = nullptr;
    void* host_[40];
    std::vector<Precision> full_;  // full coupling matrices [NC][UPS x UPS] column-major, host only

    [[noreturn]] void wrong(const char* fn, ListOfVariables v)
    {
        std::cerr << "ERROR: In solver member function " << fn << "!" << std::endl;
        std::cerr << "       Option: " << VariablesToString(v) << std::endl;
        std::cerr << "       This option needs different argument configuration or not applicable!" << std::endl;
        exit(EXIT_FAILURE);
    }

    template <class F> void unit(const char* fn, int sid, int uid, ListOfVariables v, int serial, F&& f)
    {
        mpgos::dropin::bound(fn, "SystemNumber", sid, 0, NS - 1);
        mpgos::dropin::bound(fn, "UnitNumber", uid, 0, UPS - 1);
        const size_t idx = static_cast<size_t>(sid) * UPS + uid + static_cast<size_t>(serial) * NU;
        switch (v) {
            case ActualState: mpgos::dropin::bound(fn, "ActualState", serial, 0, UD - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case UnitParameters: mpgos::dropin::bound(fn, "UnitParameters", serial, 0, NUP - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case UnitAccessories: mpgos::dropin::bound(fn, "UnitAccessories", serial, 0, NUA - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case IntegerUnitAccessories: mpgos::dropin::bound(fn, "IntegerUnitAccessories", serial, 0, NiUA - 1); f(static_cast<int*>(host_[v])[idx]); break;
            default: wrong(fn, v);
        }
    }

    template <class F> void system(const char* fn, int sid, ListOfVariables v, int serial, F&& f)
    {
        mpgos::dropin::bound(fn, "SystemNumber", sid, 0, NS - 1);
        const size_t idx = static_cast<size_t>(sid) + static_cast<size_t>(serial) * NS;
        switch (v) {
            case TimeDomain: mpgos::dropin::bound(fn, "TimeDomain", serial, 0, 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case SystemParameters: mpgos::dropin::bound(fn, "SystemParameters", serial, 0, NSP - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case SystemAccessories: mpgos::dropin::bound(fn, "SystemAccessories", serial, 0, NSA - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case IntegerSystemAccessories: mpgos::dropin::bound(fn, "IntegerSystemAccessories", serial, 0, NiSA - 1); f(static_cast<int*>(host_[v])[idx]); break;
            case CouplingStrength: mpgos::dropin::bound(fn, "CouplingStrength", serial, 0, NC - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            case DenseTime: mpgos::dropin::bound(fn, "DenseTime", serial, 0, NDO - 1); f(static_cast<Precision*>(host_[v])[idx]); break;
            default: wrong(fn, v);
        }
    }

    template <class F> void global(const char* fn, ListOfVariables v, int serial, F&& f)
    {
        switch (v) {
            case GlobalParameters: mpgos::dropin::bound(fn, "GlobalParameters", serial, 0, NGP - 1); f(static_cast<Precision*>(host_[v])[serial]); break;
            case IntegerGlobalParameters: mpgos::dropin::bound(fn, "IntegerGlobalParameters", serial, 0, NiGP - 1); f(static_cast<int*>(host_[v])[serial]); break;
            case CouplingIndex: mpgos::dropin::bound(fn, "CouplingIndex", serial, 0, NC - 1); f(static_cast<int*>(host_[v])[serial]); break;
            default: wrong(fn, v);
        }
    }

    // index of (row, col) of coupling matrix `coupling` in the stored form
    int matrix_slot(const char* fn, int coupling, ListOfVariables v, int row, int col)
    {
        if (v != CouplingMatrix) wrong(fn, v);
        mpgos::dropin::bound(fn, "CouplingNumber", coupling, 0, NC - 1);
        mpgos::dropin::bound(fn, "Coupling Matrix Row", row, 0, UPS - 1);
        mpgos::dropin::bound(fn, "Coupling Matrix Col", col, 0, UPS - 1);
        if (CCI == 0 && CBW == 0) return row + col * UPS + coupling * UPS * UPS;
        int mcol = col - row + CBW;
        if (mcol >= UPS) mcol -= UPS;
        if (mcol < 0) mcol += UPS;
        const int width = (CBW > 0) ? 2 * CBW + 1 : UPS;
        mpgos::dropin::bound(fn, "Coupling Matrix Shifted Diagonal", mcol, 0, width - 1);
        return (CCI == 0) ? row + mcol * UPS + coupling * UPS * width : mcol + coupling * width;
    }

    size_t dense_state(const char* fn, int sid, int uid, ListOfVariables v, int comp, int slot)
    {
        if (v != DenseState) wrong(fn, v);
        mpgos::dropin::bound(fn, "SystemNumber", sid, 0, NS - 1);
        mpgos::dropin::bound(fn, "UnitNumber", uid, 0, UPS - 1);
        mpgos::dropin::bound(fn, "ComponentNumber in dense state", comp, 0, UD - 1);
        mpgos::dropin::bound(fn, "DenseState", slot, 0, NDO - 1);
        return static_cast<size_t>(sid) * UPS + uid + static_cast<size_t>(comp) * NU + static_cast<size_t>(slot) * NU * UD;
    }
};

#endif
