// Host build of the reference's own text writers of the per-thread solver
// (ProblemSolver::WriteToFileGeneral and both Print overloads,
// SourceCodes/SingleSystem_PerThread_Interface.cuh:1083-1276), used to check
// that the drop-in writers (include/mpgos/dropin_print.h) produce the same
// bytes.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_oracle.py copies those member
// definitions, unchanged, from the reference header (checkout or staged copy)
// into the git-ignored oracle/_ref/ref_print_members.inc and compiles this
// file with it into oracle/_ref/ref_print_check. The class template below
// declares only what the definitions use: the host arrays they print and the
// two helpers they call on errors. Its template parameters, member names and
// enum order are the reference's (Interface.cuh:33-47, :117-176).
//
// Usage: ref_print_check <directory>: writes, for the same synthetic arrays
// as tests/textout_check.cpp (NT = 4, SD = 3, NCP = 2, NSP = 2, NISP = 1,
// NA = 1, NIA = 2, NDO = 5), ActualStateInSolverObject.txt,
// IntegerAccessoriesInSolverObject.txt and DenseOutput_2.txt into the
// directory (the reference writes into the working directory).
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <unistd.h>

enum Algorithms { RK4, RKCK45 };
enum ListOfVariables {
    All, TimeDomain, ActualState, ActualTime, ControlParameters, SharedParameters, IntegerSharedParameters,
    Accessories, IntegerAccessories, DenseOutput, DenseIndex, DenseTime, DenseState
};

static std::string VariablesToString(ListOfVariables v) { return std::to_string(static_cast<int>(v)); }

template <int NT, int SD, int NCP, int NSP, int NISP, int NE, int NA, int NIA, int NDO, Algorithms Algorithm,
          class Precision>
class ProblemSolver {
public:
    Precision* h_TimeDomain = nullptr;
    Precision* h_ActualState = nullptr;
    Precision* h_ActualTime = nullptr;
    Precision* h_ControlParameters = nullptr;
    Precision* h_SharedParameters = nullptr;
    int* h_IntegerSharedParameters = nullptr;
    Precision* h_Accessories = nullptr;
    int* h_IntegerAccessories = nullptr;
    int* h_DenseOutputIndex = nullptr;
    Precision* h_DenseOutputTimeInstances = nullptr;
    Precision* h_DenseOutputStates = nullptr;

    template <typename T>
    void WriteToFileGeneral(std::string, int, int, T*);
    void Print(ListOfVariables);
    void Print(ListOfVariables, int);
    void BoundCheck(std::string f, std::string what, int v, int lo, int hi)
    {
        if (v < lo || v > hi) {
            std::cerr << f << ": " << what << " out of range" << std::endl;
            std::exit(EXIT_FAILURE);
        }
    }
};

#include "ref_print_members.inc"

static double val(int k) { return (k % 7 - 3) * 1.2345678901234 * std::pow(10.0, k % 9 - 4); }
static std::vector<double> dv(int n, int off) { std::vector<double> v(n); for (int i = 0; i < n; i++) v[i] = val(i + off); return v; }
static std::vector<int> iv(int n, int off) { std::vector<int> v(n); for (int i = 0; i < n; i++) v[i] = (i + off) * 37 % 101 - 50; return v; }

int main(int argc, char** argv)
{
    if (argc > 1 && chdir(argv[1]) != 0) return 2;
    constexpr int nt = 4, sd = 3;
    ProblemSolver<nt, sd, 2, 2, 1, 0, 1, 2, 5, RKCK45, double> s;
    auto x = dv(sd * nt, 1);
    auto ia = iv(2 * nt, 3);
    auto cp = dv(2 * nt, 20), sp = dv(2, 30), acc = dv(nt, 40), dt = dv(5 * nt, 50), ds = dv(5 * sd * nt, 80);
    auto spi = iv(1, 7);
    std::vector<int> didx = {5, 0, 3, 2};
    s.h_ActualState = x.data();
    s.h_IntegerAccessories = ia.data();
    s.h_ControlParameters = cp.data();
    s.h_SharedParameters = sp.data();
    s.h_IntegerSharedParameters = spi.data();
    s.h_Accessories = acc.data();
    s.h_DenseOutputIndex = didx.data();
    s.h_DenseOutputTimeInstances = dt.data();
    s.h_DenseOutputStates = ds.data();
    s.Print(ActualState);
    s.Print(IntegerAccessories);
    s.Print(DenseOutput, 2);
    return 0;
}
