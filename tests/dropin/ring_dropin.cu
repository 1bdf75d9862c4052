// A user program written against the reference's coupled per-block
// interface, in the style of
// Tutorials_CoupledSystems_PerBlock/T1_RingOfDuffingOscillators: system
// definition first, interface header second, ProblemSolver with the twenty
// compile-time arguments, SetHost (system, unit, global and coupling-matrix
// overloads) / SolverOption / Synchronise / Solve / GetHost. Built against
// the GB300 drop-in header and runtime. Reads its inputs from ring_input.bin
// (written by the test) and prints the end states and counters.
#include <cstdio>
#include <vector>

#define MPGOS_SYS_UPS 16
#include "ring_duffing.cuh"
#include "CoupledSystems_PerBlock_Interface.cuh"

#define SOLVER RKCK45
#define PRECISION double
const int NS = 64, UPS = 16, UD = 2, TPB = 64, SPB = 4, NC = 1, CBW = 0, CCI = 0;
const int NUP = 0, NSP = 1, NGP = 1, NiGP = 0, NUA = 0, NiUA = 1, NSA = 0, NiSA = 1, NE = 1, NDO = 0;

int main()
{
    std::vector<double> x(2 * NS * UPS), B(NS), C(UPS * UPS), td(2);
    FILE* in = fopen("ring_input.bin", "rb");
    if (!in || fread(td.data(), 8, 2, in) != 2 || fread(x.data(), 8, x.size(), in) != x.size() ||
        fread(B.data(), 8, NS, in) != static_cast<size_t>(NS) || fread(C.data(), 8, C.size(), in) != C.size())
        return 2;
    fclose(in);

    ProblemSolver<NS, UPS, UD, TPB, SPB, NC, CBW, CCI, NUP, NSP, NGP, NiGP, NUA, NiUA, NSA, NiSA, NE, NDO, SOLVER, PRECISION>
        ring(0);
    ring.SolverOption(InitialTimeStep, 1.0e-2);
    for (int i = 0; i < UD; i++) {
        ring.SolverOption(RelativeTolerance, i, 1.0e-9);
        ring.SolverOption(AbsoluteTolerance, i, 1.0e-9);
    }
    ring.SolverOption(EventTolerance, 0, 1.0e-6);
    ring.SolverOption(EventDirection, 0, 0);
    for (int s = 0; s < NS; s++) {
        ring.SetHost(s, TimeDomain, 0, td[0]);
        ring.SetHost(s, TimeDomain, 1, td[1]);
        ring.SetHost(s, ActualTime, td[0]);
        ring.SetHost(s, SystemParameters, 0, B[s]);
        ring.SetHost(s, CouplingStrength, 0, 1.0);
        ring.SetHost(s, IntegerSystemAccessories, 0, 0);
        for (int u = 0; u < UPS; u++) {
            ring.SetHost(s, u, ActualState, 0, x[s * UPS + u]);
            ring.SetHost(s, u, ActualState, 1, x[NS * UPS + s * UPS + u]);
            ring.SetHost(s, u, IntegerUnitAccessories, 0, 0);
        }
    }
    ring.SetHost(GlobalParameters, 0, 0.25);
    ring.SetHost(CouplingIndex, 0, 1);
    for (int r = 0; r < UPS; r++)
        for (int c = 0; c < UPS; c++) ring.SetHost(0, CouplingMatrix, r, c, C[r * UPS + c]);
    ring.SynchroniseFromHostToDevice(All);
    ring.Solve();
    ring.SynchroniseFromDeviceToHost(All);
    ring.InsertSynchronisationPoint();
    ring.SynchroniseSolver();

    for (int s = 0; s < NS; s++)
        for (int u = 0; u < UPS; u++)
            printf("%d %d %.17g %.17g %d %d\n", s, u, ring.GetHost<double>(s, u, ActualState, 0),
                   ring.GetHost<double>(s, u, ActualState, 1), ring.GetHost<int>(s, u, IntegerUnitAccessories, 0),
                   ring.GetHost<int>(s, IntegerSystemAccessories, 0));
    return 0;
}
