// A user program written against the reference's per-thread interface, in
// the style of Tutorials_SingleSystem_PerThread/T2_Lorenz/Lorenz.cu: system
// definition first, interface header second, ProblemSolver with compile-time
// sizes, SetHost/SolverOption/Synchronise/Solve/GetHost. Built against the
// GB300 drop-in header and runtime; prints the end states so the test can
// compare them with the CPU oracle.
#include <cstdio>
#include <vector>

#include "lorenz.cuh"
#include "SingleSystem_PerThread_Interface.cuh"

#define SOLVER RKCK45
#define PRECISION double
const int NT   = 256;
const int SD   = 3;
const int NCP  = 1;
const int NSP  = 0;
const int NISP = 0;
const int NE   = 0;
const int NA   = 0;
const int NIA  = 1;
const int NDO  = 0;

int main()
{
    int device = SelectDeviceByClosestRevision(10, 3);
    ProblemSolver<NT, SD, NCP, NSP, NISP, NE, NA, NIA, NDO, SOLVER, PRECISION> lorenz(device);

    lorenz.SolverOption(ThreadsPerBlock, 64);
    lorenz.SolverOption(InitialTimeStep, 1.0e-2);
    for (int i = 0; i < SD; i++) {
        lorenz.SolverOption(RelativeTolerance, i, 1.0e-10);
        lorenz.SolverOption(AbsoluteTolerance, i, 1.0e-10);
    }
    for (int tid = 0; tid < NT; tid++) {
        const double rho = (tid == NT - 1) ? 21.0 : 0.0 + tid * (21.0 / (NT - 1));
        lorenz.SetHost(tid, TimeDomain, 0, 0.0);
        lorenz.SetHost(tid, TimeDomain, 1, 10.0);
        lorenz.SetHost(tid, ActualTime, 0.0);
        for (int c = 0; c < SD; c++) lorenz.SetHost(tid, ActualState, c, 10.0);
        lorenz.SetHost(tid, ControlParameters, 0, rho);
        lorenz.SetHost(tid, IntegerAccessories, 0, 0);
    }
    lorenz.SynchroniseFromHostToDevice(All);
    lorenz.Solve();
    lorenz.SynchroniseFromDeviceToHost(All);
    lorenz.InsertSynchronisationPoint();
    lorenz.SynchroniseSolver();

    for (int tid = 0; tid < NT; tid++)
        printf("%d %.17g %.17g %.17g %d\n", tid, lorenz.GetHost<double>(tid, ActualState, 0),
               lorenz.GetHost<double>(tid, ActualState, 1), lorenz.GetHost<double>(tid, ActualState, 2),
               lorenz.GetHost<int>(tid, IntegerAccessories, 0));
    return 0;
}
