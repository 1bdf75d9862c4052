// Text files of the drop-in Print functions, in the reference's formats:
// every value in an ofstream with width 18, precision 10 and
// std::scientific, data column-major ([column][row]).
//   general       per-thread Print(variable): values separated by ','
//                 (SingleSystem_PerThread_Interface.cuh:1083-1108);
//   system_scope  coupled system/global scope: every value followed by ','
//                 (CoupledSystems_PerBlock_Interface.cuh:1571-1596);
//   unit_scope    coupled unit scope: the reference's padded logical-thread
//                 rows (a block of SPB systems is padded to a multiple of
//                 TPB logical threads), padding rows as "PADDING"
//                 (:1529-1569; this library stores units without padding);
//   perthread_dense / coupled_dense  Print(DenseOutput, serial)
//                 (:1184-1276 of the per-thread interface, :1598-1806 of the
//                 coupled one).
// Host-only C++ (no CUDA), shared by both drop-in headers.
#ifndef MPGOS_DROPIN_PRINT_H
#define MPGOS_DROPIN_PRINT_H

#include <cstddef>
#include <fstream>
#include <string>

namespace mpgos {
namespace dropin {
namespace print {

inline void setup(std::ofstream& f)
{
    f.precision(10);
    f.flags(std::ios::scientific);
}

template <typename T>
void general(const std::string& name, int rows, int cols, const T* data)
{
    std::ofstream f(name);
    setup(f);
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            f.width(18);
            f << data[static_cast<size_t>(i) + static_cast<size_t>(j) * rows];
            if (j < cols - 1) f << ',';
        }
        f << '\n';
    }
}

template <typename T>
void system_scope(const std::string& name, int rows, int cols, const T* data)
{
    std::ofstream f(name);
    setup(f);
    for (int i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) {
            f.width(18);
            f << data[static_cast<size_t>(i) + static_cast<size_t>(j) * rows] << ',';
        }
        f << '\n';
    }
}

// Logical-thread layout of the reference for NS systems of UPS units, TPB
// threads and SPB systems per block (CoupledSystems_PerBlock_Interface.cuh:385-390).
struct Layout {
    int logical, padding, total, limit;
    Layout(int ns, int ups, int tpb, int spb)
    {
        logical = spb * ups;
        const int launches = logical / tpb + (logical % tpb == 0 ? 0 : 1);
        padding = launches * tpb - logical;
        const int grid = ns / spb + (ns % spb == 0 ? 0 : 1);
        total = (logical + padding) * grid;
        limit = (ns / spb) * (logical + padding) + (ns % spb) * ups;
    }
    // index of padded row r in the unpadded unit layout, -1 for padding
    long long unit(int r, int spb, int ups) const
    {
        const int per = logical + padding, b = r / per, l = r % per;
        if (l >= logical || r >= limit) return -1;
        return static_cast<long long>(b) * spb * ups + l;
    }
};

// data: [cols][ns*ups], unpadded.
template <typename T>
void unit_scope(const std::string& name, int cols, const T* data, int ns, int ups, int tpb, int spb)
{
    std::ofstream f(name);
    setup(f);
    const Layout L(ns, ups, tpb, spb);
    const size_t nu = static_cast<size_t>(ns) * ups;
    for (int r = 0; r < L.total; r++) {
        const long long u = L.unit(r, spb, ups);
        for (int j = 0; j < cols; j++) {
            f.width(18);
            if (u >= 0) f << data[static_cast<size_t>(u) + j * nu] << ',';
            else f << "PADDING" << ',';
        }
        f << '\n';
    }
}

template <typename P>
void perthread_dense(const std::string& name, int tid, int nt, int sd, int ncp, int nsp, int nisp, int na, int nia,
                     int ndo, const P* cp, const P* sp, const int* spi, const P* acc, const int* acci,
                     const int* didx, const P* dtime, const P* dstate)
{
    std::ofstream f(name);
    setup(f);
    auto row = [&](const char* title, auto* data, int n, bool per_instance) {
        f << title << "\n";
        for (int i = 0; i < n; i++) {
            f.width(18);
            f << data[per_instance ? tid + static_cast<size_t>(i) * nt : static_cast<size_t>(i)];
            if (i < n - 1) f << ',';
        }
        f << '\n';
    };
    row("ControlParameters:", cp, ncp, true);
    row("SharedParameters:", sp, nsp, false);
    row("IntegerSharedParameters:", spi, nisp, false);
    row("Accessories:", acc, na, true);
    row("IntegerAccessories:", acci, nia, true);
    f << "\nTime series:\n";
    if (ndo > 0) {
        for (int i = 0; i < didx[tid] && i < ndo; i++) {
            f.width(18);
            f << dtime[tid + static_cast<size_t>(i) * nt] << ',';
            for (int j = 0; j < sd; j++) {
                f.width(18);
                f << dstate[tid + static_cast<size_t>(j) * nt + static_cast<size_t>(i) * nt * sd];
                if (j < sd - 1) f << ',';
            }
            f << '\n';
        }
    }
}

// Coupled DenseOutput_<sid>.txt; unit arrays [field][ns*ups], system arrays
// [field][ns], dense time [ndo][ns], dense state [ndo][ud][ns*ups].
template <typename P>
void coupled_dense(const std::string& name, int sid, int ns, int ups, int ud, int nup, int nua, int niua, int nsp,
                   int nsa, int nisa, int ngp, int nigp, int ndo, const P* up, const P* uacc, const int* iuacc,
                   const P* sp, const P* sacc, const int* isacc, const P* gp, const int* igp, const int* didx,
                   const P* dtime, const P* dstate)
{
    std::ofstream f(name);
    setup(f);
    const size_t nu = static_cast<size_t>(ns) * ups, base = static_cast<size_t>(sid) * ups;
    auto units = [&](const char* title, auto* data, int n) {
        f << title << "\n";
        f.width(18);
        f << "Serial No." << ',';
        for (int u = 0; u < ups; u++) {
            f.width(18);
            f << "U" + std::to_string(u);
            if (u < ups - 1) f << ',';
        }
        f << '\n';
        for (int k = 0; k < n; k++) {
            f.width(18);
            f << k << ',';
            for (int u = 0; u < ups; u++) {
                f.width(18);
                f << data[base + u + static_cast<size_t>(k) * nu];
                if (u < ups - 1) f << ',';
            }
            f << '\n';
        }
        f << '\n';
    };
    auto list = [&](const char* title, auto* data, int n, size_t first, size_t stride) {
        f << title << "\n";
        for (int k = 0; k < n; k++) {
            f.width(18);
            f << data[first + static_cast<size_t>(k) * stride];
            if (k < n - 1) f << ',';
        }
        f << '\n' << '\n';
    };
    units("UnitParameters:", up, nup);
    units("UnitAccessories:", uacc, nua);
    units("IntegerUnitAccessories:", iuacc, niua);
    list("SystemParameters:", sp, nsp, sid, ns);
    list("SystemAccessories:", sacc, nsa, sid, ns);
    list("IntegerSystemAccessories:", isacc, nisa, sid, ns);
    list("GlobalParameters:", gp, ngp, 0, 1);
    list("IntegerGlobalParameters:", igp, nigp, 0, 1);
    f << "Time series:\n";
    f.width(18);
    f << "t" << ',';
    for (int u = 0; u < ups; u++)
        for (int c = 0; c < ud; c++) {
            f.width(18);
            f << "U" + std::to_string(u) + "/C" + std::to_string(c);
            if (u < ups - 1 || c < ud - 1) f << ',';
        }
    f << '\n';
    for (int i = 0; i < didx[sid] && i < ndo; i++) {
        f.width(18);
        f << dtime[sid + static_cast<size_t>(i) * ns] << ',';
        for (int u = 0; u < ups; u++)
            for (int c = 0; c < ud; c++) {
                f.width(18);
                f << dstate[base + u + static_cast<size_t>(c) * nu + static_cast<size_t>(i) * nu * ud];
                if (u < ups - 1 || c < ud - 1) f << ',';
            }
        f << '\n';
    }
}

}  // namespace print
}  // namespace dropin
}  // namespace mpgos

#endif
