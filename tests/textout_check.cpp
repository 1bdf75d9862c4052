// Writes every Print file format of include/mpgos/dropin_print.h for fixed
// synthetic arrays into the directory given as argv[1]; test_textout_cpu.py
// writes the same arrays through mpgos_gb300.textout and compares the bytes.
#include <cmath>
#include <string>
#include <vector>

#include "dropin_print.h"

namespace pr = mpgos::dropin::print;

static double val(int k) { return (k % 7 - 3) * 1.2345678901234 * std::pow(10.0, k % 9 - 4); }
static std::vector<double> dv(int n, int off) { std::vector<double> v(n); for (int i = 0; i < n; i++) v[i] = val(i + off); return v; }
static std::vector<int> iv(int n, int off) { std::vector<int> v(n); for (int i = 0; i < n; i++) v[i] = (i + off) * 37 % 101 - 50; return v; }

int main(int argc, char** argv)
{
    const std::string d = argc > 1 ? std::string(argv[1]) + "/" : std::string();
    // per-thread: NT = 4, SD = 3, NCP = 2, NSP = 2, NISP = 1, NA = 1, NIA = 2, NDO = 5
    const int nt = 4, sd = 3;
    auto x = dv(sd * nt, 1);
    auto ia = iv(2 * nt, 3);
    pr::general(d + "general_double.txt", nt, sd, x.data());
    pr::general(d + "general_int.txt", nt, 2, ia.data());
    auto cp = dv(2 * nt, 20), sp = dv(2, 30), acc = dv(nt, 40), dt = dv(5 * nt, 50), ds = dv(5 * sd * nt, 80);
    auto spi = iv(1, 7);
    std::vector<int> didx = {5, 0, 3, 2};
    pr::perthread_dense(d + "pt_dense.txt", 2, nt, sd, 2, 2, 1, 1, 2, 5, cp.data(), sp.data(), spi.data(),
                        acc.data(), ia.data(), didx.data(), dt.data(), ds.data());
    // coupled: NS = 5, UPS = 3, UD = 2, launch shape TPB = 4, SPB = 2 (padded rows)
    const int ns = 5, ups = 3, ud = 2, nu = ns * ups;
    auto xs = dv(ud * nu, 200);
    auto iua = iv(1 * nu, 11);
    pr::system_scope(d + "system_double.txt", ns, 2, dv(2 * ns, 300).data());
    pr::system_scope(d + "system_int.txt", ns, 1, iv(ns, 5).data());
    pr::unit_scope(d + "unit_double.txt", ud, xs.data(), ns, ups, 4, 2);
    pr::unit_scope(d + "unit_int.txt", 1, iua.data(), ns, ups, 4, 2);
    pr::unit_scope(d + "unit_unpadded.txt", ud, xs.data(), ns, ups, 3, 1);
    auto up = dv(2 * nu, 400), ua = dv(1 * nu, 450), spc = dv(1 * ns, 500), sa = dv(2 * ns, 520), gp = dv(2, 540);
    auto isa = iv(1 * ns, 9), igp = iv(1, 13);
    std::vector<int> cdidx = {0, 4, 1, 2, 3};
    auto cdt = dv(4 * ns, 600), cds = dv(4 * ud * nu, 700);
    pr::coupled_dense(d + "cb_dense.txt", 1, ns, ups, ud, 2, 1, 1, 1, 2, 1, 2, 1, 4, up.data(), ua.data(),
                      iua.data(), spc.data(), sa.data(), isa.data(), gp.data(), igp.data(), cdidx.data(), cdt.data(),
                      cds.data());
    return 0;
}
