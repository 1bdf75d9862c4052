"""CPU tests of the coupled per-block solver: plugin tables, the host-side
coupling-matrix storage of the reference's SetHost, and the coupled oracle."""
import ctypes as C

import numpy as np
import pytest

from tests.conftest import gpu_available
from mpgos_gb300 import capi, coupled_workloads as CW
from mpgos_gb300.coupled import matrix_entries, matrix_slot, store_matrices
from oracle import oracle as O


@pytest.mark.parametrize("system", sorted(CW.CB_SHAPES))
def test_coupled_plugins_export_kernel_tables(system, native_libs):
    lib = capi.plugin(system)
    assert hasattr(lib, "mpgos_cb_system_kernels") and not hasattr(lib, "mpgos_pt_system_kernels")
    ups, ud, nc, cbw, cci, nup, nsp, ngp, nigp, nua, niua, nsa, nisa, ne = CW.CB_SHAPES[system]
    for alg in (0, 1):
        t = capi.coupled_kernel_table_info(capi.coupled_kernel_table(system, alg, 8))
        s = t.shape
        assert t.abi_version == capi.ABI_VERSION and t.name.decode() == system
        assert (s.ups, s.ud, s.nc, s.cbw, s.cci, s.nup, s.nsp, s.ngp, s.nigp, s.nua, s.niua, s.nsa, s.nisa, s.ne) == \
            CW.CB_SHAPES[system]
        assert s.algorithm == alg and s.precision_bytes == 8
        assert s.matrix_entries == matrix_entries(ups, cbw, cci)
        assert t.launch and t.occupancy and t.dynamic_smem
    assert not lib.mpgos_cb_system_kernels(1, 4)
    # the oracle is built from the same plugin source
    assert O.oracle_cb_shape(system)[:14] == CW.CB_SHAPES[system]
    assert O.oracle_cb_shape(system)[14] == matrix_entries(ups, cbw, cci)


def test_per_thread_and_coupled_tables_are_not_mixed(native_libs):
    with pytest.raises(capi.MpgosError):
        capi.coupled_kernel_table("lorenz", 1, 8)
    with pytest.raises(capi.MpgosError):
        capi.kernel_table("ring64", 1, 8)


def test_coupled_create_rejects_bad_arguments(native_libs):
    lib = capi.runtime()
    h = C.c_void_p()
    assert lib.mpgos_cb_create(None, 16, 0, 0, C.byref(h)) == 1
    table = capi.coupled_kernel_table("ring16_full", 1, 8)
    assert lib.mpgos_cb_create(table, 0, 0, 0, C.byref(h)) == 1
    assert lib.mpgos_cb_create(table, 16, -1, 0, C.byref(h)) == 1
    assert not h.value
    assert lib.mpgos_cb_set_option(None, 0, 0, 1.0) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_coupled_create_without_gpu_fails_loudly(native_libs):
    from mpgos_gb300.coupled import CoupledProblemSolver
    with pytest.raises(capi.MpgosError) as e:
        CoupledProblemSolver("ring16_full", 16)
    assert e.value.code == 2


# ---- coupling-matrix storage (CoupledSystems_PerBlock_Interface.cuh:993-1080)
def test_matrix_slot_full_is_column_major():
    ups = 5
    assert matrix_slot(ups, 0, 0, 0, 2, 3) == 2 + 3 * ups
    assert matrix_slot(ups, 0, 0, 1, 0, 0) == ups * ups


def test_matrix_slot_banded_and_circular():
    ups, cbw = 8, 1
    # row 0: columns 7 (wrapped), 0, 1 -> shifted diagonals 0, 1, 2
    assert [matrix_slot(ups, cbw, 0, 0, 0, c) for c in (7, 0, 1)] == [0, 0 + ups, 0 + 2 * ups]
    assert [matrix_slot(ups, cbw, 0, 0, 3, c) for c in (2, 3, 4)] == [3, 3 + ups, 3 + 2 * ups]
    assert [matrix_slot(ups, cbw, 1, 0, 5, c) for c in (4, 5, 6)] == [0, 1, 2]
    assert matrix_slot(ups, cbw, 1, 1, 5, 6) == 3 + 2
    assert [matrix_slot(ups, 0, 1, 0, 2, c) for c in (2, 3, 1)] == [0, 1, ups - 1]
    with pytest.raises(capi.MpgosError):
        matrix_slot(ups, cbw, 0, 0, 0, 4)     # outside the band


def test_store_matrices_roundtrip_dense():
    rng = np.random.default_rng(1)
    full = rng.normal(size=(2, 6, 6))
    st = store_matrices(full, 0, 0)
    for c in range(2):
        for r in range(6):
            for col in range(6):
                assert st[matrix_slot(6, 0, 0, c, r, col)] == full[c, r, col]


# ---- the coupled oracle --------------------------------------------------------
def test_oracle_storages_agree_on_a_circulant_ring():
    """The circulant ring fits every storage; the four plugins' oracles must
    integrate it to the same end states and the same integer outputs."""
    res = {}
    for s in ("ring16_full", "ring16_band", "ring16_circband", "ring16_circ"):
        res[s] = O.run_oracle_coupled(CW.ring_case(s, ns=32, periods=2, seed=3, coupling="circulant"))
    base = res["ring16_full"]
    for s, r in res.items():
        assert np.max(np.abs(r["x"] - base["x"])) <= 1e-12, s
        for k in ("iuacc", "isacc", "nacc", "nrej"):
            np.testing.assert_array_equal(r[k], base[k], err_msg=f"{s}:{k}")


def test_oracle_counts_and_bookkeeping():
    c = CW.ring_case("ring16_full", ns=16, periods=2, seed=4)
    r = O.run_oracle_coupled(c)
    assert np.all(r["t"] == c.arrays["td"][1])
    assert np.all(r["status"] == 0)
    np.testing.assert_array_equal(r["isacc"][0], r["nacc"])       # ActionAfterSuccessfulTimeStep by unit 0
    assert np.all(r["iuacc"] >= 2)                                 # crossings of x_i = 0 over two periods


def test_oracle_uncoupled_ring_is_the_single_duffing_oscillator():
    """With a zero coupling matrix every unit is an independent forced
    Duffing oscillator; units with the same initial state and B must end in
    the same state regardless of their neighbours."""
    c = CW.ring_case("ring16_full", ns=4, periods=1, seed=6)
    c.arrays["cmat"][:] = 0.0
    c.arrays["x"][:, :16] = c.arrays["x"][:, :1]                   # system 0: 16 identical units
    r = O.run_oracle_coupled(c)
    x = r["x"][:, :16]
    assert np.all(x == x[:, :1])


def test_oracle_dense_output_slots():
    c = CW.ring_case("ring16_full", ns=8, periods=1, seed=7, ndo=6)
    c.options["dense_min_dt"] = 1.0
    r = O.run_oracle_coupled(c)
    assert np.all(r["didx"] == 6)
    assert np.all(r["dtime"][0] == 0.0)
    assert np.all(np.diff(r["dtime"], axis=0) > 1.0)
    np.testing.assert_array_equal(r["dstate"][0], c.arrays["x"])


def test_oracle_active_systems_and_subrange():
    c = CW.ring_case("ring16_full", ns=8, periods=1, seed=8)
    full = O.run_oracle_coupled(c)
    part = O.run_oracle_coupled(c, first=2, count=3)
    np.testing.assert_array_equal(part["x"][:, 2 * 16:5 * 16], full["x"][:, 2 * 16:5 * 16])
    np.testing.assert_array_equal(part["x"][:, :32], c.arrays["x"][:, :32])
