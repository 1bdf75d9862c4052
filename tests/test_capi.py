"""CPU tests of the C-ABI boundary: libraries load, export what include/mpgos.h
declares, describe the compiled systems correctly and fail loudly."""
import ctypes as C
import re

import pytest

from tests.conftest import REPO, gpu_available
from mpgos_gb300 import capi, workloads as W

HEADER = REPO / "include" / "mpgos.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(mpgos_\w+)\s*\(", text)
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "mpgos_pt_create" in names and "mpgos_pt_system_kernels" in names
    assert set(names) == set(capi.RUNTIME_SYMBOLS) | set(capi.PLUGIN_SYMBOLS)


def test_runtime_exports_every_declared_symbol(native_libs):
    lib = capi.runtime()
    for name in capi.RUNTIME_SYMBOLS:
        assert hasattr(lib, name), name
    assert lib.mpgos_abi_version() == capi.ABI_VERSION


@pytest.mark.parametrize("system", sorted(W.SHAPES))
def test_plugins_export_kernel_tables(system, native_libs):
    lib = capi.plugin(system)
    assert hasattr(lib, "mpgos_pt_system_kernels")
    sd, ncp, nsp, nisp, ne, na, nia = W.SHAPES[system]
    for alg in (0, 1):
        t = capi.kernel_table_info(capi.kernel_table(system, alg, 8))
        assert t.abi_version == capi.ABI_VERSION
        s = t.shape
        assert (s.sd, s.ncp, s.nsp, s.nisp, s.ne, s.na, s.nia) == (sd, ncp, nsp, nisp, ne, na, nia)
        assert s.algorithm == alg and s.precision_bytes == 8
        assert t.name.decode() == system
        assert t.launch and t.occupancy
        if alg == 1:
            assert s.modes & capi.MODE_FAST_CONTROL and s.modes & capi.MODE_FP32_STAGE
    # float tables only where compiled in
    ptr = lib.mpgos_pt_system_kernels(1, 4)
    assert bool(ptr) == (system == "lorenz")


def test_create_rejects_null_table(native_libs):
    lib = capi.runtime()
    h = C.c_void_p()
    rc = lib.mpgos_pt_create(None, 16, 0, 0, C.byref(h))
    assert rc == 1
    assert b"null kernel table" in lib.mpgos_last_error()
    assert not h.value


def test_create_rejects_bad_sizes(native_libs):
    lib = capi.runtime()
    table = capi.kernel_table("lorenz", 1, 8)
    h = C.c_void_p()
    assert lib.mpgos_pt_create(table, 0, 0, 0, C.byref(h)) == 1
    assert lib.mpgos_pt_create(table, 16, -1, 0, C.byref(h)) == 1
    assert lib.mpgos_pt_set_option(None, 0, 0, 32.0) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_loudly(native_libs):
    from mpgos_gb300 import ProblemSolver, MpgosError
    with pytest.raises(MpgosError) as e:
        ProblemSolver("lorenz", 16)
    assert e.value.code == 2  # MPGOS_ERR_CUDA, no silent fallback


def test_unknown_system_raises(native_libs):
    with pytest.raises(FileNotFoundError):
        capi.plugin("no_such_system")
