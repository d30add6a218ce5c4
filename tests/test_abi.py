"""CPU checks of the C-ABI boundary: the library builds, loads and exports
every entry point include/axgpu.h declares (no compute without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import axion_grav_gb300 as ag

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "axgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(axg_[a-z0-9_]+)\s*\(", src)))


def test_header_and_python_mirror_agree(built):
    assert declared_functions() == sorted(ag.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(ag.library_path())
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_params_struct_layout(built):
    # axg_params: 12 int32 + 12 double + 2 uint64 = 48 + 96 + 16 bytes
    assert ctypes.sizeof(ag.Params) == 160
    p = ag.default_params()
    assert p.num_bin == 50 and p.num_bin_grav == 25 and p.compat == ag.COMPAT_REF


def test_get_dtau_host_only(built):
    # evolve.f90:10-24, pure host arithmetic
    p = ag.default_params(ngrid=64, dspa=0.25, sigma_cr=2.0)
    lib = ag.load_library()
    dt, n = ctypes.c_double(), ctypes.c_int64()
    assert lib.axg_get_dtau(ctypes.byref(p), 1.0, 3.0, 0.5, ctypes.byref(dt), ctypes.byref(n)) == 0
    from oracle import axo
    assert (dt.value, n.value) == axo.get_dtau(p, 1.0, 3.0, 0.5)
    assert lib.axg_get_dtau(ctypes.byref(p), 3.0, 1.0, 0.5, ctypes.byref(dt), ctypes.byref(n)) == -1


def test_param_chk_roundtrip(built, tmp_path):
    lib = ag.load_library()
    f = str(tmp_path / "run_param.chk").encode()
    assert lib.axg_write_param_chk(f, 7, 12.5, 1) == 0
    i, t, fl = ctypes.c_int64(), ctypes.c_double(), ctypes.c_int()
    assert lib.axg_read_param_chk(f, ctypes.byref(i), ctypes.byref(t), ctypes.byref(fl)) == 0
    assert (i.value, t.value, fl.value) == (7, 12.5, 1)


def test_tile_table(built):
    lib = ag.load_library()
    n = lib.axg_tile_count()
    assert n >= 3
    a, b, c, d = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    pw = 0
    for i in range(n):
        assert lib.axg_tile_info(i, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)) == 0
        assert a.value % 32 == 0 and b.value >= 4 and c.value >= 2 and d.value in (0, 1)
        pw += d.value
    assert 0 < pw < n  # both pointwise paths (registers, TMA ring) are in the search space
    assert lib.axg_tile_info(0, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), None) == 0
    assert lib.axg_tile_info(n, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), None) == -1


def test_create_without_gpu_fails_loudly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(ag.AxgError):
        ag.Lattice(ag.default_params(ngrid=16))


def test_oracle_default_params_match_library(built):
    # the oracle fills the same defaults without loading the GPU library
    from oracle import axo
    a, b = ag.default_params(), axo.default_params()
    for name, _ in ag.Params._fields_:
        assert getattr(a, name) == getattr(b, name), name


def test_green_on_odd_or_tiny_gw_grid_is_rejected(built):
    # Green's mode runs on ngrid / 2^degrade_spec (grav_waves.f90:37-45); a
    # GW grid that is odd or below 4 sites is refused before any device work
    lib = ag.load_library()
    out = ctypes.c_void_p()
    for n, deg in ((24, 3), (16, 3), (8, 2)):
        p = ag.default_params(ngrid=n, degrade_spec=deg, gw_mode=ag.GW_GREEN)
        assert lib.axg_create(ctypes.byref(p), ctypes.byref(out)) == -7, (n, deg)
        assert b"GW grid" in lib.axg_last_error(None)
    # the same degrade_spec is fine without Green's mode (the field spectrum
    # coarse-grains on its own)
    p = ag.default_params(ngrid=24, degrade_spec=3, gw_mode=ag.GW_NONE)
    rc = lib.axg_create(ctypes.byref(p), ctypes.byref(out))
    assert rc != -7
    if rc == 0:
        lib.axg_destroy(out)
