"""The C ABI library: loads without a GPU, exports every symbol include/gbx.h
declares, and its host-only entry points behave (no compute calls here)."""
import ctypes
import os
import re

import pytest

from openmmcustomgbintegralforce_gb300 import _lib, build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build_cuda()
    return _lib.load()


def declared_symbols():
    text = open(os.path.join(REPO, "include", "gbx.h")).read()
    return sorted(set(re.findall(r"GBX_API\s+[\w\s\*]+?\b(gbx_\w+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_status_strings_and_version(lib):
    assert lib.gbx_version() >= 10000
    assert lib.gbx_status_string(0) == b"ok"
    assert lib.gbx_status_string(6) == b"lookup table too large"


def test_presets(lib):
    cfg = _lib.GbxConfig()
    assert lib.gbx_config_preset(0, ctypes.byref(cfg)) == 0
    assert (cfg.model, cfg.n_radial, cfg.lebedev_order, cfg.table_mode) == (0, 24, 38, 0)
    assert abs(cfg.table_buffer - 0.20) < 1e-15 and cfg.table_cap == 0
    assert abs(cfg.prefactor + 138.935456 * (1 - 1 / 80)) < 1e-12
    assert lib.gbx_config_preset(1, ctypes.byref(cfg)) == 0
    assert (cfg.lebedev_order, cfg.table_mode, cfg.table_cap) == (26, 1, 64)
    assert lib.gbx_config_preset(3, ctypes.byref(cfg)) == 0
    assert (cfg.model, cfg.table_mode, cfg.beta, cfg.lam) == (2, 2, -20.0, 0.5)
    assert lib.gbx_config_preset(99, ctypes.byref(cfg)) == 1


def test_create_rejects_bad_arguments_before_touching_the_device(lib):
    cfg = _lib.GbxConfig()
    lib.gbx_config_preset(0, ctypes.byref(cfg))
    h = ctypes.c_void_p()
    assert lib.gbx_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == 1
    assert lib.gbx_create(None, 10, ctypes.byref(h)) == 1
    cfg.lebedev_order = 37
    assert lib.gbx_create(ctypes.byref(cfg), 10, ctypes.byref(h)) == 1
    lib.gbx_config_preset(2, ctypes.byref(cfg))
    cfg.box[0] = 0.0
    assert lib.gbx_create(ctypes.byref(cfg), 10, ctypes.byref(h)) == 1


def test_create_checks_cutoff_periodic_settings_before_touching_the_device(lib):
    """CutoffPeriodic: the standalone GBSW table or the box-sampled table, a
    cutoff, and box edges of at least twice the cutoff
    (CharmmReferenceGBSW.cpp:147-159)."""
    cfg = _lib.GbxConfig()
    h = ctypes.c_void_p()
    lib.gbx_config_preset(1, ctypes.byref(cfg))  # the grid table has no periodic form
    cfg.periodic, cfg.cutoff = 1, 1.0
    assert lib.gbx_create(ctypes.byref(cfg), 10, ctypes.byref(h)) == 4  # unsupported
    lib.gbx_config_preset(0, ctypes.byref(cfg))
    cfg.periodic, cfg.cutoff = 1, 0.0
    cfg.box[0] = cfg.box[1] = cfg.box[2] = 5.0
    assert lib.gbx_create(ctypes.byref(cfg), 10, ctypes.byref(h)) == 1  # no cutoff
    cfg.cutoff = 1.2
    cfg.box[2] = 2.3
    assert lib.gbx_create(ctypes.byref(cfg), 10, ctypes.byref(h)) == 1  # box < 2 cutoff
