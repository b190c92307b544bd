"""CPU suite: the C ABI library loads and exports every symbol include/ia.h
declares; argument checks that fire before any device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from inverseacoustics_gb300 import _lib


def header_functions():
    txt = open(os.path.join(ROOT, "include", "ia.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ia_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_table_covers_header():
    assert set(header_functions()) == set(_lib.declared_symbols())


def test_config_defaults():
    cfg = _lib.default_config()
    assert (cfg.c, cfg.rho, cfg.gcv_points, cfg.gcv_mode, cfg.method) == (343.0, 1.21, 200, 0, 0)
    assert C.sizeof(_lib.Config) == _lib.lib().ia_config_size()


def test_status_strings():
    L = _lib.lib()
    assert L.ia_status_string(0) == b"ok"
    assert L.ia_status_string(7) == b"invalid quadrature rule"


def test_tsvd_k_out_of_range_is_an_error():
    """The reference prints and leaves x unset (CUDA/tsvd.cuh:124-126); here it
    is IA_ERR_ARG, raised before any device work."""
    from inverseacoustics_gb300 import api
    U = np.eye(4, dtype=np.complex128)
    s = np.ones(4)
    for k in (0, 5):
        with pytest.raises(_lib.IAError) as e:
            api.tsvd(U, s, U, np.ones(4), k)
        assert e.value.code == 1


def test_bad_arguments_rejected_before_device_work():
    from inverseacoustics_gb300 import api
    with pytest.raises(_lib.IAError) as e:
        api.esm(np.zeros((3, 4)), np.zeros((3, 4)), -1.0, 0.5)
    assert e.value.code == 1
    bad = np.zeros((3, 4))
    bad[0, 0] = np.nan
    with pytest.raises(_lib.IAError) as e:
        api.esm(bad, np.ones((3, 4)), 1.0, 0.5)
    assert e.value.code == 6
    # invr: n_am outside [1, m]
    from inverseacoustics_gb300 import geometry as g
    nodes, elems = g.icosphere(0, 0.1)
    for n_am in (0, nodes.shape[1] + 1):
        with pytest.raises(_lib.IAError) as e:
            api.invr(nodes, elems, np.ones((3, 2)), 1.0, n_am)
        assert e.value.code == 1
    # wavenumber k <= 0 or not a number (the reference has no check: k = 0
    # zeroes i rho c k B and gives a singular transfer)
    for k in (0.0, -2.0, float("nan")):
        with pytest.raises(_lib.IAError) as e:
            api.ibem(nodes, elems, np.ones((3, 2)), k)
        assert e.value.code == 1
        with pytest.raises(_lib.IAError) as e:
            api.hels(np.ones((3, 4)), np.ones((3, 4)), k, 2)
        assert e.value.code == 1


def test_release_build_reports_bounds_checks_off():
    """libia.so is the release build: ia_bounds_report answers enabled = 0 and
    touches no device (the checks exist only in libia_debug.so)."""
    L = _lib.lib()
    en, cnt, fil, line, idx, ext = C.c_int(7), C.c_ulonglong(9), C.c_char_p(), C.c_int(), C.c_longlong(), C.c_longlong()
    assert L.ia_bounds_report(C.byref(en), C.byref(cnt), C.byref(fil), C.byref(line), C.byref(idx), C.byref(ext)) == 0
    assert (en.value, cnt.value, fil.value) == (0, 0, None)
