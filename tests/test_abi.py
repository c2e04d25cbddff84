"""The C-ABI library loads without a GPU, exports every entry point that
include/pmx.h declares, and rejects bad arguments before touching a device."""

import ctypes
import os
import re

import pytest

from pmwd_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.load()


def declared_functions():
    src = open(os.path.join(ROOT, 'include', 'pmx.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(pmx_\w+)\s*\(', src)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert 'pmx_scatter' in names and 'pmx_nbody_adj_step' in names
    assert len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f'{name} has no ctypes signature'


def test_version_and_error_channel(lib):
    assert lib.pmx_version() >= 100
    assert isinstance(lib.pmx_last_error(), bytes)


def test_bad_arguments_rejected_on_host(lib):
    spec = _lib.make_spec(3, (8, 8, 8), (8, 8, 8), 1.0)
    spec.dim = 4
    st = lib.pmx_scatter(ctypes.byref(spec), None, None, 10, None, 1.0, 1, None, None)
    assert st == -1
    assert b'dim' in lib.pmx_last_error()
    spec.dim = 3
    spec.conf_cell_size = 0.0
    st = lib.pmx_gather(ctypes.byref(spec), None, None, 0, None, 1, None, 0.0, None, None)
    assert st == -1
    spec.conf_cell_size = 1.0
    # scalar val with several channels is a shape error
    st = lib.pmx_scatter(ctypes.byref(spec), None, None, 0, None, 1.0, 3, ctypes.c_void_p(16), None)
    assert st == -2
    # zero particles with valid arguments is a no-op that succeeds
    st = lib.pmx_scatter(ctypes.byref(spec), None, None, 0, None, 1.0, 1, ctypes.c_void_p(16), None)
    assert st == 0
    assert lib.pmx_force(None, ctypes.byref(spec), None, None, 0, 1, 0.3, None, None) == -1
    assert lib.pmx_kick(None, None, -1, 1.0, None) == -1
