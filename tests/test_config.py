"""Host-side semantics of the C ABI: default strides, descriptors, errors, exports.

These run without a GPU: the functions below do not touch the device.
Expected values restate the reference's host tests (test/parser.cpp:33-148) and the
stride rules of src/base/configuration.cpp:24-56."""
import ctypes
import re

import pytest

from conftest import REPO


def test_library_exports_every_declared_symbol(bb):
    header = open(REPO + '/include/bbfft_gb300.h').read()
    declared = set(re.findall(r'BBFFT_GB300_API\s+[^(]*?\b(bbfft_\w+)\s*\(', header))
    assert declared, 'no declarations found'
    L = bb.lib()
    for name in declared:
        assert hasattr(L, name), name
    assert declared == set(bb.exported_symbols()) | (declared - set(bb.exported_symbols()))
    missing_in_binding = declared - set(bb.exported_symbols())
    assert not missing_in_binding, missing_in_binding


@pytest.mark.parametrize('dim,shape,type,inplace,expected', [
    (1, [1, 64, 16384], 0, False, [1, 1, 64, 0, 0]),
    (1, [8, 64, 100], 1, False, [1, 8, 512, 0, 0]),
    (1, [8, 64, 100], 1, True, [1, 8, 8 * 66, 0, 0]),
    (1, [8, 64, 100], 2, True, [1, 8, 8 * 33, 0, 0]),
    (2, [1, 128, 128, 2048], 1, False, [1, 1, 128, 128 * 128, 0]),
    (2, [1, 128, 128, 2048], 1, True, [1, 1, 130, 130 * 128, 0]),
    (3, [2, 5, 6, 7, 3], 0, False, [1, 2, 10, 60, 420]),
])
def test_default_istride(bb, dim, shape, type, inplace, expected):
    assert bb.default_istride(dim, shape + [0] * (5 - len(shape)), type, inplace) == expected


def test_default_ostride_swaps_real_roles(bb):
    shape = [8, 64, 100, 0, 0]
    assert bb.default_ostride(1, shape, 1, True) == bb.default_istride(1, shape, 2, True)
    assert bb.default_ostride(1, shape, 2, True) == bb.default_istride(1, shape, 1, True)
    assert bb.default_ostride(1, shape, 0, False) == bb.default_istride(1, shape, 0, False)


# (descriptor, dim, shape, precision, direction, type, istride or 'i'/'o', ostride or 'i'/'o')
PARSER_CASES = [
    ('srfi5', 1, [1, 5, 1], 4, -1, 1, 'i', 'i'),
    ('dcbi4*5', 1, [1, 4, 5], 8, 1, 0, 'i', 'i'),
    ('dcbi4.5', 1, [4, 5, 1], 8, 1, 0, 'i', 'i'),
    ('drbo4.5*6', 1, [4, 5, 6], 8, 1, 2, 'o', 'o'),
    ('drfo5x6x7', 3, [1, 5, 6, 7, 1], 8, -1, 1, 'o', 'o'),
    ('srbo4.5x6*7', 2, [4, 5, 6, 7], 4, 1, 2, 'o', 'o'),
    ('scfo16*32i1,1,20', 1, [1, 16, 32], 4, -1, 0, [1, 1, 20], 'o'),
    ('scfo16*32i1,1,20o1,2,32', 1, [1, 16, 32], 4, -1, 0, [1, 1, 20], [1, 2, 32]),
    ('scfi16*32i1,1,20o1,1,20', 1, [1, 16, 32], 4, -1, 0, [1, 1, 20], [1, 1, 20]),
]


@pytest.mark.parametrize('case', PARSER_CASES, ids=[c[0] for c in PARSER_CASES])
def test_descriptor_parser(bb, case):
    """reference test/parser.cpp:33-145"""
    desc, dim, shape, prec, direction, type, ist, ost = case
    cfg = bb.parse_fft_descriptor(desc)
    assert cfg.dim == dim
    full = shape + [0] * (5 - len(shape))
    assert list(cfg.shape) == full
    assert cfg.precision == prec and cfg.direction == direction and cfg.type == type
    if isinstance(ist, str):
        assert list(cfg.istride) == bb.default_istride(dim, full, type, ist == 'i')
    else:
        assert list(cfg.istride)[:len(ist)] == ist
    if isinstance(ost, str):
        assert list(cfg.ostride) == bb.default_ostride(dim, full, type, ost == 'i')
    else:
        assert list(cfg.ostride)[:len(ost)] == ost
    assert bb.to_string(cfg) == desc


def test_descriptor_parser_rejects(bb):
    with pytest.raises(bb.ParseError):
        bb.parse_fft_descriptor('srb4x5*6x7')
    with pytest.raises(bb.ParseError) as e:
        bb.parse_fft_descriptor('qcfo8')
    assert "expected 's' (single) or 'd' (double)" in e.value.message


def test_to_string_rejects_inconsistent_direction(bb):
    cfg = bb.configuration(1, [1, 8, 1], type=1, direction=1)
    with pytest.raises(bb.BBFFTError):
        bb.to_string(cfg)


def test_last_error_is_thread_local_and_set(bb):
    cfg = bb.configuration(1, [1, 8, 1])
    cfg.istride[0] = 2
    h = ctypes.c_void_p()
    rc = bb.lib().bbfft_plan_create(ctypes.byref(cfg), None, None, ctypes.byref(h))
    assert rc == -1
    assert b's0' in bb.lib().bbfft_last_error()


@pytest.mark.parametrize('dim', [0, 4])
def test_unsupported_dimension_is_bad_configuration(bb, dim):
    """reference test/error.cpp:13-21 and src/common/algorithm.hpp:23-25"""
    cfg = bb.configuration(1, [1, 8, 1])
    cfg.dim = dim
    with pytest.raises(bb.BadConfiguration):
        bb.make_plan(cfg)


def test_nd_callbacks_need_default_layout(bb):
    """nd callbacks (the reference rejects them, src/common/algorithm/nd_fft.hpp:29-31) run in
    the first and last pass of the chain; custom nd layouts, whose chain runs on packed
    copies, cannot take them"""
    cfg = bb.configuration(2, [1, 8, 8, 2], istride=[1, 1, 9, 80, 0], ostride=[1, 1, 9, 80, 0],
                           callbacks=('x', 'load', None))
    with pytest.raises(bb.BadConfiguration, match='callbacks of nd transforms'):
        bb.make_plan(cfg)


def test_nd_custom_layout_adjoint_rejected(bb):
    """nd transforms with custom layouts run through a strided gather / scatter (the
    reference rejects them, src/common/algorithm/nd_fft.hpp:47-49); their adjoint plans
    are not offered"""
    cfg = bb.configuration(2, [1, 8, 8, 2], istride=[1, 1, 9, 80, 0], ostride=[1, 1, 9, 80, 0])
    with pytest.raises(bb.BadConfiguration, match='default tensor layout'):
        bb.make_adjoint_plan(cfg)


def test_version(bb):
    assert 'sm_103a' in bb.version()
