"""libgclaw.so loads without a GPU, exports every function include/gclaw.h
declares, and its host-side argument checks behave (no kernel is launched)."""
import ctypes
import os
import re

import pytest

from clawpack_gb300 import _lib
from clawpack_gb300.device import make_solver_struct

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADER = os.path.join(INCLUDE, "gclaw.h")
HEADERS = [HEADER, os.path.join(INCLUDE, "gclaw3.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gclaw3?_[a-z0-9_]+)\s*\(",
                                src, flags=re.M))
    return sorted(names)


@pytest.mark.parametrize("strict", [False, True])
def test_exports_every_declared_symbol(strict):
    L = _lib.lib(strict)
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def _offsets_from_header(struct_name, header=HEADER):
    src = open(header).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct_name, struct_name), src,
                     re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, rest = re.match(
            r"((?:const\s+)?(?:unsigned\s+)?(?:long\s+long|int|double))\s*\*?\s*(.*)",
            decl).groups()
        for item in rest.split(","):
            item = item.strip()
            m = re.match(r"([a-z_0-9]+)(?:\[([A-Z_0-9]+)\])?", item)
            fields.append(m.group(1))
    return fields


def test_struct_layouts_match_header():
    for cls, name in ((_lib.GclawSolver, "gclaw_solver"), (_lib.GclawCtrl, "gclaw_ctrl")):
        assert [f[0] for f in cls._fields_] == _offsets_from_header(name)
    assert [f[0] for f in _lib.GclawSolver3._fields_] == _offsets_from_header(
        "gclaw3_solver", HEADERS[1])
    assert ctypes.sizeof(_lib.GclawCtrl) == 144
    assert ctypes.sizeof(_lib.GclawCtrl) <= 256


def good_solver(**kw):
    args = dict(rp_id=2, mx=8, my=8, dx=0.1, dy=0.1, bc_lower=[3, 3], bc_upper=[3, 3],
                mthlim=[4, 4, 4], order=2, tw=2, precision=0, problem_data=[1.0])
    args.update(kw)
    return make_solver_struct(**args)


def test_check_accepts_valid_and_rejects_invalid():
    L = _lib.lib()
    assert L.gclaw_check(ctypes.byref(good_solver())) == _lib.OK
    bad = [dict(rp_id=9), dict(mx=1), dict(dx=0.0), dict(order=3), dict(tw=5),
           dict(precision=7), dict(problem_data=[0.0]), dict(bc_lower=[2, 3]),
           dict(bc_lower=[4, 3])]
    for kw in bad:
        assert L.gclaw_check(ctypes.byref(good_solver(**kw))) == _lib.ERR_ARG, kw
    assert L.gclaw_check(ctypes.byref(good_solver(bc_lower=[0, 3]))) == _lib.ERR_UNSUPPORTED
    assert L.gclaw_check(ctypes.byref(good_solver(mthlim=[9, 4, 4]))) == _lib.ERR_UNSUPPORTED
    assert L.gclaw_check(None) == _lib.ERR_ARG


def test_step_entry_points_reject_bad_arguments_before_any_launch():
    L = _lib.lib()
    s = good_solver()
    cfl = ctypes.c_double()
    assert L.gclaw_step2(ctypes.byref(s), None, None, 0.1, None, ctypes.byref(cfl), None) == \
        _lib.ERR_ARG
    assert L.gclaw_step(ctypes.byref(s), None, None, 0.1, None, None) == _lib.ERR_ARG
    assert L.gclaw_advance(ctypes.byref(s), None, None, None, 1, None) == _lib.ERR_ARG
    assert L.gclaw_ctrl_init(None, 0.0, 0.1, 1.0, 1.0, 0.9, 1e99, 10, -1, 1, None) == \
        _lib.ERR_ARG


def test_shapes_versions_workspace():
    L = _lib.lib()
    m, mw = ctypes.c_int(), ctypes.c_int()
    for rp, shape in ((1, (3, 2)), (2, (3, 3)), (3, (4, 4))):
        assert L.gclaw_rp_shape(rp, ctypes.byref(m), ctypes.byref(mw)) == 0
        assert (m.value, mw.value) == shape
    assert L.gclaw_rp_shape(0, ctypes.byref(m), ctypes.byref(mw)) == _lib.ERR_ARG
    assert b"sm_103a" in L.gclaw_version()
    for st in (0, -1, -2, -4, -5, 2, 3, 4):
        assert L.gclaw_strerror(st) and L.gclaw_strerror(st) != b"unknown status"
    s = good_solver(mx=100, my=50)
    assert L.gclaw_evolve_workspace_bytes(ctypes.byref(s)) >= 256 + 2 * 3 * 100 * 50 * 8


def test_noalloc_refuses_oversized_grids_before_any_cuda_call():
    """gclaw_step2_noalloc checks the grid against its static scratch first,
    so the refusal needs no GPU (and no state buffers)."""
    from tests.helpers import PD, SHAPES

    L = _lib.lib()
    for rp in (1, 2, 3):
        for prec in (_lib.PREC_FP64, _lib.PREC_FP32_BULK):
            s = make_solver_struct(rp, 16384, 16384, 1e-4, 1e-4, [3, 3], [3, 3],
                                   [4] * SHAPES[rp][1], 2, 2, prec, PD[rp])
            cfl = ctypes.c_double(-1.0)
            assert L.gclaw_step2_noalloc(ctypes.byref(s), None, None, 1e-5, ctypes.byref(cfl),
                                         None) == _lib.ERR_TOO_LARGE
            assert cfl.value == -1.0


def test_aux_solver_needs_aux_pointer_and_aux_bcs():
    L = _lib.lib()
    s = make_solver_struct(_lib.RP_VC_ACOUSTICS_2D, 8, 8, 0.1, 0.1, [1, 1], [1, 1], [4, 4], 2, 2,
                           0, [])
    assert L.gclaw_check(ctypes.byref(s)) == _lib.ERR_ARG  # no aux array
    s.aux = 0x100000  # any non-null device address passes the host check
    assert L.gclaw_check(ctypes.byref(s)) == 0
    s.aux_bc_lower[0] = 2  # periodic on one side only
    assert L.gclaw_check(ctypes.byref(s)) == _lib.ERR_ARG
    m, mw = ctypes.c_int(), ctypes.c_int()
    assert L.gclaw_rp_shape(_lib.RP_VC_ACOUSTICS_2D, ctypes.byref(m), ctypes.byref(mw)) == 0
    assert (m.value, mw.value) == (3, 2)


def test_fwave_solver_shape_and_checks():
    L = _lib.lib()
    FW = _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D
    m, mw = ctypes.c_int(), ctypes.c_int()
    assert L.gclaw_rp_shape(FW, ctypes.byref(m), ctypes.byref(mw)) == 0
    assert (m.value, mw.value) == (3, 3)
    s = make_solver_struct(FW, 8, 8, 0.1, 0.1, [1, 1], [1, 1], [4] * 3, 2, 2, 0, [9.81])
    assert L.gclaw_check(ctypes.byref(s)) == _lib.ERR_ARG  # no aux array
    s.aux = 0x100000
    assert L.gclaw_check(ctypes.byref(s)) == 0
    s.problem_data[0] = 0.0  # gravity must be positive
    assert L.gclaw_check(ctypes.byref(s)) == _lib.ERR_ARG


def test_split_and_3d_entry_points_refuse_unaligned_or_aliased_states():
    """The split steps (2D and 3D) and the 3D steps move cells as 16-byte
    vectors: state pointers off a 16-byte boundary, aliased state buffers
    and bad step counts are refused before any CUDA call.  The pointer
    values are never dereferenced."""
    from clawpack_gb300.device import make_solver3_struct

    L = _lib.lib()
    P = ctypes.c_void_p
    a, b, c, w = P(0x10000), P(0x20000), P(0x30000), P(0x40000)
    off = P(0x30008)
    s = good_solver()
    assert L.gclaw_step_split(ctypes.byref(s), a, b, off, 0.1, w, None) == _lib.ERR_ARG
    assert L.gclaw_step_split(ctypes.byref(s), a, b, a, 0.1, w, None) == _lib.ERR_ARG
    assert L.gclaw_advance_split(ctypes.byref(s), P(0x10008), b, c, w, 1, None) == _lib.ERR_ARG
    assert L.gclaw_advance_split(ctypes.byref(s), a, b, c, w, -1, None) == _lib.ERR_ARG
    s3 = make_solver3_struct(1, 8, 8, 8, 0.1, 0.1, 0.1, [3] * 3, [3] * 3, [4, 4], 2, 22, 0,
                             [1.0, 4.0, 2.0, 2.0])
    r = ctypes.byref(s3)
    assert L.gclaw3_step_split(r, a, b, off, 0.1, None, w, None) == _lib.ERR_ARG
    assert L.gclaw3_step_split(r, a, b, b, 0.1, None, w, None) == _lib.ERR_ARG
    assert L.gclaw3_step_split(r, a, b, c, 0.0, None, w, None) == _lib.ERR_ARG
    assert L.gclaw3_advance_split(r, a, b, c, None, w, -1, None) == _lib.ERR_ARG
    assert L.gclaw3_step(r, P(0x10008), b, 0.1, c, w, None) == _lib.ERR_ARG
    assert L.gclaw3_advance(r, a, P(0x20008), c, w, 1, None) == _lib.ERR_ARG
    s3.mx = 2000  # (mx + 3)(my + 3)(mz + 3) >= 2^31 once the others follow
    s3.my = s3.mz = 1300
    assert L.gclaw3_check(r) == _lib.ERR_ARG


def test_kernel_family_switches():
    """gclaw_split_kernel, gclaw3_split_kernel and gclaw3_unsplit_kernel
    return the previous setting and ignore values out of range."""
    L = _lib.lib()
    for fn, top in ((L.gclaw_split_kernel, 3), (L.gclaw3_split_kernel, 2),
                    (L.gclaw3_unsplit_kernel, 1)):
        prev = fn(top)
        try:
            assert fn(top + 1) == top      # out of range: unchanged
            assert fn(-1) == top
            assert fn(0) == top
            assert fn(0) == 0
        finally:
            fn(prev)
