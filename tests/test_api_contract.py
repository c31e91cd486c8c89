"""CPU tests of the C ABI: exported symbols, argument validation and error
codes (compared with the reference's own API layer when it was built into
oracle/_ref), error strings and plan-time decisions.  No kernel runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

import aclfft as A
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"ACLFFT_API\s+[\w\s\*]*?\b(aclfft\w+)\s*\(", txt)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = A.lib()
    names = _declared("cann_ops_fft.h") + _declared("aclfft_ext.h") + _declared("aclfft_ops.h")
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_header_surface_is_kept():
    """Every function of the reference's plan API header and of its
    per-operator headers is declared here with the same name."""
    root = O.reference_root()
    if not os.path.exists(os.path.join(root, "include", "cann_ops_fft.h")):
        pytest.skip("reference tree not present")
    pat = r"ACLFFT_API\s+[\w\s\*]*?\b(aclfft\w+)\s*\("
    ref = set(re.findall(pat, open(os.path.join(root, "include", "cann_ops_fft.h")).read()))
    assert ref <= set(_declared("cann_ops_fft.h"))
    ops = set()
    for h in ("src/fft1_d/fft1_d.h", "src/rfft1_d/rfft1_d.h", "src/irfft1_d/irfft1_d.h", "src/fft2_d/fft2_d.h"):
        ops |= set(re.findall(r"aclError\s+(aclfft\w+)\s*\(", open(os.path.join(root, h)).read()))
    assert len(ops) >= 20
    assert ops <= set(_declared("aclfft_ops.h")), ops - set(_declared("aclfft_ops.h"))


def _ref_lib():
    path = O.ref_lib_path()
    if path is None:
        pytest.skip("reference API layer not built (oracle/_ref)")
    L = ctypes.CDLL(path)
    for name in ("aclfftPlan1d", "aclfftPlan2d", "aclfftPlan3d"):
        getattr(L, name).argtypes = [ctypes.POINTER(ctypes.c_void_p)] + [ctypes.c_int] * 4
    L.aclfftCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    L.aclfftMakePlan1d.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [ctypes.c_void_p]
    L.aclfftMakePlan2d.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [ctypes.c_void_p]
    L.aclfftExecC2C.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.aclfftExecR2C.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.aclfftExecC2R.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.aclfftDestroy.argtypes = [ctypes.c_void_p]
    L.aclfftSetStream.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.aclfftGetErrorString.argtypes = [ctypes.c_int]
    L.aclfftGetErrorString.restype = ctypes.c_char_p
    return L


TYPES = [A.C2C, A.R2C, A.C2R, A.Z2Z, A.D2Z, A.Z2D, 0, 0x2B, -1]
PLAN1D_ARGS = [
    (nx, t, b, d)
    for nx in (0, -5, 1, 2, 7, 128, 255, 256, 300, 4096, 262144, 524288, (1 << 27), (1 << 27) + 1)
    for t in TYPES
    for b in (0, -1, 1, 128)
    for d in (0, 1, 2, -1)
]


def _plan1d_code(L, args):
    h = ctypes.c_void_p()
    code = L.aclfftPlan1d(ctypes.byref(h), *args)
    if code == 0:
        assert h.value
        L.aclfftDestroy(h)
    else:
        assert not h.value
    return code


def test_plan1d_error_codes_match_reference():
    """Every code matches the reference's, except that double precision is
    planned here (documented widening): where the reference rejects Z2Z/D2Z/
    Z2D with NOT_SUPPORTED before looking at the size, this library applies
    the size rules and plans the transform."""
    ref = _ref_lib()
    mine = A.lib()
    diffs = []
    for args in PLAN1D_ARGS:
        a, b = _plan1d_code(ref, args), _plan1d_code(mine, args)
        if a == A.NOT_SUPPORTED and args[1] in (A.Z2Z, A.D2Z, A.Z2D) and b in (A.SUCCESS, A.INVALID_SIZE):
            continue
        if a != b:
            diffs.append((args, a, b))
    assert not diffs, diffs[:20]


def test_plan2d_error_codes_match_reference_within_its_domain():
    """The reference only accepts C2C of {32,64,128}^2; elsewhere it returns
    NOT_SUPPORTED where this library plans the transform (documented
    widening: any C2C size, R2C/C2R, and double precision).  Every other
    code must match."""
    ref = _ref_lib()
    mine = A.lib()
    for nx in (0, 32, 64, 128, 2048, 7):
        for ny in (-1, 32, 128, 256):
            for b in (0, 1, 8):
                for t in TYPES:
                    h1, h2 = ctypes.c_void_p(), ctypes.c_void_p()
                    a = ref.aclfftPlan2d(ctypes.byref(h1), b, nx, ny, t)
                    c = mine.aclfftPlan2d(ctypes.byref(h2), b, nx, ny, t)
                    if a == 0:
                        ref.aclfftDestroy(h1)
                    if c == 0:
                        mine.aclfftDestroy(h2)
                    if a == A.NOT_SUPPORTED and c == 0 and t in (A.C2C, A.R2C, A.C2R, A.Z2Z, A.D2Z, A.Z2D):
                        continue
                    assert a == c, (b, nx, ny, t, a, c)


def test_plan3d_error_codes_match_reference_outside_its_stub():
    """The reference's MakePlan3d is a stub (NOT_IMPLEMENTED after Plan3d's
    argument checks, lib/fft_plan_api.cpp:127-150); here every type plans.
    Argument-check codes must match."""
    ref = _ref_lib()
    mine = A.lib()
    for nx, ny, nz in ((0, 8, 8), (8, -1, 8), (8, 8, 0), (8, 8, 8), (1, 1, 1), (7, 64, 3000)):
        for t in TYPES:
            h1, h2 = ctypes.c_void_p(), ctypes.c_void_p()
            a = ref.aclfftPlan3d(ctypes.byref(h1), nx, ny, nz, t)
            c = mine.aclfftPlan3d(ctypes.byref(h2), nx, ny, nz, t)
            if a == 0:
                ref.aclfftDestroy(h1)
            if c == 0:
                mine.aclfftDestroy(h2)
            if a == A.NOT_IMPLEMENTED:
                assert c == 0, (nx, ny, nz, t, c)  # every valid type is planned here
                continue
            assert a == c, (nx, ny, nz, t, a, c)
    h = ctypes.c_void_p()
    assert mine.aclfftCreate(ctypes.byref(h)) == 0
    assert mine.aclfftMakePlan3d(h, 4, 4, 4, A.C2C, None) == 0
    assert mine.aclfftMakePlan3d(h, 4, 4, 4, A.C2C, None) == A.INVALID_VALUE  # already made
    mine.aclfftDestroy(h)
    assert mine.aclfftMakePlan3d(None, 4, 4, 4, A.C2C, None) == A.INVALID_VALUE


def test_exec_entry_checks_match_reference():
    """Exec validation runs before any device work: NULL plan/buffers,
    uninitialised plans, type mismatch and bad direction."""
    ref = _ref_lib()
    mine = A.lib()
    buf = np.zeros(64, dtype=np.complex64)
    p = buf.ctypes.data
    for L in (ref, mine):
        pass
    results = {}
    for name, L in (("ref", ref), ("mine", mine)):
        r = []
        r.append(L.aclfftExecC2C(None, p, p, -1))
        h = ctypes.c_void_p()
        L.aclfftCreate(ctypes.byref(h))
        r.append(L.aclfftExecC2C(h, p, p, -1))  # not initialised
        r.append(L.aclfftExecR2C(h, p, p))
        L.aclfftDestroy(h)
        for t in (A.C2C, A.R2C, A.C2R):
            h = ctypes.c_void_p()
            assert L.aclfftPlan1d(ctypes.byref(h), 8, t, 1, 0) == 0
            r.append(L.aclfftExecC2C(h, None, p, -1))
            r.append(L.aclfftExecC2C(h, p, None, 1))
            r.append(L.aclfftExecR2C(h, None, p))
            r.append(L.aclfftExecC2R(h, p, None))
            r.append(L.aclfftExecC2C(h, p, p, 0) if t == A.C2C else L.aclfftExecC2C(h, p, p, -1))
            r.append(L.aclfftExecC2C(h, p, p, 7) if t == A.C2C else L.aclfftExecR2C(h, p, p) if t == A.C2R else 0)
            r.append(L.aclfftExecC2R(h, p, p) if t == A.R2C else 0)
            L.aclfftDestroy(h)
        results[name] = r
    assert results["ref"] == results["mine"]


def test_makeplan_twice_and_create_null():
    mine = A.lib()
    assert mine.aclfftCreate(None) == A.INVALID_VALUE
    h = ctypes.c_void_p()
    assert mine.aclfftCreate(ctypes.byref(h)) == 0
    assert mine.aclfftMakePlan1d(h, 64, A.C2C, 1, 0, None) == 0
    assert mine.aclfftMakePlan1d(h, 64, A.C2C, 1, 0, None) == A.INVALID_VALUE
    assert mine.aclfftSetStream(h, None) == 0
    assert mine.aclfftSetStream(None, None) == A.INVALID_VALUE
    assert mine.aclfftDestroy(h) == 0
    assert mine.aclfftDestroy(None) == A.INVALID_VALUE


def test_stubs_return_not_implemented():
    """SetStride stays a stub, as in the reference (lib/fft_utils_api.cpp:
    90-94).  The double-precision execs, stubs in the reference
    (lib/fft_exec_api.cpp:87-116), are built here and check their arguments
    like the FP32 ones."""
    mine = A.lib()
    h = ctypes.c_void_p()
    assert mine.aclfftSetStride(h, 2) == A.NOT_IMPLEMENTED
    assert mine.aclfftExecZ2Z(h, None, None, -1) == A.INVALID_VALUE
    assert mine.aclfftExecD2Z(h, None, None) == A.INVALID_VALUE
    assert mine.aclfftExecZ2D(h, None, None) == A.INVALID_VALUE
    for t in (A.R2C, A.C2R, A.D2Z, A.Z2D):
        hp = ctypes.c_void_p()
        assert mine.aclfftPlan3d(ctypes.byref(hp), 8, 8, 8, t) == A.SUCCESS
        mine.aclfftDestroy(hp)
    buf = np.zeros(64, dtype=np.complex128)
    with A.Plan.plan1d(16, A.Z2Z, 2) as p:
        assert mine.aclfftExecZ2Z(p.handle, buf.ctypes.data, buf.ctypes.data, 7) == A.INVALID_VALUE
        assert mine.aclfftExecD2Z(p.handle, buf.ctypes.data, buf.ctypes.data) == A.INVALID_TYPE
        assert mine.aclfftExecC2C(p.handle, buf.ctypes.data, buf.ctypes.data, -1) == A.INVALID_TYPE
    with A.Plan.plan1d(16, A.D2Z, 2) as p:
        assert mine.aclfftExecZ2D(p.handle, buf.ctypes.data, buf.ctypes.data) == A.INVALID_TYPE
    with A.Plan.plan1d(256, A.D2Z, 2, A.VERTICAL) as p:
        assert not p.info().supported  # real transforms are horizontal


def test_version_queries():
    """aclfftGetVersion / aclfftGetProperty (stubs in the reference,
    lib/fft_utils_api.cpp:95-109) report this library's version."""
    mine = A.lib()
    v = ctypes.c_int()
    assert mine.aclfftGetVersion(None) == A.INVALID_VALUE
    assert mine.aclfftGetVersion(ctypes.byref(v)) == A.SUCCESS
    parts = []
    for prop in (0, 1, 2):
        x = ctypes.c_int(-1)
        assert mine.aclfftGetProperty(prop, ctypes.byref(x)) == A.SUCCESS
        parts.append(x.value)
    assert v.value == parts[0] * 10000 + parts[1] * 100 + parts[2]
    assert mine.aclfftGetProperty(3, ctypes.byref(v)) == A.INVALID_TYPE
    assert mine.aclfftGetProperty(0, None) == A.INVALID_VALUE


def test_work_area_queries():
    """aclfftGetSize1d/2d estimate the work area without creating device
    state and agree with aclfftGetSize / MakePlan's *workSize of the made
    plan; argument checks follow MakePlan's."""
    mine = A.lib()
    h = ctypes.c_void_p()
    assert mine.aclfftCreate(ctypes.byref(h)) == 0
    sz = ctypes.c_size_t()
    assert mine.aclfftGetSize1d(None, 64, A.C2C, 1, ctypes.byref(sz)) == A.INVALID_VALUE
    assert mine.aclfftGetSize1d(h, 64, A.C2C, 1, None) == A.INVALID_VALUE
    assert mine.aclfftGetSize1d(h, 0, A.C2C, 1, ctypes.byref(sz)) == A.INVALID_SIZE
    assert mine.aclfftGetSize1d(h, 64, A.C2C, 0, ctypes.byref(sz)) == A.INVALID_SIZE
    assert mine.aclfftGetSize1d(h, 64, 0x2B, 1, ctypes.byref(sz)) == A.INVALID_TYPE
    assert mine.aclfftGetSize1d(h, 64, A.Z2Z, 1, ctypes.byref(sz)) == A.SUCCESS  # double precision is planned
    assert mine.aclfftGetSize2d(h, 64, 64, A.D2Z, ctypes.byref(sz)) == A.SUCCESS
    assert mine.aclfftGetSize1d(h, (1 << 27) + 1, A.C2C, 1, ctypes.byref(sz)) == A.INVALID_SIZE
    assert mine.aclfftGetSize3d(h, 8, 8, 8, A.R2C, ctypes.byref(sz)) == A.SUCCESS
    assert mine.aclfftGetSize3d(h, 8, 0, 8, A.C2C, ctypes.byref(sz)) == A.INVALID_SIZE
    assert mine.aclfftGetSize3d(h, 8, 8, 8, A.C2C, None) == A.INVALID_VALUE
    assert mine.aclfftGetSize(h, ctypes.byref(sz)) == A.INVALID_PLAN  # not made yet
    mine.aclfftDestroy(h)
    cases = [(4096, A.C2C, 256), (3000, A.R2C, 4096), (1024, A.C2R, 16), (1 << 20, A.C2C, 4), (1 << 25, A.R2C, 2),
             (46200, A.C2C, 3), (999, A.R2C, 5), (4096, A.Z2Z, 64), (3000, A.D2Z, 8), (999, A.Z2D, 3)]
    for n, t, b in cases:
        est = ctypes.c_size_t()
        made = ctypes.c_size_t()
        q = ctypes.c_void_p()
        assert mine.aclfftCreate(ctypes.byref(q)) == 0
        assert mine.aclfftGetSize1d(q, n, t, b, ctypes.byref(est)) == 0
        assert mine.aclfftMakePlan1d(q, n, t, b, 0, ctypes.byref(made)) == 0
        assert mine.aclfftGetSize(q, ctypes.byref(sz)) == 0
        assert est.value == made.value == sz.value, (n, t, b, est.value, made.value, sz.value)
        mine.aclfftDestroy(q)
    for nx, ny in ((2048, 2048), (64, 128), (7, 3000)):
        for t in (A.C2C, A.R2C, A.C2R):
            est = ctypes.c_size_t()
            with A.Plan.plan2d(1, nx, ny, t) as p:
                assert mine.aclfftGetSize2d(p.handle, nx, ny, t, ctypes.byref(est)) == 0
                assert est.value == p.work_size()
    for dims in ((64, 64, 64), (5, 3000, 7), (512, 512, 512)):
        est = ctypes.c_size_t()
        with A.Plan.plan3d(*dims) as p:
            assert mine.aclfftGetSize3d(p.handle, *dims, A.C2C, ctypes.byref(est)) == 0
            assert est.value == p.work_size()
    # a long transform needs a work area between its passes
    with A.Plan.plan1d(1 << 20, A.C2C, 4) as p:
        assert p.work_size() > 0


def test_auto_allocation_and_work_area_contract():
    """SetAutoAllocation before MakePlan is recorded; SetWorkArea needs a
    made plan, a 256-byte aligned pointer and device memory (host memory is
    refused; no device is needed to check that)."""
    mine = A.lib()
    assert mine.aclfftSetAutoAllocation(None, 0) == A.INVALID_VALUE
    h = ctypes.c_void_p()
    assert mine.aclfftCreate(ctypes.byref(h)) == 0
    assert mine.aclfftSetWorkArea(h, None) == A.INVALID_PLAN
    assert mine.aclfftSetAutoAllocation(h, 0) == 0
    ws = ctypes.c_size_t()
    assert mine.aclfftMakePlan1d(h, 1 << 20, A.C2C, 2, 0, ctypes.byref(ws)) == 0
    assert ws.value > 0
    host = np.zeros(ws.value // 4 + 64, dtype=np.float32)
    addr = host.ctypes.data
    aligned = (addr + 255) // 256 * 256
    assert mine.aclfftSetWorkArea(h, aligned + 8) == A.UNALIGNED_DATA
    assert mine.aclfftSetWorkArea(h, aligned) == A.INVALID_VALUE
    assert mine.aclfftSetWorkArea(h, None) == 0
    assert mine.aclfftSetAutoAllocation(h, 1) == 0
    assert mine.aclfftDestroy(h) == 0


def test_error_strings_match_reference():
    mine = A.lib()
    try:
        ref = _ref_lib()
    except pytest.skip.Exception:
        ref = None
    for code in list(range(0, 20)) + [-1, 100]:
        s = A.error_string(code)
        assert s
        if ref is not None:
            assert ref.aclfftGetErrorString(code).decode() == s


def test_norm_mode_extension():
    p = A.Plan.plan1d(64, A.C2C)
    for m in range(4):
        p.set_norm(m)
    with pytest.raises(A.AclfftError):
        p.set_norm(4)
    v = ctypes.c_int()
    assert A.lib().aclfftGetNormMode(p.handle, ctypes.byref(v)) == 0 and v.value == 3
    assert A.lib().aclfftSetNormMode(None, 0) == A.INVALID_PLAN


@pytest.mark.parametrize(
    "n,typ,batch,dim",
    [(4096, A.C2C, 256, 0), (3000, A.R2C, 4096, 0), (1024, A.C2R, 4096, 0), (65536, A.C2C, 64, 0),
     (16384, A.C2C, 64, 0), (46200, A.C2C, 1, 0), (1 << 27, A.C2C, 1, 0), (256, A.C2C, 128, 1),
     (262144, A.C2C, 4, 1), (999, A.R2C, 1, 0), (1025, A.C2R, 4, 0), (1, A.C2C, 1, 0), (2310, A.C2C, 1, 0),
     (5040, A.R2C, 1, 0), (25200, A.R2C, 1, 0), (1 << 25, A.R2C, 2, 0)],
)
def test_plan_decisions(n, typ, batch, dim):
    """Plan-time factorisation: every on-chip transform's radices multiply to
    its length, and the on-chip length divides the transform (bit-exact
    integer checks of the planner, no GPU)."""
    p = A.Plan.plan1d(n, typ, batch, dim)
    info = p.info()
    assert info.supported == 1
    rad = list(info.radix)[: info.nradix]
    assert int(np.prod(rad)) == info.onchip_length
    half = n // 2 if (typ != A.C2C and n % 2 == 0) else n
    assert half % info.onchip_length == 0
    assert all(r <= 47 for r in rad)
    assert info.threads_per_transform >= 1


def test_unsupported_lengths_plan_but_do_not_execute():
    """Like the reference, a length with a prime factor > 47 plans fine and is
    rejected at exec time (NOT_IMPLEMENTED); no device work is attempted."""
    p = A.Plan.plan1d(53 * 7, A.C2C)
    assert p.info().supported == 0
    buf = np.zeros(53 * 7, dtype=np.complex64)
    assert A.lib().aclfftExecC2C(p.handle, buf.ctypes.data, buf.ctypes.data, -1) == A.NOT_IMPLEMENTED
    pv = A.Plan.plan1d(256, A.R2C, 4, A.VERTICAL)
    assert A.lib().aclfftExecR2C(pv.handle, buf.ctypes.data, buf.ctypes.data) == A.NOT_IMPLEMENTED


def _sizes_for_bounds():
    sizes = set()
    for n in range(1, 130):
        sizes.add(n)
    for n in (210, 240, 250, 255, 256, 420, 512, 999, 1000, 1023, 1024, 1025, 1500, 1536, 2048, 2100, 2310, 3000,
              4096, 5040, 6561, 8190, 8192, 12288, 13312, 13500, 15625, 16384, 16807, 25200, 26624, 32768, 46200,
              65536, 100000, 131072, 1 << 20, 3 ** 13, 1 << 22, 1 << 25, 1 << 27, 47 * 43 * 41, 17 * 19 * 1024):
        sizes.add(n)
    return sorted(sizes)


@pytest.mark.parametrize("typ", [A.C2C, A.R2C, A.C2R, A.Z2Z, A.D2Z, A.Z2D])
def test_every_launch_stays_in_bounds(typ):
    """Host replay of each planned launch's indexing against its buffers."""
    for n in _sizes_for_bounds():
        for b in (1, 3, 64):
            if n * b > (1 << 28):
                continue
            p = A.Plan.plan1d(n, typ, b)
            if p.info().supported:
                p.check()
            p.destroy()


def test_vertical_and_2d_launches_stay_in_bounds():
    for n in (256, 512, 4096, 65536, 262144):
        for b in (1, 3, 128, 263168):
            if n * b > (1 << 28):
                continue
            with A.Plan.plan1d(n, A.C2C, b, A.VERTICAL) as p:
                p.check()
    for nx, ny in ((32, 32), (64, 128), (128, 32), (2048, 2048), (7, 3000), (4096, 4096), (1, 5), (17, 19),
                   (100000, 3), (3, 100000), (1, 1), (5, 1), (2, 16384), (3, 1 << 20)):
        for t in (A.C2C, A.R2C, A.C2R):
            with A.Plan.plan2d(2, nx, ny, t) as p:
                if p.info().supported:
                    p.check()
    for dims in ((1, 1, 1), (2, 2, 2), (64, 64, 64), (5, 3000, 7), (7, 5, 3000), (3000, 7, 5), (256, 256, 256),
                 (1, 64, 1), (16, 1, 65536), (4, 5000, 6)):
        for t in (A.C2C, A.R2C, A.C2R, A.Z2Z, A.D2Z, A.Z2D):
            with A.Plan.plan3d(*dims, t) as p:
                assert p.info().supported, (dims, t)
                p.check()


def test_precision_mode_extension():
    """aclfftSetPrecisionMode: validation, re-plan of a made plan, which
    lengths get tensor-core launches, and their launch bounds (no GPU)."""
    assert A.lib().aclfftSetPrecisionMode(None, 1) == A.INVALID_PLAN
    p = A.Plan.plan1d(4096, A.C2C, 256)
    assert p.precision() == A.PREC_FP32 and p.info().tc_stages == 0
    assert A.lib().aclfftSetPrecisionMode(p.handle, 3) == A.INVALID_VALUE
    assert A.lib().aclfftSetPrecisionMode(p.handle, -1) == A.INVALID_VALUE
    p.set_precision(A.PREC_TF32X3)
    assert p.precision() == A.PREC_TF32X3 and p.info().tc_stages == 2
    p.set_precision(A.PREC_FP32)
    assert p.info().tc_stages == 0
    p.destroy()
    # set before MakePlan
    h = ctypes.c_void_p()
    assert A.lib().aclfftCreate(ctypes.byref(h)) == 0
    assert A.lib().aclfftSetPrecisionMode(h, A.PREC_BF16X3) == 0
    ws = ctypes.c_size_t()
    assert A.lib().aclfftMakePlan1d(h, 65536, A.C2C, 64, 0, ctypes.byref(ws)) == 0
    assert ws.value == 65536 * 64 * 8
    A.lib().aclfftDestroy(h)
    expect = {64: 1, 256: 1, 4096: 2, 16384: 2, 65536: 2, 1024: 0, 512: 0, 3000: 0, 128: 0, 1 << 20: 0}
    for prec in (A.PREC_TF32X3, A.PREC_BF16X3):
        for n, tc in expect.items():
            for b in (1, 3, 13, 64):
                with A.Plan.plan1d(n, A.C2C, b) as q:
                    q.set_precision(prec)
                    assert q.info().tc_stages == tc, (n, b, prec)
                    assert q.check() == "ok"
    # R2C/C2R, VERTICAL and 2D plans keep the FP32 kernels
    for args in ((4096, A.R2C, 4, 0), (4096, A.C2R, 4, 0), (4096, A.C2C, 4, A.VERTICAL)):
        with A.Plan.plan1d(*args) as q:
            q.set_precision(A.PREC_TF32X3)
            assert q.info().tc_stages == 0
    with A.Plan.plan2d(2, 256, 256, A.C2C) as q:
        q.set_precision(A.PREC_TF32X3)
        assert q.info().tc_stages == 0


def test_tc_index_maps_match_numpy_emulation():
    """The tensor-core pass's row maps (stage A rows (n_a, t), stage B rows
    (k_b, t)), its real-embedded DFT matrix and the two-pass 4-step split,
    restated in numpy at FP64 and compared with the FP64 oracle."""
    def bmat(R):
        K = 2 * R
        j = np.arange(R)
        ang = 2 * np.pi * ((np.outer(j, j)) % R) / R
        c, s = np.cos(ang), np.sin(ang)
        B = np.zeros((K, K))
        B[:R, :R], B[:R, R:], B[R:, :R], B[R:, R:] = c, s, -s, c   # rows: output re/im; cols: input re/im
        return B

    def tc_pass(inp, L, nseq, S, ind, ins, inn, outd, outs, outn, outer, out):
        R = int(round(L ** 0.5))
        TS = 128 // R
        B = bmat(R)
        twl = np.exp(-2j * np.pi * np.arange(L) / L)
        m = np.arange(128)
        ra, rt = m // TS, m % TS
        for q0 in range(0, nseq, TS):
            nv = min(TS, nseq - q0)
            bb, s0 = q0 // S, q0 % S
            stg = np.zeros((TS, L), complex)
            for t in range(nv):
                stg[t] = inp[bb * ind + (s0 + t) * ins + np.arange(L) * inn]
            x = stg[rt[:, None], ra[:, None] + R * np.arange(R)[None, :]]
            D = np.concatenate([x.real, x.imag], 1) @ B.T
            y = (D[:, :R] + 1j * D[:, R:]) * twl[ra[:, None] * np.arange(R)[None, :]]
            A2 = np.zeros((128, 2 * R))
            rows = np.arange(R)[None, :] * TS + rt[:, None]
            A2[rows, ra[:, None]] = y.real
            A2[rows, R + ra[:, None]] = y.imag
            D2 = A2 @ B.T
            z = D2[:, :R] + 1j * D2[:, R:]
            for mm in range(128):
                kb, t = mm // TS, mm % TS
                if t >= nv:
                    continue
                s = (q0 + t) % S
                k = kb + R * np.arange(R)
                v = z[mm]
                if outer > 1:
                    v = v * np.exp(-2j * np.pi * ((s * k) % outer) / outer)
                out[bb * outd + s * outs + k * outn] = v

    rng = np.random.default_rng(4)
    for n, b in ((64, 19), (256, 13), (4096, 2)):
        x = rng.standard_normal(n * b) + 1j * rng.standard_normal(n * b)
        out = np.zeros(n * b, complex)
        if n <= 256:
            tc_pass(x, n, b, b, 0, n, 1, 0, n, 1, 1, out)
        else:
            L1, L2 = 64, 64
            ws = np.zeros(n * b, complex)
            tc_pass(x, L1, b * L2, L2, n, 1, L2, n, 1, L2, n, ws)
            tc_pass(ws, L2, b * L1, L1, n, L2, 1, n, 1, L1, 1, out)
        e = O.errors(out, O.c2c(x.reshape(b, n), -1))
        assert e["rel_l2"] < 1e-13, (n, b, e)


@pytest.mark.parametrize("variant", ["0", "1", "2"])
def test_codelet_variants_and_cluster_choices_stay_in_bounds(variant, monkeypatch):
    """Every specialised build of a length (OPS_FFT_CODELET_VARIANT) and both
    kernel families of the short cluster lengths (batches below and above
    OPS_FFT_CLUSTER_MAXBATCH) pass the host replay of their launches."""
    monkeypatch.setenv("OPS_FFT_CODELET_VARIANT", variant)
    for n in (256, 512, 1024, 2048, 3000, 4096, 8192):
        for typ in (A.C2C, A.R2C, A.C2R):
            for b in (7, 1500):
                with A.Plan.plan1d(n, typ, b) as p:
                    assert p.check() == "ok"
    with A.Plan.plan1d(4096, A.C2C, 256) as p:       # default: the row codelet at every batch
        assert p.info().cluster_ctas == 0 and p.check() == "ok"
    monkeypatch.setenv("OPS_FFT_CLUSTER_MAXBATCH", "1024")
    for b, want in ((1024, True), (1025, False)):
        with A.Plan.plan1d(4096, A.C2C, b) as p:
            assert (p.info().cluster_ctas > 0) == want
            assert p.check() == "ok"
    monkeypatch.setenv("OPS_FFT_COLTILE_VARIANT", variant)
    with A.Plan.plan2d(3, 2048, 2048, A.C2C) as p:
        assert p.check() == "ok"


def test_butterflies_match_fp64_dft():
    """Every in-register butterfly the kernels use (radix 1-48: hand-derived
    small radices, symmetric-pair odd primes, prime-factor splits of coprime
    composites such as 6, 10, 12, 15 and decimation-in-time splits such as 8,
    9, 16), evaluated on the host with the device's rounding, against an FP64
    DFT: relative error within a few FP32 ulps times log R."""
    mine = A.lib()
    rng = np.random.default_rng(48)
    for R in range(1, 49):
        x = (rng.standard_normal(R) + 1j * rng.standard_normal(R)).astype(np.complex64)
        out = np.empty(R, dtype=np.complex64)
        assert mine.aclfftDebugButterfly(R, x.ctypes.data, out.ctypes.data) == A.SUCCESS, R
        ref = np.fft.fft(x.astype(np.complex128))
        err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert err < 2e-7 * max(1.0, np.log2(R)) * 2, (R, err)
    buf = np.zeros(4, dtype=np.complex64)
    assert mine.aclfftDebugButterfly(0, buf.ctypes.data, buf.ctypes.data) == A.INVALID_SIZE
    assert mine.aclfftDebugButterfly(49, buf.ctypes.data, buf.ctypes.data) == A.INVALID_SIZE
