"""gfm_adlbl3_noalloc, the line solve for callers that may not allocate.

Code that runs inside a host program owning all device memory (another
framework's caching allocator, a pool sized at start-up, a process under a
device-memory quota) cannot create a gfm_gpu handle, because the handle
allocates its buffers.  gfm_adlbl3_noalloc takes caller-owned device arrays
and keeps its working storage in a fixed array inside the library.  It must
give the same solve as gfm_gpu_adlbl3 in march order with FP64 arithmetic (and
so as the oracle's ADLBL3), and a call must not be disturbed by what an
earlier one left in that shared storage, so different systems are solved back
to back, including one whose plane fills the storage to its limit.

The caller's arrays are allocated here with torch; the entry point itself
allocates nothing.  This file sorts last so a run that stops at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi, configs
from oracle import pyoracle
from oracle.pyoracle import Oracle
from tests.test_oracle_adi import manufactured

pytestmark = pytest.mark.gpu

LIMIT = 65536   # (J,K) points of one plane the fixed working storage holds


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _class_mask(case, rng):
    ib, ie, jb, je, kb, ke = rng
    m = np.zeros((case.lp, case.np, case.mp), bool)
    m[kb - 1:ke:2, jb - 1:je:2, ib - 1:ie:2] = True
    return m


def _noalloc(torch, lib, case, ibc, ap, as6, bs, x0, rng, nim, stream=None):
    xt, apd, bsd = _dev(torch, x0), _dev(torch, ap), _dev(torch, bs)
    asd = [_dev(torch, a) for a in as6]
    ptrs = (C.c_void_p * 6)(*[a.data_ptr() for a in asd])
    sp = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.gfm_adlbl3_noalloc(case.mp, case.np, case.lp, ibc.data_ptr(), xt.data_ptr(), apd.data_ptr(),
                                ptrs, bsd.data_ptr(), *rng, nim, sp)
    assert rc == abi.GFM_OK, rc
    if stream is None:
        torch.cuda.synchronize()
    else:
        stream.synchronize()
    return xt.cpu().numpy()


def _oracle(case, ap, as6, bs, x0, rng, nim):
    o = Oracle(case, adi_mode=abi.GFM_ADI_MARCH)
    xo = x0.copy()
    ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in as6])
    pyoracle.load().gfo_adlbl3(o.o, abi.dptr(xo), abi.dptr(ap), ptrs, abi.dptr(bs), *rng, nim)
    o.close()
    return xo


def _rel(got, want, sel):
    return np.abs(got - want)[sel].max() / np.abs(want[sel]).max()


def test_noalloc_matches_handle_solver_and_oracle_on_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    case = Case(configs.small_furnace())
    ref = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    ibc = _dev(torch, case.ibcell().astype(np.int16))
    side = torch.cuda.Stream()
    # systems with different plane shapes solved one after the other, the
    # last one queued on a stream other than the default one and with a
    # single z-row, which takes the y-line pass alone (Adlbl3.f90:124-130)
    for cls, seed, one_row, stream in (((0, 0, 0), 7, False, None), ((0, 1, 0), 11, False, None),
                                       ((0, 0, 1), 5, True, side)):
        ap, as6, bs, x0, _sol, rng, open_ = manufactured(case, cls, seed=seed)
        if one_row:
            rng = rng[:4] + (rng[4] + 4, rng[4] + 4)
            sel = _class_mask(case, rng) & open_
        else:
            sel = open_
        want = ref.adlbl3(x0, ap, as6, bs, *rng, 2)
        got = _noalloc(torch, lib, case, ibc, ap, as6, bs, x0, rng, 2, stream)
        assert _rel(got, want, sel) < 1e-13, cls
        assert _rel(got, _oracle(case, ap, as6, bs, x0, rng, 2), sel) < 1e-13, cls
        # positions outside the solved range are left as they were
        outside = ~_class_mask(case, rng)
        assert np.array_equal(got[outside], x0[outside])
    ref.close()


def test_noalloc_plane_at_the_storage_limit():
    """A plane of exactly 65536 (J,K) points (256 x 256) fills all four parts
    of the working storage; the solve still matches the oracle's, and a
    smaller system solved right after it is not disturbed by what it left."""
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    case = Case(configs.tiny_furnace(nx=4, ny=256, nz=256))
    ap, as6, bs, x0, _sol, rng, open_ = manufactured(case, (0, 0, 0), seed=13)
    ib, ie, jb, je, kb, ke = rng
    assert ((je - jb) // 2 + 1) * ((ke - kb) // 2 + 1) == LIMIT
    ibc = _dev(torch, case.ibcell().astype(np.int16))
    got = _noalloc(torch, lib, case, ibc, ap, as6, bs, x0, rng, 1)
    assert _rel(got, _oracle(case, ap, as6, bs, x0, rng, 1), open_) < 1e-13
    small = Case(configs.tiny_furnace())
    ap, as6, bs, x0, _sol, rng, open_ = manufactured(small, (1, 0, 0), seed=17)
    ibs = _dev(torch, small.ibcell().astype(np.int16))
    got = _noalloc(torch, lib, small, ibs, ap, as6, bs, x0, rng, 3)
    assert _rel(got, _oracle(small, ap, as6, bs, x0, rng, 3), open_) < 1e-13


def test_noalloc_rejects_oversized_planes_and_host_pointers():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    ib16 = torch.zeros(16, dtype=torch.int16, device="cuda")
    d = buf.data_ptr()
    ptrs = (C.c_void_p * 6)(*([d] * 6))
    # a 257 x 256-point plane is one row beyond the 65536-point limit:
    # refused before any device work
    rc = lib.gfm_adlbl3_noalloc(16, 600, 600, ib16.data_ptr(), d, d, ptrs, d, 4, 12, 4, 516, 4, 514, 1, None)
    assert rc == abi.GFM_E_LIMIT
    # host memory where device memory is required
    host = np.zeros(16)
    hp = host.ctypes.data
    rc = lib.gfm_adlbl3_noalloc(16, 16, 16, ib16.data_ptr(), hp, d, ptrs, d, 4, 12, 4, 12, 4, 12, 1, None)
    assert rc == abi.GFM_E_ARG
