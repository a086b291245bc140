"""gfm_adlbl3_noalloc, the line solve for callers that may not allocate.

Code that runs inside a host program owning all device memory (another
framework's caching allocator, a pool sized at start-up, a process under a
device-memory quota) cannot create a gfm_gpu handle, because the handle
allocates its buffers.  gfm_adlbl3_noalloc takes caller-owned device arrays
and keeps its working storage in a fixed array inside the library.  It must
give the same solve as gfm_gpu_adlbl3 in march order with FP64 arithmetic,
and a second call must not be disturbed by what the first one left in that
shared storage, so two different systems are solved back to back.

The caller's arrays are allocated here with torch; the entry point itself
allocates nothing.  This file sorts last so a run that stops at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi, configs
from tests.test_oracle_adi import manufactured

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _class_mask(case, rng):
    ib, ie, jb, je, kb, ke = rng
    m = np.zeros((case.lp, case.np, case.mp), bool)
    m[kb - 1:ke:2, jb - 1:je:2, ib - 1:ie:2] = True
    return m


def test_noalloc_matches_handle_solver_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    case = Case(configs.small_furnace())
    ref = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    ibc = _dev(torch, case.ibcell().astype(np.int16))
    # two systems with different plane shapes, solved one after the other
    for cls, seed in (((0, 0, 0), 7), ((0, 1, 0), 11)):
        ap, as6, bs, x0, _sol, rng, open_ = manufactured(case, cls, seed=seed)
        want = ref.adlbl3(x0, ap, as6, bs, *rng, 2)
        xt, apd, bsd = _dev(torch, x0), _dev(torch, ap), _dev(torch, bs)
        asd = [_dev(torch, a) for a in as6]
        ptrs = (C.c_void_p * 6)(*[a.data_ptr() for a in asd])
        rc = lib.gfm_adlbl3_noalloc(case.mp, case.np, case.lp, ibc.data_ptr(), xt.data_ptr(), apd.data_ptr(),
                                    ptrs, bsd.data_ptr(), *rng, 2, None)
        assert rc == abi.GFM_OK, rc
        torch.cuda.synchronize()
        got = xt.cpu().numpy()
        err = np.abs(got - want)[open_].max() / np.abs(want[open_]).max()
        assert err < 1e-13, (cls, err)
        # positions outside the solved class are left as they were
        outside = ~_class_mask(case, rng)
        assert np.array_equal(got[outside], x0[outside])
    ref.close()


def test_noalloc_rejects_oversized_planes_and_host_pointers():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    ib16 = torch.zeros(16, dtype=torch.int16, device="cuda")
    d = buf.data_ptr()
    ptrs = (C.c_void_p * 6)(*([d] * 6))
    # a 298 x 298-point plane is beyond the 65536-point limit: refused before any device work
    rc = lib.gfm_adlbl3_noalloc(16, 600, 600, ib16.data_ptr(), d, d, ptrs, d, 4, 12, 4, 598, 4, 598, 1, None)
    assert rc == abi.GFM_E_LIMIT
    # host memory where device memory is required
    host = np.zeros(16)
    hp = host.ctypes.data
    rc = lib.gfm_adlbl3_noalloc(16, 16, 16, ib16.data_ptr(), hp, d, ptrs, d, 4, 12, 4, 12, 4, 12, 1, None)
    assert rc == abi.GFM_E_ARG
