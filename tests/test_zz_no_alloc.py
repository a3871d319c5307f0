"""The allocation-free OC entry point (tg_oc_noalloc) through the C ABI.

tg_oc_noalloc serves callers that cannot allocate device memory themselves
(their device memory belongs to their own pool allocator, or they must not
change the device's allocation state while their other work runs): the
caller passes device buffers for inputs and outputs, and the library's only
extra memory is a static device array.  Two calls in a row must reproduce
the allocating entry point (tg_oc_raw) and the CPU oracle's oc_top88 with the
same move limit and bisection bounds, which also shows that the shared
scratch array left behind by one call does not leak into the next; one call
passes no element flags.  This file is named so that pytest collects it
last."""
import ctypes as C

import numpy as np
import pytest

from oracle import topopt as O

pytestmark = pytest.mark.gpu


def _inputs(rng, n):
    x = rng.uniform(0.05, 0.95, n)
    dc = -rng.uniform(0.01, 3.0, n)
    dv = rng.uniform(0.5, 1.5, n)
    flags = rng.integers(0, 3, n).astype(np.int8)
    flags[rng.uniform(size=n) < 0.8] = 0
    return x, dc, dv, flags


def test_noalloc_oc_matches_allocating_entry_and_oracle(gpu_lib):
    torch = pytest.importorskip("torch")
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.optimizer import oc_top88
    lib = _lib.load()
    rng = np.random.default_rng(11)
    dev = torch.device("cuda", 0)
    # (n, move, l1, l2, with flags)
    calls = [(200_003, 0.2, 0.0, 1e9, True), (65_536, 0.1, 1e-3, 1e8, False),
             (4_099, 0.2, 0.0, 1e9, True)]
    for call, (n, move, l1, l2, with_flags) in enumerate(calls):
        x, dc, dv, flags = _inputs(rng, n)
        fl = flags if with_flags else None
        g = 0.1 * call - 0.05
        xref, gtref = oc_top88(x, 0.5, dc, dv, g, el_flags=fl, move=move, l1=l1, l2=l2)
        xo, gto, nso = O.oc_top88(x, dc, dv, g, move=move, l1=l1, l2=l2, el_flags=fl)
        xd = torch.from_numpy(x).to(dev)
        dcd = torch.from_numpy(dc).to(dev)
        dvd = torch.from_numpy(dv).to(dev)
        fld = torch.from_numpy(flags).to(dev) if with_flags else None
        out = torch.empty(n, dtype=torch.float64, device=dev)
        gt = C.c_double()
        nsteps = C.c_int32()
        torch.cuda.synchronize()
        rc = lib.tg_oc_noalloc(n, xd.data_ptr(), dcd.data_ptr(), dvd.data_ptr(), g,
                               fld.data_ptr() if fld is not None else None, move, l1, l2,
                               out.data_ptr(), C.byref(gt), C.byref(nsteps), None)
        assert rc == 0, lib.tg_noalloc_last_error().decode()
        torch.cuda.synchronize()
        xn = out.cpu().numpy()
        np.testing.assert_allclose(xn, xref, rtol=0, atol=1e-13)
        # the allocating entry screens each bisection decision in FP32 (with an
        # error bound, FP64 where it cannot decide); the allocation-free one
        # evaluates every step in FP64: same decisions, the same densities
        np.testing.assert_array_equal(xn, xref)
        np.testing.assert_allclose(gt.value, gtref, rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(xn, xo, rtol=0, atol=1e-13)
        np.testing.assert_allclose(gt.value, gto, rtol=1e-9, atol=1e-12)
        assert nsteps.value == nso


def test_noalloc_rejects_oversize(gpu_lib):
    from topoptlab_gb300 import _lib
    lib = _lib.load()
    gt = C.c_double()
    ns = C.c_int32()
    rc = lib.tg_oc_noalloc(_lib.TG_NOALLOC_MAX_N + 1, 1, 1, 1, 0.0, None, 0.2, 0.0, 1e9, 1,
                           C.byref(gt), C.byref(ns), None)
    assert rc == _lib.TG_EINVAL
    assert "exceeds" in lib.tg_noalloc_last_error().decode()
