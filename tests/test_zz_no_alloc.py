"""mdg_observe_noalloc through the C ABI, checked against mdg_observe.

The entry point serves callers that cannot allocate device memory (a host
application with its own memory pool, code in a host callback, a caller with
device arrays but no handle): it takes caller-owned device arrays and works in
one fixed static device array.  Here it is called twice in a row on the state
of a handle and must give the observer sums of the allocating entry point
mdg_observe to 1e-12 relative, then reject a particle count above its fixed
maximum.  This file sorts last so a stop-at-first-failure run has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

from tests.helpers import liquid_like

pytestmark = pytest.mark.gpu


def test_observe_noalloc_matches_observe_twice():
    import torch
    from mdacp_gb300 import native
    from mdacp_gb300.manager import MDManager

    q, p, L = liquid_like(0.5, 12, seed=71)
    n = len(q)
    m = MDManager(L, capacity=n, cutoff=2.5, margin=0.5, dt=0.001)
    m.set_state(q, p)
    m.calculate(37)  # positions partly outside the box since the last rebuild
    expected = m.observe_raw()
    qs, ps = m.state()
    m.close()
    q4 = np.zeros((n, 4))
    p4 = np.zeros((n, 4))
    q4[:, :3], p4[:, :3] = qs, ps
    dq = torch.from_numpy(q4).cuda()
    dp = torch.from_numpy(p4).cuda()
    out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    lib = native.load()
    box = (ctypes.c_double * 3)(*[float(x) for x in L])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        out.fill_(float("nan"))
        rc = lib.mdg_observe_noalloc(ctypes.c_void_p(dq.data_ptr()), ctypes.c_void_p(dp.data_ptr()), n, box, 2.5,
                                     ctypes.c_void_p(out.data_ptr()), stream)
        assert rc == native.MDG_OK
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), expected, rtol=1e-12, atol=0.0)

    # above the fixed maximum the call is refused before touching any memory
    rc = lib.mdg_observe_noalloc(ctypes.c_void_p(dq.data_ptr()), ctypes.c_void_p(dp.data_ptr()), (1 << 20) + 1, box,
                                 2.5, ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 3
