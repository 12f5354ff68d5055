"""The allocation-free gradient entry point, gi_mlp_gradients_noalloc, through
the C ABI.  It serves callers that cannot call cudaMalloc (an arena allocator
owns their device memory, or they are at a memory cap): they pass caller-owned weights, inputs and outputs, and the
library works in a scratch array compiled into it.  This file is collected
last, so that a run that stops at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PIXELS = 8192


def _batch(torch, seed, n):
    rng = np.random.default_rng(seed)
    x = torch.from_numpy(rng.normal(0, 1, (n, 32)).astype(np.float32)).to(torch.bfloat16).cuda()
    t = np.zeros((n, 4), np.float32)
    t[:, :3] = rng.uniform(0, 1, (n, 3))
    t[:, 3] = rng.uniform(0.25, 2.0, n)  # per-pixel loss weight
    s = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return x, torch.from_numpy(t).cuda(), torch.from_numpy(s).cuda()


def _noalloc(gi, torch, params, x, t, s):
    grads = torch.empty(gi.Mlp.PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    st = gi.lib().gi_mlp_gradients_noalloc(C.c_void_p(params.data_ptr()), C.c_void_p(x.data_ptr()),
                                          C.c_void_p(t.data_ptr()), C.c_void_p(s.data_ptr()), x.shape[0],
                                          C.c_void_p(grads.data_ptr()), C.c_void_p(loss.data_ptr()),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, gi.lib().gi_last_error()
    torch.cuda.synchronize()
    return float(loss.item()), grads.cpu().numpy()


def test_gradients_without_allocation_match_the_allocating_entry_point(gi, cuda):
    torch = cuda
    net = gi.Mlp(seed=21)
    params = torch.from_numpy(net.get_params()).cuda()
    # Two calls in a row: a full batch, then a smaller one that leaves stale slots
    # of the first call in the scratch array.
    for seed, n in ((1, MAX_PIXELS), (2, 1000)):
        x, t, s = _batch(torch, seed, n)
        l_ref, g_ref = net.gradients(x, t, scale=s)
        l, g = _noalloc(gi, torch, params, x, t, s)
        assert abs(l - l_ref) <= 1e-4 * abs(l_ref)
        err = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
        print(f"n={n}: loss {l:.6g} vs {l_ref:.6g}, gradient rel err {err:.2e}")
        assert err < 1e-3
        # The fixed-order reduction returns the same bits on a repeated call.
        l2, g2 = _noalloc(gi, torch, params, x, t, s)
        assert l2 == l and np.array_equal(g2, g)


def test_batches_above_the_scratch_limit_are_rejected(gi, cuda):
    torch = cuda
    params = torch.zeros(gi.Mlp.PARAMS, dtype=torch.float32, device="cuda")
    x, t, s = _batch(torch, 3, MAX_PIXELS + 1)
    grads = torch.empty(gi.Mlp.PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    st = gi.lib().gi_mlp_gradients_noalloc(C.c_void_p(params.data_ptr()), C.c_void_p(x.data_ptr()),
                                          C.c_void_p(t.data_ptr()), C.c_void_p(s.data_ptr()), MAX_PIXELS + 1,
                                          C.c_void_p(grads.data_ptr()), C.c_void_p(loss.data_ptr()), None)
    assert st == 1
    assert b"exceeds the allocation-free maximum of 8192" in gi.lib().gi_last_error()
