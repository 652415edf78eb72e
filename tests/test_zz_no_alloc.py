"""GPU test of tsph_hnet_loss_grad_noalloc, the h-network loss/gradient
entry point that allocates no device memory (for callers that reserve all
device memory up front and cannot call cudaMalloc inside their step loop).

It is called through the C ABI on device buffers the test owns, three times
in a row with different inputs -- 5000 samples, then the 16384-sample limit,
then 1000 (fewer warps than the call before, not a multiple of 32, so stale
partials of the larger call would show) -- and each result is checked
against the allocating entry point (tsph_hnet_loss_grad) and against the
FP64 numpy reference at the tolerance the h-network tests use.  Free device
memory is the same before and after a call.  This file sorts last so that a
run stopping at the first failure has run every other test first; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import gasoline_gb300 as g
from oracle import hnet_ref

pytestmark = pytest.mark.gpu

GRAD_REL = 2e-4     # same bar as the h-network gradient test
LOSS_REL = 1e-4


def _fp(t):
    return ctypes.c_void_p(t.data_ptr())


def _bind(lib):
    f = lib.tsph_hnet_loss_grad_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_matches_allocating_entry_point_and_reference():
    torch = pytest.importorskip("torch")
    lib = g.load()
    noalloc = _bind(lib)
    nparam = lib.tsph_hnet_num_params()
    ctx = g.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(11)
    try:
        for n in (5000, 16384, 1000):
            w = rng.normal(0.0, 0.3, nparam).astype(np.float32)
            x = rng.normal(0.0, 1.0, (n, 3)).astype(np.float32)
            y = rng.normal(0.0, 1.0, n).astype(np.float32)
            ctx.hnet_set_params(w)
            loss_alloc, grad_alloc = ctx.hnet_loss_grad(x, y)
            loss_ref, grad_ref = hnet_ref.loss_grad(w.astype(np.float64), x.astype(np.float64),
                                                    y.astype(np.float64))

            w_d = torch.from_numpy(w).to(dev)
            x_d = torch.from_numpy(x.reshape(-1)).to(dev)
            y_d = torch.from_numpy(y).to(dev)
            grad_d = torch.full((nparam,), float("nan"), dtype=torch.float32, device=dev)
            loss_d = torch.full((1,), float("nan"), dtype=torch.float32, device=dev)
            torch.cuda.synchronize(dev)
            rc = noalloc(_fp(w_d), n, _fp(x_d), _fp(y_d), _fp(grad_d), _fp(loss_d),
                         ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0
            torch.cuda.synchronize(dev)
            grad = grad_d.cpu().numpy()
            loss = float(loss_d.cpu().numpy()[0])
            for lref, gref in ((loss_alloc, grad_alloc), (loss_ref, grad_ref)):
                assert loss == pytest.approx(lref, rel=LOSS_REL)
                scale = np.max(np.abs(gref))
                assert np.max(np.abs(grad - gref)) <= GRAD_REL * scale

        # the call itself allocates nothing: free device memory is unchanged
        # across one more call (no torch allocation in between)
        torch.cuda.synchronize(dev)
        free0, _ = torch.cuda.mem_get_info(dev)
        rc = noalloc(_fp(w_d), n, _fp(x_d), _fp(y_d), _fp(grad_d), _fp(loss_d),
                     ctypes.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize(dev)
        free1, _ = torch.cuda.mem_get_info(dev)
        assert rc == 0
        assert free1 == free0

        # more samples than the fixed scratch holds: rejected, nothing launched
        big = torch.zeros(3 * 16385, dtype=torch.float32, device=dev)
        rc = noalloc(_fp(w_d), 16385, _fp(big), _fp(big), _fp(grad_d), _fp(loss_d),
                     ctypes.c_void_p(stream.cuda_stream))
        assert rc == 1
    finally:
        ctx.close()
