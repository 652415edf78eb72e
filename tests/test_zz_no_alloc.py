"""GPU test of tsph_hnet_loss_grad_noalloc, the h-network loss/gradient
entry point that allocates no device memory (for callers that reserve all
device memory up front and cannot call cudaMalloc inside their step loop).

It is called through the C ABI on device buffers the test owns, twice in a
row with different inputs, and checked against the allocating entry point
(tsph_hnet_loss_grad) at the tolerance the h-network tests use.  This file
sorts last so that a run stopping at the first failure has run every other
test first; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import gasoline_gb300 as g

pytestmark = pytest.mark.gpu

GRAD_REL = 2e-4     # same bar as the h-network gradient test
LOSS_REL = 1e-4


def _fp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    lib = g.load()
    lib.tsph_hnet_loss_grad_noalloc.restype = ctypes.c_int
    lib.tsph_hnet_loss_grad_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]
    nparam = lib.tsph_hnet_num_params()
    ctx = g.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(11)
    try:
        for n in (5000, 16384):          # two calls in a row, the second at the size limit
            w = rng.normal(0.0, 0.3, nparam).astype(np.float32)
            x = rng.normal(0.0, 1.0, (n, 3)).astype(np.float32)
            y = rng.normal(0.0, 1.0, n).astype(np.float32)
            ctx.hnet_set_params(w)
            loss_ref, grad_ref = ctx.hnet_loss_grad(x, y)

            w_d = torch.from_numpy(w).to(dev)
            x_d = torch.from_numpy(x.reshape(-1)).to(dev)
            y_d = torch.from_numpy(y).to(dev)
            grad_d = torch.full((nparam,), float("nan"), dtype=torch.float32, device=dev)
            loss_d = torch.full((1,), float("nan"), dtype=torch.float32, device=dev)
            torch.cuda.synchronize(dev)
            rc = lib.tsph_hnet_loss_grad_noalloc(_fp(w_d), n, _fp(x_d), _fp(y_d), _fp(grad_d),
                                                 _fp(loss_d), ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0
            torch.cuda.synchronize(dev)
            grad = grad_d.cpu().numpy()
            loss = float(loss_d.cpu().numpy()[0])
            assert loss == pytest.approx(loss_ref, rel=LOSS_REL)
            scale = np.max(np.abs(grad_ref))
            assert np.max(np.abs(grad - grad_ref)) <= GRAD_REL * scale
        # more samples than the fixed scratch holds: rejected, nothing launched
        big = torch.zeros(3 * 16385, dtype=torch.float32, device=dev)
        rc = lib.tsph_hnet_loss_grad_noalloc(_fp(w_d), 16385, _fp(big), _fp(big), _fp(grad_d),
                                             _fp(loss_d), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 1
    finally:
        ctx.close()
