"""swc_mlp_gradient_noalloc: the loss gradient of the learned warm-start network
for callers that cannot allocate device memory when they need it (frameworks
that plan their device memory up front, callers under a fixed memory budget).
It takes device pointers only and keeps its scratch in fixed device arrays, so
it must give the same result as the allocating swc_mlp_gradient, call after
call, although every call reuses (and leaves behind) the same scratch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(n, 8)).astype(np.float32)  # SWC_MLP_IN features
    t = (np.tanh(f[:, 0]) + 0.5 * f[:, 4] - 0.2 * f[:, 1] * f[:, 5]).astype(np.float32)
    norm = np.concatenate([f.mean(0), f.std(0), [t.mean(), t.std()]]).astype(np.float32)
    return f, t, norm


def test_noalloc_gradient_matches_allocating_entry_point(swc_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from swc import _lib, learn

    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    limit = 2048  # SWC_MLP_NOALLOC_MAX_ROWS
    d_grad = torch.empty(learn.N_PARAMS, dtype=torch.float32, device="cuda")
    d_loss = torch.empty(1, dtype=torch.float32, device="cuda")
    # consecutive calls of different sizes share the scratch arrays
    for call, n in enumerate((1500, limit, 700)):
        f, t, norm = _batch(n, seed=call)
        params = learn.init_params(call)
        g_ref, loss_ref = learn.gradient(params, norm, f, t)
        dp, dq = torch.from_numpy(params).cuda(), torch.from_numpy(norm).cuda()
        df, dt = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
        torch.cuda.synchronize()
        rc = L.swc_mlp_gradient_noalloc(dp.data_ptr(), dq.data_ptr(), df.data_ptr(), dt.data_ptr(), n,
                                        d_grad.data_ptr(), d_loss.data_ptr(), stream)
        assert rc == _lib.SWC_OK
        torch.cuda.synchronize()
        g = d_grad.cpu().numpy()
        np.testing.assert_allclose(g, g_ref, rtol=1e-5, atol=1e-6 * np.abs(g_ref).max())
        assert d_loss.item() == pytest.approx(loss_ref, rel=1e-5)
    # a batch above the fixed scratch size is rejected
    f, t, norm = _batch(limit + 1, seed=9)
    df, dt = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    rc = L.swc_mlp_gradient_noalloc(dp.data_ptr(), dq.data_ptr(), df.data_ptr(), dt.data_ptr(), limit + 1,
                                    d_grad.data_ptr(), d_loss.data_ptr(), stream)
    assert rc == _lib.SWC_BAD_ARG
