"""Allocation-free dense solve (refeff_complex_lu_solve_device_noalloc) against the
allocating entry point refeff_complex_lu_solve_batched, through the C ABI.

Both run the same FP64 elimination, so the solutions agree to rounding
(tolerance 1e-12 relative to max|X|); two calls in a row must both agree,
which also shows that nothing stale survives in the shared scratch.
"""
import numpy as np
import pytest

from refeff_gb300 import fms

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _systems(seed, n, m, batch):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(batch, n, n)) + 1j * rng.normal(size=(batch, n, n))
    A += np.eye(n) * (2.0 * np.sqrt(n))
    B = rng.normal(size=(batch, n, m)) + 1j * rng.normal(size=(batch, n, m))
    return A, B


def _device(torch, X):
    flat = np.ascontiguousarray(np.stack([x.reshape(-1, order="F") for x in X]))
    return torch.from_numpy(flat).to("cuda")


def _noalloc_solve(torch, A, B):
    batch, n, _ = A.shape
    m = B.shape[2]
    dA, dB = _device(torch, A), _device(torch, B)
    dX = torch.zeros(batch, n * m, dtype=torch.complex128, device="cuda")
    st = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    pv = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fms.complex_lu_solve_device_noalloc(n, m, batch, dA.data_ptr(), dB.data_ptr(), dX.data_ptr(), st.data_ptr(),
                                        pv.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    X = dX.cpu().numpy()
    return np.stack([X[b].reshape((n, m), order="F") for b in range(batch)]), st.cpu().numpy(), pv.cpu().numpy()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("n,m,batch", [(130, 3, 4), (700, 16, 2)])
def test_noalloc_matches_allocating_solve_twice(torch_cuda, n, m, batch):
    ctx = fms.Context(0)
    for call, seed in enumerate([n, n + 1]):
        A, B = _systems(seed, n, m, batch)
        X_ref, st_ref, _ = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
        X, st, pv = _noalloc_solve(torch_cuda, A, B)
        assert list(st) == [0] * batch and list(st_ref) == [0] * batch, call
        assert list(pv) == [0] * batch
        assert np.abs(X - X_ref).max() <= TOL * np.abs(X_ref).max(), call
        assert np.abs(X - np.linalg.solve(A, B)).max() <= 1e-10 * np.abs(X_ref).max()
    ctx.close()


def test_noalloc_on_a_second_device(torch_cuda):
    """The scratch address and the kernels' shared-memory limits are set up per device: a call with device 1
    current must match the allocating solve on device 1 (skipped with one GPU)."""
    if torch_cuda.cuda.device_count() < 2:
        pytest.skip("one GPU")
    with torch_cuda.cuda.device(1):
        ctx = fms.Context(1)
        A, B = _systems(21, 700, 16, 2)
        X_ref, st_ref, _ = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
        X, st, _ = _noalloc_solve(torch_cuda, A, B)
        assert list(st) == [0, 0] and list(st_ref) == [0, 0]
        assert np.abs(X - X_ref).max() <= TOL * np.abs(X_ref).max()
        ctx.close()


def test_noalloc_singular_system_status_matches(torch_cuda):
    ctx = fms.Context(0)
    A, B = _systems(9, 64, 2, 2)
    A[1][:, 7] = 0.0
    A[1][7, :] = 0.0
    _, st_ref, pv_ref = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
    _, st, pv = _noalloc_solve(torch_cuda, A, B)
    assert list(st) == list(st_ref) and st[0] == 0 and st[1] == 9
    assert list(pv) == list(pv_ref) and pv[1] > 0
    ctx.close()


def test_noalloc_rejects_requests_beyond_the_scratch(torch_cuda):
    with pytest.raises(fms.FmsError) as e:
        fms.complex_lu_solve_device_noalloc(2000, 16, 1, 16, 16, 16)
    assert e.value.code == 18
    with pytest.raises(fms.FmsError) as e:
        fms.complex_lu_solve_device_noalloc(300, 8, 64, 16, 16, 16)
    assert e.value.code == 18
