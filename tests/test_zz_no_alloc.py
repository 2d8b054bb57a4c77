"""The SpMV entry point that allocates nothing (blqh_spmv_f32_noalloc).

It exists for callers that cannot call cudaMalloc themselves or let a library
do it (their device memory comes from a host framework's pool, or an
allocation would stall their streams). Here the inputs and outputs are device
buffers owned by the test (torch allocates them, as such a framework would),
and the result is checked against the library's regular SpMV entry point
(blqh_spmv) on two calls in a row. Both accumulate in double-float, with
different summation trees: the tolerance is 1e-12 relative to max |y|, the one
test_double_float_spmv_accuracy uses. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_spmv_matches_regular_spmv():
    torch = pytest.importorskip("torch")
    import blqh_gb300 as B
    from blqh_gb300._lib import check, lib

    b = B.Basis(12, 12, 6, 0, 0)
    H = B.Hamiltonian(b, 1.0, precision=B.VAL_FP32)
    assert not H.is_complex
    rp, col, val = H.csr()
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(rp).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(val.astype(np.float32)).to(dev)
    rng = np.random.default_rng(11)
    for _ in range(2):  # two calls in a row: the built-in scratch keeps the previous call's contents
        x = rng.standard_normal(b.dim)
        d_x = torch.from_numpy(x).to(dev)
        d_y = torch.full((b.dim,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        check(lib().blqh_spmv_f32_noalloc(_p(d_rp), _p(d_col), _p(d_val), b.dim, _p(d_x), _p(d_y), None))
        torch.cuda.synchronize()
        y = d_y.cpu().numpy()
        y_ref = H.spmv(x)
        assert np.all(np.isfinite(y))
        assert np.max(np.abs(y - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))


def test_noalloc_spmv_at_the_size_limit():
    """dim = 2^20, the largest the built-in scratch takes: a synthetic ragged CSR
    (0 to 15 entries per row, empty rows included, random columns) so that every
    thread and warp of the capped grids loops over many rows. Checked against an
    FP64 product with the same FP32 values, relative 1e-12, on two calls in a row."""
    torch = pytest.importorskip("torch")
    sp = pytest.importorskip("scipy.sparse")
    from blqh_gb300._lib import check, lib

    n = 1 << 20
    rng = np.random.default_rng(2)
    lens = rng.integers(0, 16, size=n)
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    col = rng.integers(0, n, size=int(rp[-1])).astype(np.int32)
    val = rng.standard_normal(int(rp[-1])).astype(np.float32)
    A = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    dev = torch.device("cuda", 0)
    d_rp, d_col, d_val = (torch.from_numpy(a).to(dev) for a in (rp, col, val))
    for _ in range(2):
        x = rng.standard_normal(n)
        d_x = torch.from_numpy(x).to(dev)
        d_y = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        check(lib().blqh_spmv_f32_noalloc(_p(d_rp), _p(d_col), _p(d_val), n, _p(d_x), _p(d_y), None))
        torch.cuda.synchronize()
        y = d_y.cpu().numpy()
        y_ref = A @ x
        assert np.all(y[lens == 0] == 0.0)
        assert np.max(np.abs(y - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))


def test_noalloc_spmv_rejects_oversize():
    torch = pytest.importorskip("torch")
    from blqh_gb300._lib import lib

    dev = torch.device("cuda", 0)
    z = torch.zeros(4, dtype=torch.float64, device=dev)
    n = (1 << 20) + 1
    rc = lib().blqh_spmv_f32_noalloc(_p(z), _p(z), _p(z), n, _p(z), _p(z), None)
    assert rc == -1
    assert b"scratch" in lib().blqh_last_error(None)
