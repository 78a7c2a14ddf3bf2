"""The conjugate gradient entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc when they solve -- a fixed
memory pool or budget, a loop that must not touch the allocator, or device
buffers owned by another framework.  Here the caller's buffers are torch
tensors: the matrix (full-row CSR), right-hand side and solution are handed
to nlgpu_cg_solve_noalloc as device pointers, and its work vectors come from
the library's fixed scratch array.  Its result must match the existing
nlgpu_cg_solve (host buffers, same identity preconditioner) within the
solution tolerance of the parity tests, on two calls in a row (the second
call finds the first call's leftovers in the shared scratch array).

Collected last on purpose (file name), so a failure here comes after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

SOLUTION_RTOL = 1e-10


def full_rows(rp, col, val, n):
    """Full-row CSR (both triangles, sorted columns) of an upper-stored symmetric matrix."""
    rows = np.repeat(np.arange(n), np.diff(rp))
    off = col != rows
    r = np.concatenate([rows, col[off]])
    c = np.concatenate([col, rows[off]])
    v = np.concatenate([val, val[off]])
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    frp = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=n))]).astype(np.int64)
    return frp, c.astype(np.int32), v.astype(np.float64)


def test_noalloc_cg_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    from nonlocal_gb300 import _lib as L
    from nonlocal_gb300 import build
    from nonlocal_gb300 import thermal as T
    build.build()
    lib = L.load()
    assert L.device_count() > 0, "no CUDA device visible"
    fx = gc.load("b12_fastpoly")
    rp, col, val, b = fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"], fx["rhs"]
    n = b.shape[0]
    assert n <= 65536   # NLGPU_NOALLOC_MAX_ROWS

    ctx = T.Context()
    x_ref, rep = T.conjugate_gradient(ctx, (rp, col, val), b, tolerance=1e-12, max_iterations=20000)
    assert rep.residual <= 1e-12

    frp, fcol, fval = full_rows(rp, col, val, n)
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(frp).to(dev)
    d_col = torch.from_numpy(fcol).to(dev)
    d_val = torch.from_numpy(fval).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev)
    for call in range(2):
        d_x = torch.zeros(n, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        iterations, residual = ctypes.c_int64(), ctypes.c_double()
        L.check(lib.nlgpu_cg_solve_noalloc(None, n, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                           d_b.data_ptr(), d_x.data_ptr(), 1e-12, 20000, ctypes.byref(iterations),
                                           ctypes.byref(residual)))
        x = d_x.cpu().numpy()
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err < SOLUTION_RTOL, f"call {call}: relative difference {err}"
        assert residual.value <= 1e-10, f"call {call}: residual {residual.value}"
        assert abs(iterations.value - rep.iterations) <= 3, (call, iterations.value, rep.iterations)


def test_noalloc_rejects_sizes_beyond_the_maximum():
    from nonlocal_gb300 import _lib as L
    lib = L.load()
    it, res = ctypes.c_int64(), ctypes.c_double()
    rc = lib.nlgpu_cg_solve_noalloc(None, 65537, 1, 1, 1, 1, 1, 1e-10, 10, ctypes.byref(it), ctypes.byref(res))
    assert rc == 1   # NLGPU_ERR_ARG, before touching any pointer


def _device_system(torch, name="b12_fastpoly"):
    fx = gc.load(name)
    rp, col, val, b = fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"], fx["rhs"]
    n = b.shape[0]
    frp, fcol, fval = full_rows(rp, col, val, n)
    dev = torch.device("cuda:0")
    return (n, torch.from_numpy(frp).to(dev), torch.from_numpy(fcol).to(dev), torch.from_numpy(fval).to(dev),
            torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev))


def _call(lib, n, d_rp, d_col, d_val, d_b, d_x, tol, maxit):
    iterations, residual = ctypes.c_int64(), ctypes.c_double()
    rc = lib.nlgpu_cg_solve_noalloc(None, n, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_b.data_ptr(),
                                    d_x.data_ptr(), tol, maxit, ctypes.byref(iterations), ctypes.byref(residual))
    return rc, iterations.value, residual.value


def test_noalloc_reports_no_convergence_at_the_iteration_cap():
    """A cap of 5 iterations cannot reach 1e-12: the call says so (status
    NLGPU_ERR_NO_CONVERGENCE) and still fills x, the count and the residual."""
    torch = pytest.importorskip("torch")
    from nonlocal_gb300 import _lib as L
    lib = L.load()
    n, d_rp, d_col, d_val, d_b = _device_system(torch)
    d_x = torch.zeros(n, dtype=torch.float64, device=d_b.device)
    rc, its, res = _call(lib, n, d_rp, d_col, d_val, d_b, d_x, 1e-12, 5)
    assert rc == 6, rc   # NLGPU_ERR_NO_CONVERGENCE
    assert its == 5 and 1e-12 < res < 1.0
    assert torch.count_nonzero(d_x).item() > 0


def test_noalloc_zero_rhs_and_converged_start():
    """b = 0 gives x = 0 whatever the starting guess; a starting guess that
    already solves the system takes no iteration and reports |b - A x| / |b|
    recomputed from it."""
    torch = pytest.importorskip("torch")
    from nonlocal_gb300 import _lib as L
    lib = L.load()
    n, d_rp, d_col, d_val, d_b = _device_system(torch)
    zero_b = torch.zeros_like(d_b)
    d_x = torch.ones(n, dtype=torch.float64, device=d_b.device)
    rc, its, res = _call(lib, n, d_rp, d_col, d_val, zero_b, d_x, 1e-12, 100)
    assert rc == 0 and its == 0 and res == 0.0
    assert torch.count_nonzero(d_x).item() == 0
    d_x = torch.zeros(n, dtype=torch.float64, device=d_b.device)
    rc, its1, res1 = _call(lib, n, d_rp, d_col, d_val, d_b, d_x, 1e-12, 20000)
    assert rc == 0 and res1 <= 1e-10
    x1 = d_x.clone()
    rc, its2, res2 = _call(lib, n, d_rp, d_col, d_val, d_b, d_x, 1e-8, 20000)
    assert rc == 0 and its2 == 0
    assert abs(res2 - res1) <= 1e-3 * res1 + 1e-15
    assert torch.equal(d_x, x1)
