"""The allocation-free moments entry point (kpm_moments_diag_noalloc).

It serves callers that cannot let a library allocate device memory (cudaMalloc
may synchronize the device; frameworks that own all device memory cannot
accept hidden allocations). The caller passes device buffers for the matrix,
the two vector blocks and the output; the recursion's scratch is a fixed array
inside the library. This test builds those buffers with torch, calls the entry
point twice in a row through the C ABI, and checks both results against the
allocating entry point kpm_moments_diag on the same Hamiltonian and starters.
It lives in its own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _padded_ell(h2, dtype):
    """H~ as padded row-major ELL; FP32 types hold each value as (hi, lo) FP32 parts."""
    h2 = sp.csr_matrix(h2)
    h2.sort_indices()
    n = h2.shape[0]
    w = int(np.max(np.diff(h2.indptr)))
    col = np.repeat(np.arange(n, dtype=np.int32)[:, None], w, axis=1)
    val = np.zeros((n, w), np.complex128 if np.iscomplexobj(h2.data) else np.float64)
    for r in range(n):
        s, e = h2.indptr[r], h2.indptr[r + 1]
        col[r, :e - s] = h2.indices[s:e]
        val[r, :e - s] = h2.data[s:e]
    if np.dtype(dtype) in (np.dtype(np.float32), np.dtype(np.complex64)):
        hi = val.astype(dtype)
        lo = (val - hi.astype(val.dtype)).astype(dtype)
        val = np.stack([hi, lo], axis=-1)
    else:
        val = val.astype(dtype)[..., None]
    return col, np.ascontiguousarray(val), w


@pytest.mark.parametrize("dtype,num_vectors,tol", [(np.float64, 4, 1e-10), (np.float32, 8, 1e-5),
                                                   (np.float64, 1, 1e-10)])
def test_noalloc_matches_allocating_entry_point(dtype, num_vectors, tol):
    torch = pytest.importorskip("torch")
    from pybinding_gb300 import _native, lattice as L

    model = L.graphene_flake(3000, onsite_modifiers=[L.anderson_disorder(1.0, 5)])
    h = model.hamiltonian.astype(dtype)
    n = h.shape[0]
    M = 130
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.0, 9.0)))
    a, b = eng.scaling_factors()
    rng = np.random.default_rng(11)
    starters = np.where(rng.integers(0, 2, (num_vectors, n)) == 0, -1.0, 1.0).astype(dtype)
    ref = eng.moments_diag(M, starters[None])[0]  # (num_vectors, M), complex
    eng.close()

    h2 = (sp.csr_matrix(h, dtype=np.float64) - b * sp.identity(n, format="csr")) * (2.0 / a)
    col, val, w = _padded_ell(h2, dtype)
    dev = torch.device("cuda")
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(val.view(np.uint8).reshape(-1)).to(dev)
    lib = _native.lib()
    code = _native.SCALAR_CODE[np.dtype(dtype)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):  # the scratch keeps the previous call's contents: both calls must agree
        r0 = torch.from_numpy(np.ascontiguousarray(starters.T)).to(dev)  # [rows][K]
        r1 = torch.empty_like(r0)
        out = torch.full((num_vectors, M, 2), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.kpm_moments_diag_noalloc(code, n, w, C.c_void_p(d_col.data_ptr()), C.c_void_p(d_val.data_ptr()),
                                          num_vectors, C.c_void_p(r0.data_ptr()), C.c_void_p(r1.data_ptr()), M,
                                          C.c_void_p(out.data_ptr()), stream)
        assert rc == 0, lib.kpm_last_error().decode()
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        got = o[..., 0] + 1j * o[..., 1]
        err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        assert err <= tol, err


def test_noalloc_rejects_oversized_problem():
    from pybinding_gb300 import _native
    lib = _native.lib()
    fake = C.c_void_p(1 << 20)  # never dereferenced: the size check fails first
    rc = lib.kpm_moments_diag_noalloc(1, 1000, 4, fake, fake, 64, fake, fake, 100000, fake, None)
    assert rc == _native.KPM_ERR_VALUE
    assert "too large for the fixed scratch" in lib.kpm_last_error().decode()
