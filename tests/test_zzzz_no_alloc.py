"""Allocation-free eigen-solver entry point (forge_gpu_zheevr_noalloc).

It exists for callers that cannot allocate device memory when they call the solver (a pool
or arena owning the GPU, hosts that manage all device buffers); its workspace is a static
device array.  Two calls in a row through the C-ABI must agree with the existing entry point
forge_gpu_zheevr_batch within the FP64 tolerances the other tests use (eigenvalues 1e-12
relative, eigenvector projectors 1e-10), and independently with LAPACK (numpy's eigh) to the
same tolerances.  The file name sorts after every other test file, so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(rt, nbytes):
    p = C.c_void_p()
    assert rt.cudaMalloc(C.byref(p), C.c_size_t(nbytes)) == 0
    return p


def test_noalloc_matches_batch_entry_point_twice(lib):
    import forge_gb300 as fg
    rt = C.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    lib.forge_gpu_zheevr_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.forge_gpu_zheevr_noalloc.restype = C.c_int
    hf = fg.HartreeFock(fg.Setup(ntheta=5, numk=1))          # N = 364 for the existing entry point
    n = hf.N
    iu = n // 2 + 10
    rng = np.random.default_rng(11)
    # the test allocates its own device buffers; the entry point under test allocates nothing
    dA, dw, dZ = _dev(rt, n * n * 16), _dev(rt, iu * 8), _dev(rt, n * iu * 16)
    for call in range(2):
        M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        M = (M + M.conj().T) / 2
        if call == 1:
            M[:10, :10] += np.eye(10) * 3.0          # a different spectrum on the second call
        A = np.asfortranarray(np.tril(M))
        assert rt.cudaMemcpy(dA, A.ctypes.data_as(C.c_void_p), n * n * 16, 1) == 0
        rc = lib.forge_gpu_zheevr_noalloc(dA, n, iu, dw, dZ, None)
        assert rc == 0, lib.forge_gpu_last_error()
        w = np.zeros(iu)
        Z = np.zeros((n, iu), dtype=np.complex128, order="F")
        assert rt.cudaMemcpy(w.ctypes.data_as(C.c_void_p), dw, iu * 8, 2) == 0
        assert rt.cudaMemcpy(Z.ctypes.data_as(C.c_void_p), dZ, n * iu * 16, 2) == 0
        wb, Zb, info = hf.zheevr_batch(A, iu)
        assert info == 0
        assert np.max(np.abs(w - wb[:, 0])) <= 1e-12 * np.max(np.abs(wb))
        k = n // 2 - 9
        Pn = Z[:, :k] @ Z[:, :k].conj().T
        Pb = Zb[:, :k, 0] @ Zb[:, :k, 0].conj().T
        assert np.max(np.abs(Pn - Pb)) <= 1e-10
        # independent of the library's solver: LAPACK eigenvalues and occupied projector
        wl, Zl = np.linalg.eigh(M)
        assert np.max(np.abs(w - wl[:iu])) <= 1e-12 * np.max(np.abs(wl))
        Pl = Zl[:, :k] @ Zl[:, :k].conj().T
        assert np.max(np.abs(Pn - Pl)) <= 1e-10
        assert np.max(np.abs(Z.conj().T @ Z - np.eye(iu))) <= 1e-12
    for p in (dA, dw, dZ):
        rt.cudaFree(p)
    hf.close()


def test_noalloc_rejects_oversized_problem(lib):
    lib.forge_gpu_zheevr_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)
    rc = lib.forge_gpu_zheevr_noalloc(dummy, 513, 10, dummy, dummy, None)
    assert rc < 0
    assert b"exceeds" in lib.forge_gpu_last_error()
