"""GPU test of the allocation-free CG entry point.

wap_cg_screened_laplacian_noalloc is for callers that cannot let the library
allocate device memory (a memory pool that has reserved the device, or a
serving loop that cannot take cudaFree's device-wide synchronisation).  It is
called here through the C ABI, twice in a row on different right-hand sides
(its fixed scratch keeps the previous call's contents), and each result is
checked bit for bit against the allocating entry point
wap_cg_screened_laplacian on the same input: both run the same kernels in the
same order with fixed-order FP64 reductions, so their solutions and iteration
counts are identical.  The file name sorts last so a stop-at-first-failure run has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_cg_matches_allocating_entry_point(wapmod, torch_cuda):
    torch = torch_cuda
    L = wapmod.load()
    fn = L.wap_cg_screened_laplacian_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]
    n = 40  # 64,000 voxels, inside the 262,144-voxel capacity
    dims = np.array([n, n, n], np.int32)
    ctx = wapmod.Context(wapmod.make_scan((16, 16, 16), (16, 16), 4), np.zeros(4))
    stream = torch.cuda.Stream()
    try:
        for call, (seed, mode) in enumerate([(11, 0), (12, 1)]):
            rhs = torch.from_numpy(np.random.default_rng(seed).normal(size=(n, n, n)).astype(np.float32)).cuda()
            x_ref = torch.zeros((n, n, n), device="cuda")
            x = torch.zeros((n, n, n), device="cuda")
            # the solvers run on their own streams, which do not wait for torch's
            torch.cuda.synchronize()
            it_ref = ctx.cg_screened_laplacian(dims, 1.0, 0.5, rhs, x_ref, 1e-5, 200, 1e-9, mode)
            ctx.synchronize()
            it = ctypes.c_int(-1)
            rc = fn(stream.cuda_stream, dims.ctypes.data, 1.0, 0.5, rhs.data_ptr(), x.data_ptr(), 1e-5, 200, 1e-9,
                    mode, ctypes.addressof(it))
            stream.synchronize()
            assert rc == wapmod.WAP_OK, "call %d returned %d" % (call, rc)
            assert it.value == it_ref
            assert np.array_equal(x.cpu().numpy(), x_ref.cpu().numpy())
        # a grid beyond the fixed capacity is refused, not truncated
        big = np.array([65, 64, 64], np.int32)
        rc = fn(stream.cuda_stream, big.ctypes.data, 1.0, 0.5, rhs.data_ptr(), x.data_ptr(), 1e-5, 10, 1e-9, 0, None)
        assert rc == 6  # WAP_ETOOBIG
    finally:
        ctx.close()
