"""cbns_diagnostics_noalloc: kinetic energy and enstrophy without any allocation.

This entry point exists for callers that cannot call cudaMalloc while they run
(an in-situ monitor inside another solver's time loop, a framework whose
allocator owns the device budget, a real-time loop).  Such a caller owns its
device buffers already, so this test allocates the state and the 2-double result
up front, as that caller would, then calls the entry point twice in a row
through the C ABI and checks both results against cbns_diagnostics (the
handle-based entry point) to the 1e-13 relative tolerance the diagnostics tests
use.  The output is poisoned with NaN before each call, so each call must write
it; the second call also exercises the scratch array left over from the first.
Free device memory (cudaMemGetInfo) is the same before and after further calls
made once the first call has set up its device, so the calls allocate nothing.
"""
import ctypes
import math

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_BAD_DIMS, CBNS_ERR_INVALID_ARG, CBNS_OK, tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]


def test_noalloc_diagnostics_matches_handle_entry_point():
    import torch

    from cbns3d_cart_mpi_gb300 import _lib
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed

    IM, JM, KM = 40, 36, 32
    p = tgv_params(IM, JM=JM, KM=KM, Re=700.0, Mach=0.2)
    s = Solver(p)
    s.upload_Q(initial_condition_perturbed(p, seed=9, amp=5e-3), 0.0)
    s.step()
    Q = s.download_Q()  # the reference's layout, ghosts filled
    ke_ref, en_ref = s.diagnostics()
    s.close()

    dev = torch.device("cuda", torch.cuda.current_device())
    Q_dev = torch.from_numpy(np.ascontiguousarray(Q).reshape(-1)).to(dev)
    out_dev = torch.empty(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    dx, dy, dz = 2.0 * math.pi / IM, 2.0 * math.pi / JM, 2.0 * math.pi / KM
    lib = _lib.gpu()

    def call_and_check(call):
        out_dev.fill_(float("nan"))
        st = lib.cbns_diagnostics_noalloc(ctypes.c_void_p(Q_dev.data_ptr()), IM, JM, KM, dx, dy, dz,
                                          ctypes.c_void_p(out_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == CBNS_OK, _lib.last_error()
        stream.synchronize()
        ke, en = out_dev.tolist()
        assert abs(ke - ke_ref) <= 1e-13 * abs(ke_ref), (call, ke, ke_ref)
        assert abs(en - en_ref) <= 1e-13 * abs(en_ref), (call, en, en_ref)

    for call in range(2):
        call_and_check(call)
    # The device is set up (symbol address looked up, kernels loaded): further
    # calls must leave free device memory unchanged.
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for call in range(2, 6):
        call_and_check(call)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free_before


def test_noalloc_diagnostics_rejects_what_it_cannot_hold():
    import torch

    from cbns3d_cart_mpi_gb300 import _lib

    dev = torch.device("cuda", torch.cuda.current_device())
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    lib = _lib.gpu()
    ptr = ctypes.c_void_p(buf.data_ptr())
    # 407^3 cells exceed the static scratch (4096 partial sums of 16384 cells);
    # the check happens before any launch, so the small buffer is never read.
    st = lib.cbns_diagnostics_noalloc(ptr, 407, 407, 407, 0.01, 0.01, 0.01, ptr, None)
    assert st == CBNS_ERR_BAD_DIMS
    assert "scratch capacity" in _lib.last_error()
    st = lib.cbns_diagnostics_noalloc(None, 8, 8, 8, 0.1, 0.1, 0.1, ptr, None)
    assert st == CBNS_ERR_INVALID_ARG
