"""sb_dsb_solve_noalloc — the dSB solve for callers that cannot allocate device memory.

Such callers (code inside a host process that owns the device-memory budget, or code that must
not pay cudaMalloc's synchronisation, latency or out-of-memory risk mid-work) pass every input and
output as a device buffer they own; the entry point keeps its scratch in a fixed array inside the
library. Here it is called through the C ABI on buffers PyTorch allocated, twice in a row, and
its outputs must equal those of sb_solve on the same problem (tensor-core dSB, FP8 operands):
bit for bit, the tolerance every tensor-core dSB test uses.
"""
import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from annealing_gb300.sb import lib

pytestmark = pytest.mark.gpu


def _device_buffers(torch, J, h, R, n):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(J).to(dev), torch.from_numpy(h).to(dev),
            torch.empty((R, n), dtype=torch.float32, device=dev),
            torch.empty((R, n), dtype=torch.float32, device=dev),
            torch.empty(R, dtype=torch.float64, device=dev))


def test_noalloc_matches_sb_solve_on_two_calls():
    torch = pytest.importorskip("torch")
    n, R, steps, seed = 300, 130, 40, 21
    J = instances.erdos_renyi(n, 0.6, seed=7, jmax=3, allow_zero=True)
    h = np.random.default_rng(5).integers(-2, 3, n).astype(np.float32)
    ctx = sb.Context(0)
    prob = sb.Problem.from_dense(J, h)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC,
                            operand_dtype=sb.OPERAND_FP8)
    ref = ctx.solve(prob, prm, want_state=True)
    assert ref.field_dtype == "fp8e4m3"
    dJ, dh, dx, dy, de = _device_buffers(torch, J, h, R, n)
    stream = torch.cuda.current_stream(0).cuda_stream
    for _ in range(2):
        for buf in (dx, dy, de):
            buf.fill_(7.0)  # every output must be overwritten
        st = lib().sb_dsb_solve_noalloc(dJ.data_ptr(), dh.data_ptr(), n, R, steps, seed, 1.25, 1.0,
                                        prob.default_c0(), dx.data_ptr(), dy.data_ptr(),
                                        de.data_ptr(), stream)
        assert st == 0, lib().sb_last_error(None)
        np.testing.assert_array_equal(dx.cpu().numpy(), ref.final_x)
        np.testing.assert_array_equal(dy.cpu().numpy(), ref.final_y)
        np.testing.assert_array_equal(de.cpu().numpy(), ref.replica_energies)
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    n, R = 64, 8
    J = instances.complete_pm1(n, seed=1)
    dJ, dh, dx, dy, de = _device_buffers(torch, J, np.zeros(n, np.float32), R, n)
    stream = torch.cuda.current_stream(0).cuda_stream
    for big_n, big_r, big_s in ((4096, R, 10), (n, 2048, 10), (n, R, 100000)):
        st = lib().sb_dsb_solve_noalloc(dJ.data_ptr(), None, big_n, big_r, big_s, 1, 1.25, 1.0, 0.01,
                                        dx.data_ptr(), dy.data_ptr(), de.data_ptr(), stream)
        assert st == 1
        assert b"limits are n <= 2048" in lib().sb_last_error(None)
