"""sb_dsb_solve_noalloc — the dSB solve for callers that cannot allocate device memory.

Such callers (code inside a host process that owns the device-memory budget, or code that must
not pay cudaMalloc's synchronisation, latency or out-of-memory risk mid-work) pass every input and
output as a device buffer they own; the entry point keeps its scratch in a fixed array inside the
library. Here it is called through the C ABI on buffers PyTorch allocated, twice in a row, and
its outputs must equal those of sb_solve on the same problem (tensor-core dSB with FP8 operands;
the entry point runs packed E2M1 operands when the couplings allow it, which give the same bits):
bit for bit, the tolerance every tensor-core dSB test uses. The cases cover the largest shape the
scratch array holds (n = 2048, 1024 replicas: 128 units, whose flags fill the most control bytes),
zero steps, no fields (d_h = NULL), and couplings that need FP8 rather than E2M1.
"""
import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from annealing_gb300.sb import lib

pytestmark = pytest.mark.gpu


def _device_buffers(torch, J, h, R, n):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(J).to(dev), None if h is None else torch.from_numpy(h).to(dev),
            torch.empty((R, n), dtype=torch.float32, device=dev),
            torch.empty((R, n), dtype=torch.float32, device=dev),
            torch.empty(R, dtype=torch.float64, device=dev))


def _call(dJ, dh, n, R, steps, seed, c0, dx, dy, de, stream):
    return lib().sb_dsb_solve_noalloc(dJ.data_ptr(), None if dh is None else dh.data_ptr(), n, R, steps,
                                      seed, 1.25, 1.0, c0, dx.data_ptr(), dy.data_ptr(), de.data_ptr(),
                                      stream)


CASES = [
    # n, R, steps, coupling bound, with fields
    pytest.param(300, 130, 40, 3, True, id="n300-r130-e2m1"),
    pytest.param(300, 130, 40, 9, True, id="n300-r130-fp8"),
    pytest.param(2048, 1024, 12, 1, False, id="n2048-r1024-largest-noh"),
    pytest.param(2048, 1024, 0, 1, True, id="n2048-r1024-zero-steps"),
]


@pytest.mark.parametrize("n,R,steps,jmax,with_h", CASES)
def test_noalloc_matches_sb_solve_on_two_calls(n, R, steps, jmax, with_h):
    torch = pytest.importorskip("torch")
    seed = 21
    if jmax == 1:
        J = instances.complete_pm1(n, seed=7)
    else:
        J = instances.erdos_renyi(n, 0.6, seed=7, jmax=jmax, allow_zero=True)
    h = np.random.default_rng(5).integers(-2, 3, n).astype(np.float32) if with_h else None
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
        st = _call(dJ, dh, n, R, steps, seed, prob.default_c0(), dx, dy, de, stream)
        assert st == 0, lib().sb_last_error(None)
        np.testing.assert_array_equal(dx.cpu().numpy(), ref.final_x)
        np.testing.assert_array_equal(dy.cpu().numpy(), ref.final_y)
        np.testing.assert_array_equal(de.cpu().numpy(), ref.replica_energies)
    ctx.close()


def test_noalloc_rejects_inexact_couplings_before_solving():
    """A coupling no operand type holds exactly (0.5 here) is rejected by the scan that runs before
    the solve, at the largest shape, and the next call on the same array still succeeds."""
    torch = pytest.importorskip("torch")
    n, R = 2048, 1024
    J = instances.complete_pm1(n, seed=3)
    J[5, 9] = J[9, 5] = 0.5
    dJ, dh, dx, dy, de = _device_buffers(torch, J, None, R, n)
    stream = torch.cuda.current_stream(0).cuda_stream
    st = _call(dJ, dh, n, R, 16384, 1, 0.01, dx, dy, de, stream)
    assert st == 6  # SB_ERR_UNSUPPORTED
    assert b"integers with |J| <= 16" in lib().sb_last_error(None)
    J[5, 9] = J[9, 5] = 17.0
    dJ.copy_(torch.from_numpy(J))
    assert _call(dJ, dh, n, R, 10, 1, 0.01, dx, dy, de, stream) == 6
    J[5, 9] = J[9, 5] = 1.0
    dJ.copy_(torch.from_numpy(J))
    assert _call(dJ, dh, n, R, 4, 1, 0.01, dx, dy, de, stream) == 0, lib().sb_last_error(None)
    assert np.isfinite(de.cpu().numpy()).all()


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
