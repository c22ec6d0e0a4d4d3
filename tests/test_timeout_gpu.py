"""The bounded-wait failure path of the persistent tensor-core kernels, on a GB300.

The failure is injected on the host (sb_debug_skip_publish): one unit leaves out its published flag
of one SB step, so the units of its replica column wait for a flag nothing sets. With a short wait
limit (sb_set_wait_limit, 1e6 SM cycles, ~0.5 ms) the kernel must give up, let its copies and
contractions finish, free its tensor memory and return a status; the call returns SB_ERR_TIMEOUT
within milliseconds, and the same context then solves normally, bit for bit against the oracle.
Nothing here faults or traps the GPU: every wait in these kernels is bounded.
"""
import time

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu

SB_ERR_TIMEOUT = 7


@pytest.mark.parametrize("operand,jmax", [(sb.OPERAND_FP4, 1), (sb.OPERAND_FP8, 9)], ids=["e2m1", "fp8"])
def test_wait_expires_then_context_solves(operand, jmax):
    n, R, steps, seed = 300, 96, 24, 5
    J = instances.erdos_renyi(n, 0.5, seed=3, jmax=jmax, allow_zero=True)
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC,
                            operand_dtype=operand)
    ctx = sb.Context(0)
    try:
        ctx.solve(prob, prm)  # warm-up: kernels loaded, plan cached
        ctx.set_wait_limit(1_000_000)
        ctx.debug_skip_publish(steps // 2)
        t0 = time.perf_counter()
        with pytest.raises(sb.SBError) as ei:
            ctx.solve(prob, prm)
        wall_ms = 1e3 * (time.perf_counter() - t0)
        assert ei.value.status == SB_ERR_TIMEOUT, str(ei.value)
        assert wall_ms < 500.0, f"timeout path took {wall_ms:.1f} ms"
        # the same context, the default limit again: a normal solve, bit-exact against the oracle
        ctx.set_wait_limit(0)
        res = ctx.solve(prob, prm, want_state=True)
        assert res.field_dtype == ("fp4e2m1" if operand == sb.OPERAND_FP4 else "fp8e4m3")
        x, y = orc.init_uniform(n, R, seed)
        orc.sb_run_f32(2, J, None, x, y, steps, 1.0, prob.default_c0(), 1.25)
        np.testing.assert_array_equal(res.final_x, x)
        np.testing.assert_array_equal(res.final_y, y)
        assert res.energy_check_ok
    finally:
        ctx.close()


def test_wait_limit_arguments():
    ctx = sb.Context(0)
    try:
        with pytest.raises(sb.SBError):
            ctx.set_wait_limit(-1)
        with pytest.raises(sb.SBError):
            ctx.debug_skip_publish(-3)
    finally:
        ctx.close()
