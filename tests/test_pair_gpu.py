"""The CTA-pair form of the E2M1 tensor-core kernel (clusters of two CTAs, tcgen05 cta_group::2),
selected with SB_TC_PAIR=1, against the CPU oracle through the C ABI.

A pair runs one M = 256 MMA per K chunk over two spin tiles: each CTA keeps its own 128 J rows and
stages half of the chunk's replicas. The field and the update are the single-CTA kernel's, so the
trajectories are bit-exact against the oracle; the bounded-wait failure path (a unit that leaves out
its published flag, injected on the host) returns SB_ERR_TIMEOUT and leaves the context usable.
"""
import time

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu


@pytest.fixture
def pair_ctx(monkeypatch):
    monkeypatch.setenv("SB_TC_PAIR", "1")
    ctx = sb.Context(0)  # a fresh context: its engines are created with the variable set
    yield ctx
    ctx.close()


def _oracle(J, h, R, steps, seed, c0, trace=False):
    n = J.shape[0]
    x, y = orc.init_uniform(n, R, seed)
    if trace or n * n * R * steps < 4e8:
        _, tra = orc.sb_run_f32(2, J, h, x, y, steps, 1.0, c0, 1.25, trace=trace, trace_all=trace)
        return x, y, tra
    orc.cpu_run(2, J, h, x, y, steps, 1.0, c0, 1.25)
    return x, y, None


@pytest.mark.parametrize("n,R,steps,jmax", [
    (2000, 1024, 20, 1),  # the batched workload's shape: 16 spin tiles x 8 replica tiles, 64 pairs
    (300, 130, 40, 3),    # spin tiles padded from 3 to 4, replicas padded to 256
    (129, 200, 25, 4),
])
def test_pair_bit_exact(pair_ctx, n, R, steps, jmax):
    J = instances.complete_pm1(n, seed=1234) if jmax == 1 else \
        instances.erdos_renyi(n, 0.6, seed=n + R, jmax=jmax, allow_zero=True)
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=21, field_mode=sb.FIELD_TC,
                            operand_dtype=sb.OPERAND_FP4)
    res = pair_ctx.solve(prob, prm, want_state=True)
    assert res.field_dtype == "fp4e2m1"
    x, y, _ = _oracle(J, None, R, steps, 21, prob.default_c0())
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.final_y, y)
    np.testing.assert_array_equal(res.replica_energies, orc.energies_of_x(J, None, x))
    assert res.energy_check_ok


def test_pair_with_field_and_trace(pair_ctx):
    n, R, steps = 200, 160, 30
    J = instances.complete_pm1(n, seed=12)
    h = np.random.default_rng(3).integers(-2, 3, n).astype(np.float32)
    prob = sb.Problem.from_dense(J, h)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=5, field_mode=sb.FIELD_TC, trace=1,
                            trace_all=1, operand_dtype=sb.OPERAND_FP4)
    res = pair_ctx.solve(prob, prm, want_state=True)
    x, _, tra = _oracle(J, h, R, steps, 5, prob.default_c0(), trace=True)
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.energy_trace_all, tra)


def test_pair_wait_expires_then_context_solves(pair_ctx):
    n, R, steps, seed = 300, 130, 24, 5
    J = instances.erdos_renyi(n, 0.5, seed=3, jmax=1, allow_zero=True)
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC,
                            operand_dtype=sb.OPERAND_FP4)
    pair_ctx.solve(prob, prm)
    pair_ctx.set_wait_limit(1_000_000)
    pair_ctx.debug_skip_publish(steps // 2)
    t0 = time.perf_counter()
    with pytest.raises(sb.SBError) as ei:
        pair_ctx.solve(prob, prm)
    assert ei.value.status == 7, str(ei.value)  # SB_ERR_TIMEOUT
    assert 1e3 * (time.perf_counter() - t0) < 500.0
    pair_ctx.set_wait_limit(0)
    res = pair_ctx.solve(prob, prm, want_state=True)
    x, y, _ = _oracle(J, None, R, steps, seed, prob.default_c0())
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.final_y, y)
