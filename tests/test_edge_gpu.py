"""Edge cases of the tensor-core paths against the CPU oracle (bit-exact dSB, through the C ABI).

Tiny and ragged shapes (one spin, one replica, spin and replica tiles cut short, K padding), zero
couplings, zero steps, the largest shape whose couplings stay resident in shared memory as E2M1,
the first size past it (FP8 operands), and grouped batches holding such instances.
"""
import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu

OPERAND = {"fp4e2m1": sb.OPERAND_FP4, "fp8e4m3": sb.OPERAND_FP8, "fp6e2m3": sb.OPERAND_FP6}


def oracle(J, h, R, steps, seed, c0):
    x, y = orc.init_uniform(J.shape[0], R, seed)
    if J.shape[0] ** 2 * R * steps < 4e8:
        orc.sb_run_f32(2, J, h, x, y, steps, 1.0, c0, 1.25)
    else:
        orc.cpu_run(2, J, h, x, y, steps, 1.0, c0, 1.25)  # same operation order, multithreaded
    return x, y


def couplings(n, kind, seed):
    if kind == "zero":
        return np.zeros((n, n), np.float32)
    if n == 1:
        return np.zeros((1, 1), np.float32)
    return instances.erdos_renyi(n, 0.5, seed=seed, jmax=3, allow_zero=True)


def check(res, J, h, x, y):
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.final_y, y)
    e = orc.energies_of_x(J, h, x)
    np.testing.assert_array_equal(res.replica_energies, e)
    assert res.energy_check_ok and res.best_energy == e.min()
    s = np.where(x[res.best_replica] > 0, 1, -1).astype(np.int8)
    np.testing.assert_array_equal(res.best_spins, s)


@pytest.mark.parametrize("dtype", ["fp4e2m1", "fp8e4m3"])
@pytest.mark.parametrize("n,R,steps,kind,with_h", [
    (1, 1, 10, "er", True),      # one spin, one replica: every tile almost all padding
    (2, 1, 10, "er", False),
    (3, 33, 12, "er", True),     # replica tile cut one past 32
    (127, 65, 12, "er", False),  # spin tile cut one short
    (129, 64, 12, "er", True),   # one spin into a second tile
    (256, 130, 12, "er", False), # K exactly one E2M1 chunk
    (257, 40, 12, "er", True),   # one spin into the next E2M1 chunk
    (200, 48, 15, "zero", True), # no couplings: the field is h alone
    (150, 32, 0, "er", True),    # zero steps: energies of the initial state
])
def test_tensor_core_edge_shapes(ctx, dtype, n, R, steps, kind, with_h):
    J = couplings(n, kind, seed=n + 7)
    h = np.random.default_rng(n).integers(-2, 3, n).astype(np.float32) if with_h else None
    prob = sb.Problem.from_dense(J, h)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=31, field_mode=sb.FIELD_TC,
                            operand_dtype=OPERAND[dtype])
    res = ctx.solve(prob, prm, want_state=True)
    assert res.field_mode == sb.FIELD_TC and res.field_dtype == dtype
    x, y = oracle(J, h, R, steps, 31, prob.default_c0())
    check(res, J, h, x, y)


def test_largest_resident_e2m1_shape(ctx):
    """N = 2304 (nine 256-spin chunks of J per unit in shared memory), R = 1024: 144 units."""
    n, R, steps = 2304, 1024, 6
    J = instances.complete_pm1(n, seed=5)
    prob = sb.Problem.from_dense(J)
    res = ctx.solve(prob, sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=9, field_mode=sb.FIELD_TC),
                    want_state=True)
    assert res.field_dtype == "fp4e2m1"
    x, y = oracle(J, None, R, steps, 9, prob.default_c0())
    check(res, J, None, x, y)


def test_past_the_resident_shape_falls_back_to_fp8(ctx):
    """N = 2400 does not fit the E2M1 kernel's shared memory: the automatic choice is FP8."""
    n, R, steps = 2400, 256, 6
    J = instances.complete_pm1(n, seed=6)
    prob = sb.Problem.from_dense(J)
    res = ctx.solve(prob, sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=4, field_mode=sb.FIELD_TC),
                    want_state=True)
    assert res.field_dtype == "fp8e4m3"
    x, y = oracle(J, None, R, steps, 4, prob.default_c0())
    check(res, J, None, x, y)
    with pytest.raises(sb.SBError) as e:
        ctx.solve(prob, sb.Params.default(sb.DSB, steps=steps, replicas=R, field_mode=sb.FIELD_TC,
                                          operand_dtype=sb.OPERAND_FP4))
    assert e.value.status == 6


@pytest.mark.parametrize("dtype", ["fp4e2m1", "fp8e4m3", "fp6e2m3"])
def test_batch_with_tiny_and_empty_instances(ctx, dtype):
    ns, kinds = [1, 2, 5, 300, 255, 64], ["er", "er", "zero", "er", "zero", "er"]
    Js = [couplings(n, k, seed=i) for i, (n, k) in enumerate(zip(ns, kinds))]
    hs = [np.random.default_rng(i).integers(-2, 3, n).astype(np.float32) if i % 2 == 0 else None
          for i, n in enumerate(ns)]
    probs = [sb.Problem.from_dense(J, h) for J, h in zip(Js, hs)]
    R, steps, seed = 40, 20, 77
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC,
                            operand_dtype=OPERAND[dtype])
    res = ctx.batch(probs, prm, want_state=True).run()
    for k, (J, h, p, r) in enumerate(zip(Js, hs, probs, res)):
        assert r.field_dtype == dtype
        x, y = oracle(J, h, R, steps, seed + k, p.default_c0())
        check(r, J, h, x, y)
