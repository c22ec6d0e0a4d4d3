"""Grouped tensor-core batches (sb_batch_*): every instance bit-exact against the CPU oracle.

Instances whose couplings are integers |J| <= 4 run packed E2M1 operands, others packed E2M3 (J / 4
in six bits against signs of +-4); FP8 E4M3 on request. All three give the same integer fields.
"""
import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu


def make_instances(ns, jmax=4, with_h=(2,)):
    out = []
    for k, n in enumerate(ns):
        J = instances.erdos_renyi(n, 0.3 + 0.1 * (k % 5), seed=50 + k, jmax=jmax, allow_zero=jmax > 1)
        h = np.random.default_rng(k).integers(-3, 4, n).astype(np.float32) if k in with_h else None
        out.append((J, h))
    return out


@pytest.mark.parametrize("R,jmax,odt,dtype", [
    (64, 4, sb.OPERAND_AUTO, "fp4e2m1"), (32, 4, sb.OPERAND_AUTO, "fp4e2m1"), (100, 4, sb.OPERAND_AUTO, "fp4e2m1"),
    (32, 1, sb.OPERAND_AUTO, "fp4e2m1"),
    (64, 16, sb.OPERAND_AUTO, "fp6e2m3"), (100, 16, sb.OPERAND_AUTO, "fp6e2m3"), (32, 9, sb.OPERAND_AUTO, "fp6e2m3"),
    (128, 16, sb.OPERAND_AUTO, "fp6e2m3"), (64, 4, sb.OPERAND_FP6, "fp6e2m3"),
    (64, 4, sb.OPERAND_FP8, "fp8e4m3"), (100, 16, sb.OPERAND_FP8, "fp8e4m3")])
def test_batch_matches_oracle(ctx, R, jmax, odt, dtype):
    # odd sizes: a last E2M1 byte with one spin, a last E2M3 group of sixteen with a few spins,
    # padded K chunks, partial spin and replica tiles
    ns = [64, 100, 129, 301, 513, 1000]
    insts = make_instances(ns, jmax=jmax)
    probs = [sb.Problem.from_dense(J, h) for J, h in insts]
    steps, seed = 30, 100
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC, operand_dtype=odt)
    batch = ctx.batch(probs, prm, want_state=True)
    res = batch.run()
    assert all(r.field_dtype == dtype for r in res)
    for k, ((J, h), p, r) in enumerate(zip(insts, probs, res)):
        x, y = orc.init_uniform(J.shape[0], R, seed + k)
        orc.sb_run_f32(2, J, h, x, y, steps, 1.0, p.default_c0(), 1.25)
        np.testing.assert_array_equal(r.final_x, x, err_msg=f"instance {k}")
        np.testing.assert_array_equal(r.final_y, y, err_msg=f"instance {k}")
        np.testing.assert_array_equal(r.replica_energies, orc.energies_of_x(J, h, x))
        assert r.energy_check_ok and r.best_energy_i64 == r.best_energy
    again = batch.run()
    for r, r2 in zip(res, again):
        np.testing.assert_array_equal(r.final_x, r2.final_x)
    batch.close()


def test_batch_rejects_real_couplings(ctx):
    J, h = instances.gaussian(64, seed=1)
    prm = sb.Params.default(sb.DSB, steps=10, replicas=32, field_mode=sb.FIELD_TC)
    with pytest.raises(sb.SBError) as e:
        ctx.batch([sb.Problem.from_dense(J, h)], prm)
    assert e.value.status == 6


def test_batch_profile_reports_step_kernel_time(ctx):
    probs = [sb.Problem.from_dense(J, h) for J, h in make_instances([256, 700])]
    prm = sb.Params.default(sb.DSB, steps=12, replicas=64, field_mode=sb.FIELD_TC, profile=1)
    res = ctx.batch(probs, prm).run()
    assert res[0].kernel_ms_avg > 0 and res[0].steps_per_launch == 1


def test_batch_mixed_operands_per_instance(ctx):
    """A batch mixing couplings |J| <= 4 and |J| <= 9 runs two operand buckets: the first instances on
    packed E2M1, the others on packed E2M3, each bit-exact against the oracle, in one run."""
    ns = [64, 129, 300, 513, 700, 1000]
    insts = []
    for k, n in enumerate(ns):
        jmax = 4 if k % 2 == 0 else 9
        J = instances.erdos_renyi(n, 0.5, seed=70 + k, jmax=jmax, allow_zero=True)
        if jmax == 9:
            J[0, 1] = J[1, 0] = 9.0  # at least one coupling E2M1 cannot hold
        h = np.random.default_rng(k).integers(-3, 4, n).astype(np.float32) if k == 3 else None
        insts.append((J, h))
    probs = [sb.Problem.from_dense(J, h) for J, h in insts]
    steps, seed, R = 25, 300, 64
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_TC)
    batch = ctx.batch(probs, prm, want_state=True)
    res = batch.run()
    assert [r.field_dtype for r in res] == ["fp4e2m1", "fp6e2m3"] * 3
    for k, ((J, h), p, r) in enumerate(zip(insts, probs, res)):
        x, y = orc.init_uniform(J.shape[0], R, seed + k)
        orc.sb_run_f32(2, J, h, x, y, steps, 1.0, p.default_c0(), 1.25)
        np.testing.assert_array_equal(r.final_x, x, err_msg=f"instance {k}")
        np.testing.assert_array_equal(r.final_y, y, err_msg=f"instance {k}")
        np.testing.assert_array_equal(r.replica_energies, orc.energies_of_x(J, h, x))
        assert r.energy_check_ok
    batch.close()
