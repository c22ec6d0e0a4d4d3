"""Plain FP32 kernels (one launch per step, and the one-launch dSB form) against the CPU oracle,
through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_dsb(ctx, J, h, R, steps, seed, **kw):
    prob = sb.Problem.from_dense(J, h)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=seed, field_mode=sb.FIELD_FP32, **kw)
    res = ctx.solve(prob, prm, want_state=True)
    n = J.shape[0]
    x, y = orc.init_uniform(n, R, seed)
    tr = orc.sb_run_f32(2, J, h, x, y, steps, 1.0, prob.default_c0(), 1.25,
                        trace=bool(kw.get("trace")), trace_all=bool(kw.get("trace_all")))
    return prob, res, x, y, tr


@pytest.mark.parametrize("n,R,steps,h", [(200, 3, 60, False), (37, 9, 25, True), (2000, 1, 100, False),
                                         (1, 1, 5, False), (130, 16, 0, True)])
def test_dsb_fp32_bit_exact(ctx, n, R, steps, h):
    J = instances.erdos_renyi(n, 0.5, seed=n, jmax=4, allow_zero=True) if n > 1 else np.zeros((1, 1), np.float32)
    hv = np.random.default_rng(n).integers(-3, 4, n).astype(np.float32) if h else None
    prob, res, x, y, _ = run_dsb(ctx, J, hv, R, steps, seed=17)
    assert res.field_mode == sb.FIELD_FP32
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.final_y, y)
    e = orc.energies_of_x(J, hv, x)
    np.testing.assert_array_equal(res.replica_energies, e)
    assert res.energy_check_ok and res.best_energy_i64 == res.best_energy == e.min()
    s = np.where(x[res.best_replica] > 0, 1, -1).astype(np.int8)
    np.testing.assert_array_equal(res.best_spins, s)


@pytest.mark.parametrize("n,R,steps,persist", [(2048, 1, 50, True), (1000, 2, 40, True), (257, 5, 30, True),
                                               (2049, 1, 10, False), (2000, 2, 10, False)])
def test_dsb_one_launch_equals_per_step(ctx, n, R, steps, persist, monkeypatch):
    """Plain FP32 dSB whose rows fit one co-resident grid (pitch <= 2048, ceil(n / 16) R CTAs) runs
    the whole solve in one cooperative launch, exchanging signs through tagged words; it is bit
    for bit the oracle's and the per-step kernel's (SB_PLAIN_PERSIST=0). Larger shapes keep one
    launch per step."""
    J = instances.erdos_renyi(n, 0.5, seed=n + 1, jmax=2, allow_zero=True)
    hv = np.random.default_rng(n).integers(-2, 3, n).astype(np.float32)
    prob, res, x, y, _ = run_dsb(ctx, J, hv, R, steps, seed=29)
    np.testing.assert_array_equal(res.final_x, x)
    np.testing.assert_array_equal(res.final_y, y)
    assert res.steps_per_launch == (steps if persist else 1)
    assert res.kernel_launches == (3 if persist else steps + 2)
    monkeypatch.setenv("SB_PLAIN_PERSIST", "0")
    ctx2 = sb.Context(0)
    try:
        prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=29, field_mode=sb.FIELD_FP32)
        r2 = ctx2.solve(prob, prm, want_state=True)
    finally:
        ctx2.close()
    assert r2.steps_per_launch == 1
    np.testing.assert_array_equal(r2.final_x, res.final_x)
    np.testing.assert_array_equal(r2.final_y, res.final_y)
    np.testing.assert_array_equal(r2.replica_energies, res.replica_energies)


@pytest.mark.parametrize("variant,n,R,steps", [(sb.BSB, 2000, 1, 60), (sb.BSB, 300, 3, 40), (sb.ASB, 2048, 1, 30),
                                               (sb.ASB, 130, 2, 25)])
def test_bsb_asb_one_launch_equals_per_step(variant, n, R, steps, monkeypatch):
    """bSB and aSB (the reference's update, its FP64 sub-steps for a CTA's 16 rows in one warp) in
    one cooperative launch, their default, exchange x itself (16 tagged words on a CTA's line): bit
    for bit the one-launch-per-step kernel's trajectories and energies (SB_PLAIN_PERSIST=0)."""
    J = instances.complete_pm1(n, seed=n) if variant == sb.ASB else instances.gaussian(n, seed=n)[0]
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(variant, steps=steps, replicas=R, seed=11, field_mode=sb.FIELD_FP32)
    monkeypatch.delenv("SB_PLAIN_PERSIST", raising=False)
    ctx1 = sb.Context(0)
    try:
        res = ctx1.solve(prob, prm, want_state=True)
    finally:
        ctx1.close()
    assert res.steps_per_launch == steps
    monkeypatch.setenv("SB_PLAIN_PERSIST", "0")
    ctx2 = sb.Context(0)
    try:
        r2 = ctx2.solve(prob, prm, want_state=True)
    finally:
        ctx2.close()
    assert r2.steps_per_launch == 1
    np.testing.assert_array_equal(r2.final_x, res.final_x)
    np.testing.assert_array_equal(r2.final_y, res.final_y)
    # real couplings: the FP64 energy pass adds its per-CTA partial sums with atomics (order not
    # fixed, last bits may differ between runs); integer couplings: exact
    np.testing.assert_allclose(r2.replica_energies, res.replica_energies, rtol=1e-12, atol=0)
    assert res.energy_check_ok


def test_dsb_trace_matches_oracle(ctx):
    J = instances.complete_pm1(300, seed=3)
    prob, res, x, y, (tr, tra) = run_dsb(ctx, J, None, 5, 40, seed=2, trace=1, trace_all=1)
    np.testing.assert_array_equal(res.energy_trace_all, tra)
    np.testing.assert_array_equal(res.energy_trace, tr)


def test_bsb_fp32_tracks_fp64_oracle(ctx):
    """bSB with real couplings, FP32 field: for the first K = 20 steps the trajectory stays within
    1e-3 (max abs) of the FP64 oracle, and within 4x the CPU FP32 oracle's own distance to FP64
    (the FP32 field's inherent error; the dynamics amplify rounding roughly 3x every 10 steps)."""
    Jg, hg = instances.gaussian(512, seed=4)
    prob = sb.Problem.from_dense(Jg, hg)
    R, K = 4, 20
    prm = sb.Params.default(sb.BSB, steps=K, replicas=R, seed=8, field_mode=sb.FIELD_FP32)
    res = ctx.solve(prob, prm, want_state=True)
    x0, y0 = orc.init_uniform(512, R, 8)
    c0 = prob.default_c0()
    xd, yd = orc.sb_run_f64(1, Jg, hg, x0, y0, K, 1.0, float(c0), 1.25)
    xf, yf = x0.copy(), y0.copy()
    orc.sb_run_f32(1, Jg, hg, xf, yf, K, 1.0, c0, 1.25)
    err_gpu = np.max(np.abs(res.final_x - xd))
    err_cpu32 = np.max(np.abs(xf - xd))
    assert err_gpu <= 1e-3
    assert err_gpu <= 4 * err_cpu32 + 1e-6
    assert res.energy_check_ok  # FP64 device energy of the returned spins == host FP64


def test_asb_reference_init_and_trajectory(ctx):
    n, R = 256, 3
    J = instances.complete_pm1(n, seed=5)
    prob = sb.Problem.from_dense(J)
    p0 = sb.Params.default(sb.ASB, steps=0, replicas=R, field_mode=sb.FIELD_FP32)
    r0 = ctx.solve(prob, p0, want_state=True)
    xr, yr = orc.init_reference(n, R)
    np.testing.assert_array_equal(r0.final_x, xr)
    np.testing.assert_array_equal(r0.final_y, yr)
    steps = 20
    p = sb.Params.default(sb.ASB, steps=steps, replicas=R, field_mode=sb.FIELD_FP32)
    r = ctx.solve(prob, p, want_state=True)
    x, y = xr.copy(), yr.copy()
    orc.asb_run(J, x, y, steps)
    assert np.max(np.abs(r.final_x - x)) < 1e-4
    assert r.energy_check_ok


def test_plan_reuse_and_seeds(ctx):
    J = instances.complete_pm1(128, seed=6)
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=50, replicas=8, field_mode=sb.FIELD_FP32)
    plan = ctx.plan(prob, prm, want_state=True)
    a = plan.run(seed=1)
    b = plan.run(seed=1)
    c = plan.run(seed=2)
    np.testing.assert_array_equal(a.final_x, b.final_x)
    assert not np.array_equal(a.final_x, c.final_x)
    plan.close()


def test_profile_mode_reports_kernel_time(ctx):
    J = instances.complete_pm1(512, seed=7)
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=20, replicas=2, field_mode=sb.FIELD_FP32, profile=1)
    r = ctx.solve(prob, prm)  # the one-launch form: one timed launch of 20 steps
    assert r.kernel_ms_avg > 0 and r.steps_per_launch == 20 and r.kernel_launches == 3
    prm = sb.Params.default(sb.ASB, steps=20, replicas=2, field_mode=sb.FIELD_FP32, profile=1, trace=1)
    r = ctx.solve(prob, prm)  # with a trace: one launch per step, each timed
    assert r.kernel_ms_avg > 0 and r.steps_per_launch == 1 and r.kernel_launches >= 22


def test_cli_drop_in(tmp_path):
    J = instances.complete_pm1(64, seed=8)
    g = str(tmp_path / "k64.txt")
    instances.write_graph(g, J)
    out = subprocess.run([os.path.join(ROOT, "annealing_gb300", "sb"), g, "--trials", "3", "--steps", "20"],
                         cwd=tmp_path, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    lines = open(tmp_path / "output.txt").read().split()
    assert len(lines) == 3
    spins = np.array(open(tmp_path / "best_spins.txt").read().split(), dtype=np.int8)
    assert spins.shape == (64,) and int(min(map(int, lines))) == orc.energy_i64(J, None, spins)


@pytest.mark.parametrize("N", [256, 2048])
def test_asb_matches_reference_golden(ctx, N):
    """aSB on the plain kernel against the reference's own kernels + cuBLAS (tests/golden):
    identical initial state, positions within 2e-4 over 20 steps, identical final spins."""
    d = np.load(os.path.join(ROOT, "tests", "golden", f"ref_m2opt_n{N}.npz"))
    n, T = int(d["n_spins"]), d["x0"].shape[0]
    J = np.zeros((N, N), np.float32)
    J[:n, :n] = instances.complete_pm1(n, seed=int(d["seed"]))
    prob = sb.Problem.from_dense(J)
    steps = d["xs"].shape[1]  # the golden schedule: amplitude s / 20
    p = sb.Params.default(sb.ASB, steps=steps, replicas=T, field_mode=sb.FIELD_FP32, trace_all=1)
    r = ctx.solve(prob, p, want_state=True)
    ref = d["xs"][:, steps - 1]
    assert np.max(np.abs(r.final_x - ref)) <= 2e-4
    np.testing.assert_array_equal(r.final_x > 0, ref > 0)
    # trace slot s + 1 is the energy after reference step s
    for s in (0, 9, 19):
        e_ref = [orc.energy_f64(J, None, np.where(d["xs"][t, s] > 0, 1, -1).astype(np.int8)) for t in range(T)]
        np.testing.assert_array_equal(r.energy_trace_all[s + 1], e_ref)
