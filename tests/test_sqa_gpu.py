"""SQA on the GPU (sb_sqa_solve) against the oracle and the reference's own kernels."""
import os

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = sb.Context(0)
    yield c
    c.close()


def _oracle(J, M, R, steps, rng, seed):
    s, rnd = orc.sqa_init(J.shape[0], M, R, rng, seed)
    tr = orc.sqa_run(J, s, steps, rng, rnd=rnd, seed=seed)
    return s, tr


@pytest.mark.parametrize("n,M,R,steps,kind", [
    (64, 4, 3, 5, "pm1"),        # one row word per plane
    (100, 7, 2, 4, "er3"),       # ragged last word, |J| <= 3 (two magnitude planes)
    (300, 33, 2, 2, "er5"),      # more slices than warps (two per warp), three planes
    (2, 2, 2, 6, "pm1"),         # smallest instance
    (40, 40, 1, 3, "pm1"),       # as many slices as spins
    (129, 1, 3, 5, "er3"),       # one slice (its own Trotter neighbour)
    (520, 128, 1, 1, "pm1"),     # the most slices: four per warp
    (96, 12, 2, 3, "er9"),       # |J| <= 9: four magnitude planes
    (80, 6, 2, 3, "er127"),      # |J| <= 127, the reference's char range: seven planes
])
def test_hash_mode_bit_exact(ctx, n, M, R, steps, kind):
    J = instances.complete_pm1(n, seed=n) if kind == "pm1" else \
        instances.erdos_renyi(n, 0.6, n, jmax=int(kind[2:]), allow_zero=True)
    prm = sb.SqaParams.default(trotter=M, steps=steps, replicas=R, rng_mode=sb.SQA_RNG_HASH, seed=77, trace=1)
    res = ctx.sqa_solve(sb.Problem.from_dense(J), prm, want_spins=True)
    s, tr = _oracle(J, M, R, steps, 1, 77)
    np.testing.assert_array_equal(res.final_spins, s)
    np.testing.assert_array_equal(res.energy_trace, tr.astype(np.float64))
    np.testing.assert_array_equal(res.replica_energies, tr[:, -1].astype(np.float64))
    assert res.energy_check_ok and res.best_energy == tr[:, -1].min()
    assert np.array_equal(res.best_spins, s[res.best_replica, 0])


@pytest.mark.parametrize("N,M", [(256, 8), (512, 16)])
def test_reference_mode_matches_the_reference_kernels(ctx, N, M):
    d = np.load(os.path.join(GOLDEN, f"ref_sqa_n{N}_m{M}.npz"))
    trials, steps = d["energy"].shape
    prm = sb.SqaParams.default(trotter=M, steps=steps, replicas=trials, rng_mode=sb.SQA_RNG_REFERENCE, trace=1)
    res = ctx.sqa_solve(sb.Problem.from_dense(d["J"].astype(np.float32)), prm, want_spins=True)
    np.testing.assert_array_equal(res.final_spins, d["spins"][:, -1].transpose(0, 2, 1))
    np.testing.assert_array_equal(res.energy_trace, d["energy"].astype(np.float64))


def test_larger_instance_matches_oracle(ctx):
    n, M, R, steps = 2000, 16, 2, 3
    J = instances.complete_pm1(n, seed=5)
    prm = sb.SqaParams.default(trotter=M, steps=steps, replicas=R, seed=3)
    res = ctx.sqa_solve(sb.Problem.from_dense(J), prm, want_spins=True)
    s, tr = _oracle(J, M, R, steps, 1, 3)
    np.testing.assert_array_equal(res.final_spins, s)
    np.testing.assert_array_equal(res.replica_energies, tr[:, -1].astype(np.float64))
    assert res.spin_updates_per_s > 0 and res.kernel_launches == 3


def test_rejects_what_it_cannot_run(ctx):
    J = instances.complete_pm1(16, seed=1)
    p = sb.Problem.from_dense(J)
    for kw in ({"trotter": 17}, {"trotter": 0}, {"steps": 0}, {"replicas": 0}, {"rng_mode": 5}):
        with pytest.raises(sb.SBError) as e:
            ctx.sqa_solve(p, sb.SqaParams.default(**kw))
        assert e.value.status == 1
    Jr = J.copy()
    Jr[0, 1] = Jr[1, 0] = 0.5
    with pytest.raises(sb.SBError) as e:
        ctx.sqa_solve(sb.Problem.from_dense(Jr), sb.SqaParams.default(trotter=4))
    assert e.value.status == 6
    with pytest.raises(sb.SBError) as e:
        ctx.sqa_solve(sb.Problem.from_dense(J, np.ones(16, np.float32)), sb.SqaParams.default(trotter=4))
    assert e.value.status == 6


def test_cli_drop_in_reproduces_the_reference_program(tmp_path):
    """`sb <graph> --variant sqa --init reference` on the pinned instance writes the final slice-0
    energy of each trial to output.txt, as pre_calculate.cu:242-246 does, equal to the run of the
    reference's own kernels."""
    import subprocess

    d = np.load(os.path.join(GOLDEN, "ref_sqa_n256_m8.npz"))
    trials, steps = d["energy"].shape
    g = str(tmp_path / "k256.txt")
    instances.write_graph(g, d["J"].astype(np.float32))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [os.path.join(root, "annealing_gb300", "sb"), g, "--variant", "sqa", "--trotter", "8", "--trials",
           str(trials), "--steps", str(steps), "--init", "reference"]
    out = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    got = np.array(open(tmp_path / "output.txt").read().split(), dtype=np.int64)
    np.testing.assert_array_equal(got, d["energy"][:, -1])
