"""The bounds-checked build (-DSB_CHECKS), the debug stand-in for a memory sanitizer: every kernel
path (plain FP32 step in both layouts, aSB; E2M1 / FP8 / BF16 / BF16 hi+lo tensor cores; the
grouped batch; SQA; NMFA in both fields) runs small parity cases against the CPU oracle with every
device bounds check on, in a subprocess that loads annealing_gb300/_checked/libsbsolve.so through
SB_LIBRARY. A failing check would come back as an error naming it; none may fire, and the results
must equal the oracle's as in the unchecked runs."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

assert sb.sb.LIB_PATH.endswith("_checked/libsbsolve.so"), sb.sb.LIB_PATH
ctx = sb.Context(0)

def dsb(J, R, steps, field, operand=sb.OPERAND_AUTO):
    prob = sb.Problem.from_dense(J)
    prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=5, field_mode=field, operand_dtype=operand)
    res = ctx.solve(prob, prm, want_state=True)
    x, y = orc.init_uniform(J.shape[0], R, 5)
    orc.sb_run_f32(2, J, None, x, y, steps, 1.0, prob.default_c0(), 1.25)
    assert np.array_equal(res.final_x, x) and np.array_equal(res.final_y, y), (J.shape, R, field, operand)
    assert res.energy_check_ok
    return res

# plain FP32 step: ring layout (1, 2 replicas per CTA), staged layout (3+), ragged rows, several chunks
for n, R in ((130, 1), (37, 2), (600, 3), (1030, 9)):
    dsb(instances.erdos_renyi(n, 0.5, seed=n, jmax=3, allow_zero=True), R, 12, sb.FIELD_FP32)
# aSB, the reference update
J = instances.complete_pm1(200, seed=2)
res = ctx.solve(sb.Problem.from_dense(J), sb.Params.default(sb.ASB, steps=10, replicas=2, field_mode=sb.FIELD_FP32))
assert res.energy_check_ok
# tensor cores: E2M1, FP8, BF16 operands, edge shapes
J = instances.complete_pm1(257, seed=4)
for op in (sb.OPERAND_FP4, sb.OPERAND_FP8, sb.OPERAND_BF16):
    for R in (33, 130):
        dsb(J, R, 6, sb.FIELD_TC, op)
# bSB on BF16 hi+lo (real couplings): runs and stays close to the FP32 oracle
Jg, _ = instances.gaussian(256, seed=3)
prob = sb.Problem.from_dense(Jg)
res = ctx.solve(prob, sb.Params.default(sb.BSB, steps=4, replicas=64, seed=9, field_mode=sb.FIELD_TC), want_state=True)
x, y = orc.init_uniform(256, 64, 9)
orc.sb_run_f32(1, Jg, None, x, y, 4, 1.0, prob.default_c0(), 1.25)
assert np.abs(res.final_x - x).max() < 1e-3
# grouped batch of uneven sizes
probs = [sb.Problem.from_dense(instances.erdos_renyi(n, 0.4, seed=n, jmax=1)) for n in (64, 129, 300)]
b = ctx.batch(probs, sb.Params.default(sb.DSB, steps=8, replicas=32, seed=1))
for r in b.run(seed=1):
    assert r.energy_check_ok
b.close()
# the same with couplings up to 9: packed E2M3 operands
probs = [sb.Problem.from_dense(instances.erdos_renyi(n, 0.4, seed=n, jmax=9, allow_zero=True)) for n in (64, 129, 300)]
b = ctx.batch(probs, sb.Params.default(sb.DSB, steps=8, replicas=64, seed=1))
for r in b.run(seed=1):
    assert r.energy_check_ok and r.field_dtype == "fp6e2m3"
b.close()
# SQA (hash mode)
J = instances.erdos_renyi(96, 0.5, seed=6, jmax=3)
s, _ = orc.sqa_init(96, 8, 2, 1, 3)
tr = orc.sqa_run(J, s, 3, 1, seed=3)
r = ctx.sqa_solve(sb.Problem.from_dense(J), sb.SqaParams.default(trotter=8, steps=3, replicas=2, rng_mode=sb.SQA_RNG_HASH, seed=3, trace=1), want_spins=True)
assert np.array_equal(r.final_spins, s) and r.energy_check_ok
# NMFA: FP32 field (bit-exact) and tensor cores
J = instances.nmfa_fully(300, seed=8)
betas = sb.nmfa_schedule(100)[:6]
for R, field in ((3, sb.FIELD_FP32), (40, sb.FIELD_TC)):
    res = ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=R, seed=2, field_mode=field),
                         betas=betas, want_states=True)
    st, sp, _ = orc.nmfa_run(J, R, betas, 0.15, 0.15, 2)
    if field == sb.FIELD_FP32:
        assert np.array_equal(res.states.view(np.uint32), st.view(np.uint32))
    else:
        assert np.abs(res.states - st).max() < 1e-4
    assert res.energy_check_ok
ctx.close()
print("checked build: every path ran with its bounds checks, no check fired")
"""


def test_checked_build_runs_every_path():
    from annealing_gb300 import _build

    lib = _build.build_library(checks=True)
    env = dict(os.environ, SB_LIBRARY=lib)
    out = subprocess.run([sys.executable, "-c", SCRIPT, ROOT], env=env, capture_output=True, text=True,
                         timeout=1200, cwd=ROOT)
    print(out.stdout[-2000:])
    assert out.returncode == 0, out.stdout[-3000:] + out.stderr[-3000:]
    assert "no check fired" in out.stdout
