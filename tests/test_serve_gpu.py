"""Serving loop (sb_submit / sb_poll / sb_cancel): continuous batching, same result alone and in
the mix, cancellation, stats."""
import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances

pytestmark = pytest.mark.gpu


def test_requests_match_solo_solves():
    """Requests of uneven size (one of them, N = 13500, has packed E2M3 couplings of 138 MB, more
    than the L2 cache holds) and a bSB request outside the grouped engine, submitted together: each
    result equals the same request solved alone (there on the single-instance FP8 path)."""
    ctx = sb.Context(0)
    rng = np.random.default_rng(0)
    reqs = []
    for k, (n, steps) in enumerate([(100, 200), (700, 60), (1300, 150), (257, 120), (2000, 90), (64, 30),
                                    (13500, 60)]):
        p = sb.Problem.random(n, float(rng.uniform(0.05, 1.0)), 8, 2 if k == 3 else 0, seed=300 + k)
        prm = sb.Params.default(sb.DSB, steps=steps, replicas=32, seed=900 + k, field_mode=sb.FIELD_TC)
        reqs.append((p, prm))
    Jg, hg = instances.gaussian(150, seed=3)
    reqs.append((sb.Problem.from_dense(Jg, hg),
                 sb.Params.default(sb.BSB, steps=40, replicas=16, seed=5, field_mode=sb.FIELD_FP32)))
    tickets = [ctx.submit(p, prm) for p, prm in reqs]
    served = [ctx.poll(t, p.n, prm, wait_ms=-1) for t, (p, prm) in zip(tickets, reqs)]
    stats = ctx.serving_stats()
    assert stats["finished"] == len(reqs) and stats["peak_inflight"] >= 2
    solo = sb.Context(0)
    for (p, prm), r in zip(reqs, served):
        alone = solo.solve(p, prm)
        np.testing.assert_array_equal(r.best_spins, alone.best_spins)
        np.testing.assert_array_equal(r.replica_energies, alone.replica_energies)
        assert r.best_energy == alone.best_energy and r.energy_check_ok
        assert r.total_ms >= r.device_ms > 0
    solo.close()
    ctx.close()


def test_cancel_and_unknown_ticket():
    ctx = sb.Context(0)
    p = sb.Problem.random(3000, 1.0, 1, seed=1)
    prm = sb.Params.default(sb.DSB, steps=4000, replicas=32, field_mode=sb.FIELD_TC)
    t = ctx.submit(p, prm)
    ctx.cancel(t)
    with pytest.raises(sb.SBError) as e:
        ctx.poll(t, p.n, prm, wait_ms=-1)
    assert e.value.status == 10  # cancelled
    with pytest.raises(sb.SBError) as e:
        ctx.poll(12345, p.n, prm, wait_ms=0)
    assert e.value.status == 9  # not found
    ctx.close()
