"""Time-to-target analysis (sb_time_to_target) against the restatement of the reference's scripts.

The traces are the reference's own published ones (plot_energy_decrease/{m1,m2,opt}_stats.csv,
packed by tests/golden/make_stats_traces.py), analysed at the two targets plot.r uses (-62059,
-60278). The first-passage summary and the success-probability time must equal the oracle's
(oracle/tts.py, a step-by-step restatement of plot.r:88-240 and test.sh:26-32).
"""
import math
import os

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300.sb import lib
from oracle import tts as orc_tts

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_stats_traces.npz")
TARGETS = (-62059.0, -60278.0)  # plot.r:68-69 ("HNN", "GW-SDP")


def _traces():
    z = np.load(GOLDEN)
    return {name: (z[f"{name}_energy"], z[f"{name}_time_s"]) for name in ("m1", "m2", "opt")}


@pytest.mark.parametrize("name", ["m1", "m2", "opt"])
@pytest.mark.parametrize("target", TARGETS)
def test_first_passage_matches_plot_r(name, target):
    e, t = _traces()[name]  # [trials, steps]
    rows = [list(zip(t[k].tolist(), e[k].tolist())) for k in range(e.shape[0])]
    count, best, avg, worst = orc_tts.first_passage(rows, target)
    got = sb.time_to_target(e.T.astype(np.float64), t.T, target, run_ms=1.0)
    assert got["trials"] == e.shape[0]
    assert got["reached"] == count
    assert got["best_ms"] == best and got["worst_ms"] == worst
    assert got["mean_ms"] == pytest.approx(avg, rel=1e-12)


def test_first_passage_known_values():
    # counted independently with awk over opt_stats.csv / m1_stats.csv
    e, t = _traces()["opt"]
    got = sb.time_to_target(e.T.astype(np.float64), t.T, -62059.0, run_ms=1.0)
    assert (got["reached"], got["best_ms"], got["worst_ms"]) == (64, 0.000149, 0.000427)
    assert got["mean_ms"] == pytest.approx(0.000222297, abs=5e-10)
    e1, t1 = _traces()["m1"]
    assert sb.time_to_target(e1.T.astype(np.float64), t1.T, -62059.0, 1.0)["succeeded"] == 71


@pytest.mark.parametrize("name", ["m1", "m2", "opt"])
def test_success_probability_time_matches_test_sh(name):
    e, t = _traces()[name]
    final = e[:, -1].tolist()
    cut = orc_tts.success_cut(final)
    assert sb.success_threshold(np.array(final)) == cut
    rate = orc_tts.success_rate(final, cut)
    run_ms = float(t[:, -1].mean() * 1e3)
    got = sb.time_to_target(e.T.astype(np.float64), t.T * 1e3, cut, run_ms=run_ms, p_target=0.99)
    assert got["success_rate"] == rate
    if 0.0 < rate < 0.99:
        assert got["tts_ms"] == pytest.approx(orc_tts.annealing_time(run_ms, rate), rel=1e-12)


def test_edges_and_shared_times():
    # rows x trials; trial 0 reaches -3 at row 1 and ends there, trial 1 never gets below -1
    e = np.array([[0.0, 0.0], [-3.0, -1.0], [-3.0, -1.0]])
    times = np.array([0.0, 2.0, 4.0])
    got = sb.time_to_target(e, times, -2.0, run_ms=4.0, p_target=0.9)
    assert (got["reached"], got["succeeded"], got["best_ms"], got["worst_ms"]) == (1, 1, 2.0, 2.0)
    assert got["success_rate"] == 0.5
    assert got["tts_ms"] == pytest.approx(4.0 * math.log(0.1) / math.log(0.5), rel=1e-12)
    none = sb.time_to_target(e, times, -10.0, run_ms=4.0)
    assert none["reached"] == 0 and math.isnan(none["best_ms"]) and math.isnan(none["mean_ms"])
    assert none["tts_ms"] == math.inf
    every = sb.time_to_target(e, times, 1.0, run_ms=4.0)
    assert every["reached"] == 2 and every["best_ms"] == 0.0 and every["tts_ms"] == 4.0
    # the success test looks at the final row only, first passage at any row
    back = np.array([[0.0], [-5.0], [0.0]])
    g2 = sb.time_to_target(back, times, -2.0, run_ms=1.0)
    assert (g2["reached"], g2["succeeded"], g2["tts_ms"]) == (1, 0, math.inf)


def test_invalid_arguments():
    e = np.zeros((3, 2))
    for kw in ({"p_target": 1.0}, {"p_target": 0.0}, {"run_ms": -1.0}):
        args = dict(threshold=0.0, run_ms=1.0, p_target=0.99)
        args.update(kw)
        with pytest.raises(sb.SBError):
            sb.time_to_target(e, np.zeros(3), **args)
    with pytest.raises(ValueError):
        sb.time_to_target(e, np.zeros(4), 0.0, 1.0)
    assert lib().sb_time_to_target(None, None, 3, 2, 0, 0.0, 1.0, 0.99, None) == 1


@pytest.mark.gpu
def test_solve_trace_time_to_target_matches_oracle():
    """A traced dSB solve on the GPU, analysed by the library and by the restated scripts."""
    from annealing_gb300 import instances

    n, R, steps = 200, 64, 120
    J = instances.complete_pm1(n, seed=3)
    ctx = sb.Context(0)
    try:
        prm = sb.Params.default(sb.DSB, steps=steps, replicas=R, seed=5, trace_all=1)
        res = ctx.solve(sb.Problem.from_dense(J), prm)
    finally:
        ctx.close()
    tr = res.energy_trace_all  # [steps + 1, R]
    assert np.array_equal(tr[-1], res.replica_energies)
    step_ms = res.device_ms / steps
    target = float(np.percentile(tr[-1], 30))
    got = sb.result_time_to_target(res, target)
    rows = [[(t * step_ms, tr[t, k]) for t in range(steps + 1)] for k in range(R)]
    count, best, avg, worst = orc_tts.first_passage(rows, target)
    assert got["reached"] == count and got["best_ms"] == best and got["worst_ms"] == worst
    assert got["mean_ms"] == pytest.approx(avg, rel=1e-12)
    rate = orc_tts.success_rate(tr[-1].tolist(), target)
    assert got["success_rate"] == rate
    if 0.0 < rate < 0.99:
        assert got["tts_ms"] == pytest.approx(orc_tts.annealing_time(res.device_ms, rate), rel=1e-12)


@pytest.mark.gpu
def test_cli_time_to_target(tmp_path):
    """`sb <graph> --target E` prints the summary of its replicas' traces."""
    import json
    import subprocess

    from annealing_gb300 import instances

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    J = instances.complete_pm1(128, seed=9)
    g = str(tmp_path / "k128.txt")
    instances.write_graph(g, J)
    cmd = [os.path.join(root, "annealing_gb300", "sb"), g, "--variant", "dsb", "--replicas", "32",
           "--steps", "100", "--target", "-900", "--json"]
    out = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("time_to_target ")]
    assert len(line) == 1
    tts = json.loads(line[0][len("time_to_target "):])
    finals = np.array(open(tmp_path / "output.txt").read().split(), dtype=np.int64)
    assert tts["trials"] == 32 and tts["succeeded"] == int(np.sum(finals < -900))
    assert tts["reached"] >= tts["succeeded"]
