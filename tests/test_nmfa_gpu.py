"""NMFA on the GPU (sb_nmfa_solve, sb_gpu_nmfa) against the oracle and the reference's own kernel.

Bit-exact against oracle/nmfa_oracle.c (same sweep semantics, the library's own transcendental
functions on both sides, the kernel's summation order restated), over both field layouts (up to two
samples per CTA: the bulk-copy ring with overlapped launches; more: the staged layout), ragged and
multi-chunk rows. Against the reference's own kernel (tests/golden/ref_nmfa_*.npz, made by
tests/golden/make_nmfa_golden.py on a GB300): the states after K stages at N = 32 (one warp, where the
reference's sweeps are race-free) within a stated tolerance, and the energy distributions at N = 128
and N = 1024 by a two-sample Kolmogorov-Smirnov test.
"""
import os
import subprocess

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from oracle import binding as orc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ctx():
    c = sb.Context(0)
    yield c
    c.close()


def _energies(J, samples):
    s = samples.astype(np.int64)
    return np.einsum("ri,ij,rj->r", s, np.rint(J).astype(np.int64), s) // 2


@pytest.mark.parametrize("n,R,stages,kind", [
    (1, 1, 3, "fully"),        # a single spin (an empty row: norm 0, noise only)
    (5, 3, 4, "fully"),        # ragged row (padding to 8), three samples: staged layout
    (32, 1, 20, "fully"),      # one warp of spins, one sample: ring layout
    (33, 2, 10, "pm1"),        # two samples per CTA: ring layout
    (100, 8, 6, "fully"),      # eight samples per CTA
    (130, 13, 5, "pm1"),       # a partial last sample block (13 = 8 + 5)
    (600, 9, 3, "fully"),      # two chunks of K, staged layout
    (2050, 2, 2, "pm1"),       # five chunks of K through a four-stage ring (refills)
])
@pytest.mark.parametrize("one_launch", [True, False], ids=["one-launch", "per-sweep"])
def test_bit_exact_vs_oracle(ctx, monkeypatch, n, R, stages, kind, one_launch):
    """Both FP32 forms: every sweep in one cooperative launch (shapes whose rows fit one co-resident
    grid: ceil(n / 16) x samples CTAs, padded rows <= 2048) and one launch per sweep."""
    if not one_launch:
        monkeypatch.setenv("SB_PLAIN_PERSIST", "0")
    fits = ((n + 15) // 16) * R <= 152 and (n + 3) // 4 * 4 <= 2048
    J = instances.nmfa_fully(n, seed=n + 7) if kind == "fully" else instances.complete_pm1(n, seed=n + 7)
    betas = sb.nmfa_schedule(100)[:stages]
    p = sb.NmfaParams.default(samples=R, seed=99 + n, field_mode=sb.FIELD_FP32)
    res = ctx.nmfa_solve(sb.Problem.from_dense(J), p, betas=betas, want_states=True)
    st, sp, _ = orc.nmfa_run(J, R, betas, 0.15, 0.15, 99 + n)
    assert np.array_equal(res.states.view(np.uint32), st.view(np.uint32)), \
        f"max |diff| {np.abs(res.states - st).max()}"
    assert np.array_equal(res.samples.astype(np.int32), sp)
    e = _energies(J, sp)
    assert np.array_equal(res.energies, e.astype(np.float64))
    assert res.best_energy == e.min() and res.energy_check_ok
    sweeps = 1 if (one_launch and fits) else 2 * stages
    assert res.kernel_launches == 1 + sweeps + 1 and res.field_mode_used == sb.FIELD_FP32


def test_real_couplings_bit_exact(ctx):
    """Real-valued J (FP32 fields, FP64 energy pass): states and samples bit-exact."""
    J, _ = instances.gaussian(70, seed=5)
    betas = sb.nmfa_schedule(100)[:8]
    res = ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=4, seed=3, field_mode=sb.FIELD_FP32),
                         betas=betas, want_states=True)
    st, sp, _ = orc.nmfa_run(J, 4, betas, 0.15, 0.15, 3)
    assert np.array_equal(res.states.view(np.uint32), st.view(np.uint32))
    assert np.array_equal(res.samples.astype(np.int32), sp)
    s = sp.astype(np.float64)
    e = np.einsum("ri,ij,rj->r", s, J.astype(np.float64), s) / 2
    assert np.allclose(res.energies, e, rtol=0, atol=1e-9 * (1 + np.abs(e).max()))
    assert res.energy_check_ok


def test_parameters(ctx):
    """Noise, recombination and seed reach the kernel as the oracle uses them."""
    J = instances.nmfa_fully(64, seed=11)
    betas = sb.nmfa_schedule(30)
    for noise, rc, seed in ((0.0, 0.15, 1), (0.5, 0.3, 2), (0.15, 1.0, 4294967295)):
        p = sb.NmfaParams.default(samples=3, noise=noise, recombination=rc, seed=seed, field_mode=sb.FIELD_FP32)
        res = ctx.nmfa_solve(sb.Problem.from_dense(J), p, betas=betas, want_states=True)
        st, _, _ = orc.nmfa_run(J, 3, betas, noise, rc, seed)
        assert np.array_equal(res.states.view(np.uint32), st.view(np.uint32)), (noise, rc, seed)


def test_gpu_nmfa_entry_point(ctx):
    """sb_gpu_nmfa, the reference's gpu_nmfa signature: int32 +-1 samples and the device time."""
    J = instances.nmfa_fully(150, seed=3)  # NMFA/CUDA_GPU/Makefile's default N
    betas = sb.nmfa_schedule(100)
    out, ms = ctx.gpu_nmfa(J, betas, 5, 0.15, 0.15, 1234)
    _, sp, _ = orc.nmfa_run(J, 5, betas, 0.15, 0.15, 1234)
    assert out.dtype == np.int32 and np.array_equal(out, sp)
    assert ms > 0


def test_rejects(ctx):
    J = instances.nmfa_fully(16, seed=1)
    h = np.ones(16, np.float32)
    with pytest.raises(sb.SBError):
        ctx.nmfa_solve(sb.Problem.from_dense(J, h), sb.NmfaParams.default())
    with pytest.raises(sb.SBError):
        ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=0))
    with pytest.raises(sb.SBError):
        ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(recombination=1.5))


@pytest.mark.parametrize("field", ["fp32", "tc"])
def test_reference_states_one_warp(ctx, field):
    """N = 32: the reference kernel's states after the first K stages of the 100-stage anneal (256
    samples, its own seeds). Its noise and tanh are CUDA fast-math intrinsics, ours are the library's
    FP32 functions, and its field is summed in another order, so states agree to a tolerance: within
    2e-3 for every spin after one and two stages and for 99 % of the spins throughout; the final
    samples (after 100 stages) agree in 99 % of the spins. The same bounds hold for the tensor-core
    field (states as BF16 hi + lo)."""
    g = np.load(os.path.join(GOLDEN, "ref_nmfa_n32.npz"))
    J = g["J"].astype(np.float32)
    full = sb.nmfa_schedule(100)
    mode = sb.FIELD_FP32 if field == "fp32" else sb.FIELD_TC
    for K in g["ks"]:
        ref = g[f"states_k{K}"]
        res = ctx.nmfa_solve(sb.Problem.from_dense(J),
                             sb.NmfaParams.default(samples=int(g["samples"]), field_mode=mode),
                             betas=full[:K], want_states=True)
        d = np.abs(res.states - ref)
        print(f"K={K}: max |ds| {d.max():.3e}, 99th pct {np.quantile(d, 0.99):.3e}, "
              f"sign agreement {np.mean(np.sign(res.states) == np.sign(ref)):.4f}")
        if K <= 2:
            assert d.max() <= 2e-3
        assert np.quantile(d, 0.99) <= 2e-3
        if K == 100:
            assert np.mean((res.states > 0) == (ref > 0)) >= 0.99


@pytest.mark.parametrize("n,field", [(128, "fp32"), (1024, "fp32"), (128, "tc"), (1024, "tc")])
def test_reference_energy_distribution(ctx, n, field):
    """1000 samples of ours against 1000 of the reference kernel on the same seeded instance: the
    energy distributions pass a two-sample KS test (p >= 0.01) and the means agree within 3
    standard errors. Beyond one warp the reference's sweeps race, so only the distribution is
    comparable."""
    from scipy import stats

    g = np.load(os.path.join(GOLDEN, f"ref_nmfa_n{n}.npz"))
    J = instances.nmfa_fully(n, int(g["seed"]))
    mode = sb.FIELD_FP32 if field == "fp32" else sb.FIELD_TC
    res = ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=1000, seed=20240, field_mode=mode))
    ours, ref = res.energies, g["energies"].astype(np.float64)
    ks = stats.ks_2samp(ours, ref)
    se = np.sqrt(ours.var() / len(ours) + ref.var() / len(ref))
    print(f"n={n} {field}: ours mean {ours.mean():.2f} sd {ours.std():.2f}, reference mean {ref.mean():.2f} "
          f"sd {ref.std():.2f}, KS p {ks.pvalue:.3f}")
    assert ks.pvalue >= 0.01
    assert abs(ours.mean() - ref.mean()) <= 3 * se


@pytest.mark.parametrize("n,R,stages", [
    (32, 32, 20),      # one replica tile of 32 samples
    (130, 40, 10),     # ragged spin tile, two replica tiles
    (300, 200, 10),    # several spin and replica tiles
    (1024, 256, 20),   # the bench's N
])
def test_tensor_core_vs_oracle(ctx, n, R, stages):
    """The tcgen05 field (states as BF16 hi + lo, about 16 bits, FP32 accumulation) against the
    oracle's FP32 field: states after `stages` stages within 2e-3 at the 99th percentile, and the
    samples' signs equal for 99 % of the spins."""
    J = instances.nmfa_fully(n, seed=n + 3)
    betas = sb.nmfa_schedule(100)[:stages]
    res = ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=R, seed=5, field_mode=sb.FIELD_TC),
                         betas=betas, want_states=True)
    st, sp, _ = orc.nmfa_run(J, R, betas, 0.15, 0.15, 5)
    d = np.abs(res.states - st)
    agree = np.mean(res.samples.astype(np.int32) == sp)
    print(f"tc n={n} R={R} K={stages}: max |ds| {d.max():.3e}, 99th pct {np.quantile(d, 0.99):.3e}, "
          f"median {np.median(d):.3e}, sign agreement {agree:.4f}")
    assert np.quantile(d, 0.99) <= 2e-3
    assert agree >= 0.99
    assert res.energy_check_ok and res.field_mode_used == sb.FIELD_TC and res.kernel_launches == 6
    assert np.array_equal(res.energies, _energies(J, res.samples).astype(np.float64))


def test_tensor_core_needs_integer_couplings(ctx):
    J, _ = instances.gaussian(64, seed=1)
    with pytest.raises(sb.SBError):
        ctx.nmfa_solve(sb.Problem.from_dense(J), sb.NmfaParams.default(samples=64, field_mode=sb.FIELD_TC))


def test_cli_nmfa(tmp_path):
    """`sb --variant nmfa <graph>`: the reference program NMFA/CUDA_GPU/Ising.cpp (reads the graph,
    anneals one sample with its schedule, prints the elapsed ms)."""
    J = instances.nmfa_fully(64, seed=2)
    path = tmp_path / "g.txt"
    instances.write_graph(str(path), J)
    exe = os.path.join(ROOT, "annealing_gb300", "sb")
    out = subprocess.run([exe, "--variant", "nmfa", "--json", str(path)], capture_output=True, text=True,
                         cwd=tmp_path, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    float(lines[0])  # the elapsed time, Ising.cpp:48
    import json
    d = json.loads(lines[-1])
    betas = sb.nmfa_schedule(100)
    _, sp, _ = orc.nmfa_run(J, 1, betas, 0.15, 0.15, 1234)
    assert d["best_energy"] == float(_energies(J, sp)[0])
    spins = np.loadtxt(tmp_path / "best_spins.txt", dtype=np.int64)
    assert np.array_equal(spins, sp[0])
