"""C-ABI library: loads, exports what include/sb.h declares, host-side entry points (CPU only)."""
import os
import re
import ctypes as C
import subprocess

import numpy as np
import pytest

import annealing_gb300 as sb
from annealing_gb300 import instances
from annealing_gb300.sb import lib
from oracle import binding as orc
from oracle.reader import read_reference_format

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sb_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 20
    L = lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_and_status_strings():
    assert lib().sb_abi_version() == 3
    assert lib().sb_status_string(0) == b"ok"
    assert lib().sb_status_string(3) == b"parse error"


def test_defaults_follow_reference_constants():
    p = sb.Params.default(sb.ASB)
    # m2_opt.cu:15-22
    assert (p.mts_m, p.mts_dt, p.coupling_dt, p.detune, p.kerr) == (2, 0.5, 1.0, 1.0, 1.0)
    assert abs(p.xi - 0.01565) < 1e-9 and p.steps == 100 and p.replicas == 1
    assert p.init_mode == sb.INIT_REFERENCE
    q = sb.Params.default(sb.DSB)
    assert (q.dt, q.a0, q.c0, q.init_mode) == (1.25, 1.0, 0.0, sb.INIT_UNIFORM)


def test_pump_and_c0_match_oracle():
    for steps in (1, 7, 1000, 3000):
        for t in range(0, steps, max(1, steps // 13)):
            assert sb.pump(1.0, t, steps) == orc.pump(1.0, t, steps)
    for J in (instances.complete_pm1(100, 1), instances.gaussian(90, 2)[0],
              instances.erdos_renyi(70, 0.1, 3, jmax=8, allow_zero=True)):
        p = sb.Problem.from_dense(J)
        assert p.default_c0() == orc.default_c0(J)


def test_energy_evaluators_match_oracle():
    rng = np.random.default_rng(1)
    J = instances.erdos_renyi(120, 0.4, 11, jmax=8, allow_zero=True)
    h = rng.integers(-5, 6, 120).astype(np.float32)
    s = (rng.integers(0, 2, 120) * 2 - 1).astype(np.int8)
    p = sb.Problem.from_dense(J, h)
    assert p.integer_valued
    assert p.energy(s) == orc.energy_i64(J, h, s)
    Jg, hg = instances.gaussian(80, 5)
    pg = sb.Problem.from_dense(Jg, hg)
    assert not pg.integer_valued
    assert pg.energy(s[:80]) == orc.energy_f64(Jg, hg, s[:80])


def test_exact_energy_paths():
    """sb_energy_i64: the scanned int32-row path (threaded from n = 1024 on), the per-element
    checked int64 path of a problem whose struct carries no scan, and its refusal of a real J."""
    rng = np.random.default_rng(4)
    for n, jmax in ((1500, 1), (1100, 16)):
        J = instances.erdos_renyi(n, 0.7, n, jmax=jmax, allow_zero=True)
        h = rng.integers(-3, 4, n).astype(np.float32)
        s = (rng.integers(0, 2, n) * 2 - 1).astype(np.int8)
        p = sb.Problem.from_dense(J, h)
        ref = orc.energy_i64(J, h, s)
        assert p.energy(s) == ref
        p.s.integer_valued = 0  # as if the caller filled the struct by hand
        out = C.c_int64()
        assert lib().sb_energy_i64(C.byref(p.s), s.ctypes.data_as(C.POINTER(C.c_int8)), C.byref(out)) == 0
        assert out.value == ref
    J = instances.complete_pm1(1200, seed=2)
    J[3, 700] = J[700, 3] = 0.5
    p = sb.Problem.from_dense(J)
    s = np.ones(1200, np.int8)
    out = C.c_int64()
    assert lib().sb_energy_i64(C.byref(p.s), s.ctypes.data_as(C.POINTER(C.c_int8)), C.byref(out)) == 6


@pytest.mark.parametrize("n,jmax,density,with_h", [
    (1, 1, 1.0, False),
    (63, 1, 1.0, True),      # one bit-plane word per row, a partial one
    (64, 1, 0.5, False),     # exactly one word
    (200, 1, 0.3, True),     # bit planes, zero couplings, a field
    (1030, 1, 1.0, False),   # many words, ragged tail
    (300, 7, 0.6, True),     # int8 copy
    (700, 127, 1.0, False),  # int8 copy at its largest magnitude
    (150, 300, 0.5, False),  # |J| > 127: no copy, the FP32 evaluator
])
def test_batched_exact_energies(n, jmax, density, with_h):
    """sb_energies_i64 (bit planes for J in {-1, 0, 1}, int8 for |J| <= 127, else the FP32
    evaluator) gives the oracle's int64 energy for every vector, including all-up and all-down."""
    rng = np.random.default_rng(n + jmax)
    J = instances.erdos_renyi(n, density, n + 1, jmax=jmax, allow_zero=True) if n > 1 else np.zeros((1, 1), np.float32)
    h = rng.integers(-9, 10, n).astype(np.float32) if with_h else None
    p = sb.Problem.from_dense(J, h)
    S = (rng.integers(0, 2, (6, n)) * 2 - 1).astype(np.int8)
    S[0] = 1
    S[1] = -1
    got = p.energies(S)
    assert [int(v) for v in got] == [orc.energy_i64(J, h, s) for s in S]
    assert int(p.energies(S[2])[0]) == orc.energy_i64(J, h, S[2])


def test_batched_exact_energies_refuses_real_couplings():
    Jg, hg = instances.gaussian(40, 5)
    p = sb.Problem.from_dense(Jg, hg)
    S = np.ones((3, 40), np.int8)
    out = np.zeros(3, np.int64)
    rc = lib().sb_energies_i64(C.byref(p.s), S.ctypes.data_as(C.POINTER(C.c_int8)), 3,
                               out.ctypes.data_as(C.POINTER(C.c_int64)))
    assert rc == 6  # SB_ERR_UNSUPPORTED


def test_graph_reader_reference_format(tmp_path):
    J = instances.erdos_renyi(60, 0.3, 2, jmax=3)
    path = str(tmp_path / "g.txt")
    instances.write_graph(path, J)
    p = sb.Problem.load(path)
    hdr, Jr = read_reference_format(path)
    assert hdr == 60 and p.n == 60
    assert np.array_equal(p.J, Jr) and np.array_equal(p.J, J)
    assert p.h is None and p.integer_valued
    assert p.s.n_edges == int(np.count_nonzero(np.triu(J, 1)))
    off = J.astype(np.float64) - np.diag(np.diag(J))
    assert p.s.stats_valid == 1
    assert p.s.sum_j == int(off.sum()) and p.s.sum_j2 == int((off * off).sum())


@pytest.mark.parametrize("n,jmax,with_h", [(2, 1, False), (300, 1, False), (1100, 7, True), (513, 300, True)])
def test_default_c0_from_scan_sums(n, jmax, with_h):
    """The default c0 from the scan's exact coupling sums equals the one computed by a pass over J
    (the same float, bit for bit); real couplings carry no sums."""
    J = instances.erdos_renyi(n, 0.6, n, jmax=jmax, allow_zero=True)
    h = np.random.default_rng(n).integers(-4, 5, n).astype(np.float32) if with_h else None
    p = sb.Problem.from_dense(J, h)
    assert p.s.stats_valid == 1
    fast = p.default_c0()
    p.s.stats_valid = 0
    slow = p.default_c0()
    assert np.float32(fast).tobytes() == np.float32(slow).tobytes()
    Jg, _ = instances.gaussian(50, 2)
    assert sb.Problem.from_dense(Jg).s.stats_valid == 0


def test_graph_reader_fields_realweights_onebased(tmp_path):
    Jg, hg = instances.gaussian(40, 3)
    path = str(tmp_path / "g.txt")
    instances.write_graph(path, Jg, hg, header_edges=True)
    p = sb.Problem.load(path)
    assert np.allclose(p.J, Jg, rtol=1e-7, atol=0) and np.allclose(p.h, hg, rtol=1e-7, atol=0)
    assert not p.integer_valued
    one = str(tmp_path / "one.txt")
    with open(one, "w") as f:
        f.write("# rudy style, 1-based\n3 2\n1 2 1\n2 3 -1\n")
    q = sb.Problem.load(one)
    assert q.n == 3 and q.J[0, 1] == 1 and q.J[1, 2] == -1 and q.J[2, 1] == -1
    z = sb.Problem.load(one, index_base=0, n=4)  # explicit base and an N override
    assert z.n == 4 and z.J[1, 2] == 1 and z.J[2, 3] == -1


def test_graph_reader_errors(tmp_path):
    def write(txt):
        p = str(tmp_path / "bad.txt")
        open(p, "w").write(txt)
        return p

    with pytest.raises(sb.SBError) as e:
        sb.Problem.load(str(tmp_path / "missing.txt"))
    assert e.value.status == 2
    for txt in ("3\n0 1\n", "3\n0 1 x\n", "3\n0 5 1\n", "abc\n", "3\n0 1 1 2\n"):
        with pytest.raises(sb.SBError) as e:
            sb.Problem.load(write(txt))
        assert e.value.status == 3, txt
    # a later line for the same pair wins (m2_opt.cu:120-121), unless strict
    p = sb.Problem.load(write("3\n0 1 1\n0 1 -2\n"))
    assert p.J[0, 1] == -2 and p.J[1, 0] == -2
    with pytest.raises(sb.SBError):
        sb.Problem.load(write("3\n0 1 1\n0 1 -2\n"), strict=True)


def test_graph_reader_large_file_in_file_order(tmp_path):
    """Files of a few MB are parsed in chunks on several host threads and filled by row owners: the
    couplings, fields, duplicates (the later line wins), index base and the line of the first error
    (parse, range or strict conflict) are those of one pass in file order."""
    rng = np.random.default_rng(5)
    n, m = 700, 250_000
    i = rng.integers(1, n + 1, m)
    j = rng.integers(1, n + 1, m)
    w = rng.integers(-3, 4, m)
    i[-1], j[-1] = n, 1  # the largest index is N: 1-based
    lines = [f"# generated\n{n} {m}\n"]
    for k in range(m):
        sep = "," if k % 89 == 0 else " "
        lines.append(f"{i[k]}{sep}{j[k]}{sep}{w[k]}" + ("  # note" if k % 1000 == 3 else "") +
                     ("\r\n" if k % 2 else "\n"))
        if k % 7000 == 11:
            lines.append("\n# a comment line\n")
    path = str(tmp_path / "big.txt")
    open(path, "w", newline="").write("".join(lines))
    J = np.zeros((n, n), np.float32)
    h = np.zeros(n, np.float32)
    for a, b, v in zip(i - 1, j - 1, w):
        if a == b:
            h[a] = v
        else:
            J[a, b] = J[b, a] = v
    p = sb.Problem.load(path)
    np.testing.assert_array_equal(p.J, J)
    np.testing.assert_array_equal(np.ctypeslib.as_array(p.s.h, shape=(n,)), h)
    text = "".join(lines).split("\n")
    # (index N + 1 with the base given: with the base detected it would make the file 0-based)
    for bad, base in (("1 2", -1), ("1.5 2 3", -1), (f"1 {n + 1} 1", 1)):
        at = len(text) * 3 // 4
        while text[at].startswith("#") or not text[at].strip():
            at += 1
        t = list(text)
        t[at] = bad
        open(path, "w", newline="").write("\n".join(t))
        with pytest.raises(sb.SBError) as e:
            sb.Problem.load(path, index_base=base)
        assert e.value.status == 3 and f"line {at + 1}:" in str(e.value), (bad, str(e.value))
    # strict: the first conflicting line in file order, although the rows belong to other threads
    t = list(text)
    at = len(text) - 3
    t.insert(at, f"{i[0]} {j[0]} {int(J[i[0] - 1, j[0] - 1]) + 10}")
    open(path, "w", newline="").write("\n".join(t))
    with pytest.raises(sb.SBError) as e:
        sb.Problem.load(path, strict=True)
    assert "conflicting" in str(e.value)
    first = int(str(e.value).split("line ")[1].split(":")[0])
    assert first <= at + 1  # an earlier duplicate with another weight may conflict first


def test_footprint_is_positive_and_grows_with_replicas():
    J = instances.complete_pm1(256, 1)
    p = sb.Problem.from_dense(J)
    f1 = lib().sb_plan_footprint(p.s, sb.Params.default(sb.DSB, replicas=1, field_mode=1))
    f2 = lib().sb_plan_footprint(p.s, sb.Params.default(sb.DSB, replicas=64, field_mode=1))
    assert 0 < f1 < f2


def test_cli_prints_usage():
    out = subprocess.run([os.path.join(ROOT, "annealing_gb300", "sb")], capture_output=True, text=True)
    assert out.returncode == 0 and "Usage" in out.stdout


def test_create_without_gpu_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sb.SBError) as e:
        sb.Context(0)
    assert e.value.status == 11
