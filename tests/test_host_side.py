"""CPU tests of the host half of the drop-in (libgpuropolis.so, no GPU call)
against the reference's own code compiled for the host (oracle/ref.py):
expression formatting (main.cu:821-976), description length and polynomial
degree folds (main.cu:477-526, 615-654), the data loader (main.cu:319-363),
and the host-RNG initialisation (main.cu:1133-1137)."""
import glob
import os

import numpy as np
import pytest

from tests import helpers as H

g = pytest.importorskip("gpuropolis_gb300")
oref = pytest.importorskip("oracle.ref")

from oracle import build_ref  # noqa: E402

NIST = os.path.join(build_ref.REF_DIR, "data-sources", "NIST")


def _need_ref():
    if not oref.available():
        pytest.skip("reference oracle source not available")


def _lib():
    try:
        g.library()
    except ImportError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("PL", [31, 63])
def test_format_expression_matches_reference(PL):
    _need_ref(); _lib()
    P, C = H.random_programs(400, PL, seed=3, shallow_frac=0.8)
    o = oref.get(pl=PL, project_math=1)
    n_checked = 0
    for i in range(P.shape[1]):
        for fmt, latex in (("C", False), ("%.10f", False), ("%.2f", True)):
            ours = g.format_expression(P, C, i, fmt, latex)
            ref = o.display(fmt, P, C, i, latex)
            if len(ref) < 99 and len(ours) < 99:
                # the reference is only defined while its 100-byte buffers hold
                assert ours == ref, (i, fmt, ours, ref)
                n_checked += 1
    assert n_checked > 300


@pytest.mark.parametrize("PL", [31, 63])
def test_length_and_degree_match_reference(PL):
    _need_ref(); _lib()
    P, C = H.random_programs(2000, PL, seed=4)
    o = oref.get(pl=PL, project_math=1)
    for i in range(P.shape[1]):
        assert g.program_length_of(P, C, i) == o.length(P, C, i)
        a, b = g.polynomial_degree(P, C, i), o.degree(P, C, i)
        assert (a == b) or (np.isnan(a) and np.isnan(b)), (i, a, b)


def test_format_samples_line_layout():
    _lib()
    P, C = H.random_programs(8, 31, seed=5, shallow_frac=1.0)
    prior = np.linspace(-10, -1, 8)
    lik = np.linspace(-100, -50, 8)
    s = g.format_samples(P, C, prior, lik, block=3, show_constants=True)
    lines = s.splitlines()
    assert len(lines) == 8
    for h, line in enumerate(lines):
        f = line.split("\t")
        # h, block, posterior, prior, likelihood, length, degree, 3 quoted strings, code, 31 constants, ''
        assert f[0] == str(h) and f[1] == "3"
        assert f[2] == "%.3f" % (prior[h] + lik[h])
        assert f[7].startswith('"') and f[10].startswith('"') and len(f[10]) == 31 + 2
        assert len(f) == 11 + 31 + 1 and f[-1] == ""


@pytest.mark.skipif(not os.path.isdir(NIST), reason="reference data not mounted")
@pytest.mark.parametrize("trim", [(False, False), (True, False), (False, True), (True, True)])
def test_data_loader_matches_reference(trim):
    _need_ref(); _lib()
    o = oref.get(pl=31, project_math=1)
    files = sorted(glob.glob(os.path.join(NIST, "*", "data.txt")))
    assert files
    for f in files:
        ours = g.load_data_file(f, 1.5, *trim)
        ref = o.load_data(f, 1.5, *trim)
        for a, b in zip(ours, ref):
            np.testing.assert_array_equal(a, b)


def test_data_loader_errors(tmp_path):
    _lib()
    p = tmp_path / "bad.txt"
    p.write_text("# comment\n1 2 0.5\nnot numbers\n")
    with pytest.raises(g.GprError):
        g.load_data_file(str(p))
    p.write_text("1 2 0\n")
    with pytest.raises(g.GprError):
        g.load_data_file(str(p))
    with pytest.raises(g.GprError):
        g.load_data_file(str(tmp_path / "missing.txt"))
    p.write_text("# c\n\n1\t2\t0.5\n  \n3.0e0 4.5 2e-1\n")
    x, y, sd = g.load_data_file(str(p))
    np.testing.assert_array_equal(x, [1, 3])
    np.testing.assert_array_equal(sd, np.float32([0.5, 0.2]))


@pytest.mark.parametrize("trim", [(False, False), (True, False), (False, True), (True, True)])
def test_three_variable_loader(tmp_path, trim):
    """Lines "x1 x2 x3 y sd" under the reference's parse rules (comment and
    blank lines skipped, sd scaled and > 0, first-half / even-half trims in
    the reference's order), checked against the same rules written out in
    Python, and against the single-variable loader on its x1, y, sd columns."""
    _lib()
    r = np.random.default_rng(4)
    n = 37
    cols = r.normal(size=(5, n))
    cols[4] = np.abs(cols[4]) + 0.1
    lines = ["# header", ""]
    for i in range(n):
        lines.append("\t".join("%.6g" % v for v in cols[:, i]))
        if i % 9 == 0:
            lines.append("   ")
    p = tmp_path / "d3.txt"
    p.write_text("\n".join(lines) + "\n")
    got = g.load_data_file3(str(p), 2.0, *trim)
    want = np.array([[float("%.6g" % v) for v in c] for c in cols])
    want[4] *= 2.0
    idx = np.arange(n)
    if trim[0]:
        idx = idx[: n // 2]
    if trim[1]:
        idx = idx[1::2]
    for k in range(5):
        np.testing.assert_array_equal(got[k], want[k][idx].astype(np.float32))
    p1 = tmp_path / "d1.txt"
    p1.write_text("\n".join(["\t".join("%.6g" % cols[k, i] for k in (0, 3, 4)) for i in range(n)]) + "\n")
    one = g.load_data_file(str(p1), 2.0, *trim)
    for a, b in zip(one, (got[0], got[3], got[4])):
        np.testing.assert_array_equal(a, b)


def test_three_variable_loader_errors(tmp_path):
    _lib()
    p = tmp_path / "bad3.txt"
    p.write_text("1 2 3 4 0.5\n1 2 3\n")           # a three-column line is not five columns
    with pytest.raises(g.GprError):
        g.load_data_file3(str(p))
    p.write_text("1 2 3 4 0\n")
    with pytest.raises(g.GprError, match="sd must be > 0"):
        g.load_data_file3(str(p))


@pytest.mark.parametrize("opset", [0, 1])
def test_host_init_matches_reference(opset):
    _need_ref(); _lib()
    o = oref.get(pl=31, opset=opset, project_math=1)
    P0, C0 = o.host_init(64, 12345)
    P1, C1 = g.host_init_chains(64, 31, 12345, ops=o.ops)
    np.testing.assert_array_equal(P0, P1)
    np.testing.assert_array_equal(C0.view(np.int32), C1.view(np.int32))


def _declared_functions(path):
    """Names of the functions a public header declares (comments stripped)."""
    import re
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return sorted(set(re.findall(r"\b(gpr_\w+)\s*\(", text)) - {"gpr_config"})


@pytest.mark.parametrize("header", ["gpuropolis.h", "gpuropolis_host.h"])
def test_library_exports_every_declared_function(header):
    """libgpuropolis.so loads without a GPU and exports every function its
    headers declare (no compute call is made)."""
    _lib()
    import ctypes
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", header)
    names = _declared_functions(path)
    assert len(names) >= 8, names
    lib = ctypes.CDLL(g.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _samples_text(N, PL, blocks, seed):
    """A samples.txt as the CLI writes it: the parameter and data header, then
    the lines of `blocks` blocks (ties, -inf and nan posteriors included)."""
    r = np.random.default_rng(seed)
    head = ["# -----------------------------------------------------------------",
            "# -- Parameters:", "# \tInput data path: data.txt", "# \tOutput path: out/",
            "# \tMCMC Iterations (per block): 1000", "# \tBlocks: %d" % blocks, "# \tN chains: %d" % N,
            "# \tSeed: 5", "# \tMax program length: %d" % PL, "# \tGPU: 0", "#", "#", "# -- Data:"]
    head += ["# \t%f\t%f\t%f" % (a, b, c) for a, b, c in r.normal(0, 30, (20, 3))]
    text = "\n".join(head + ["#", "#"]) + "\n"
    out = [text]
    for b in range(1, blocks + 1):
        P, C = H.random_programs(N, PL, seed=seed + b)
        lik = -np.abs(r.normal(0, 50, N)).round(2)
        lik[r.integers(0, N, N // 20)] = -np.inf
        lik[r.integers(0, N, 3)] = np.nan
        lik[r.integers(0, N, N // 8)] = -7.25
        prior = np.where(r.random(N) < 0.1, -0.0, -np.abs(r.normal(0, 5, N)).round(3))
        out.append(g.format_samples(P, C, prior, lik, b))
    return "".join(out)


@pytest.mark.parametrize("k", [1, 7, 100, 250, 5000])
def test_tops_matches_sort_tail(tmp_path, k):
    """gpr_tops keeps exactly what `LC_ALL=C sort -g -k3 samples.txt | tail -n k`
    (run-all.sh:45) prints, header lines with numeric third fields included."""
    import shutil
    import subprocess
    _lib()
    if not shutil.which("sort") or not shutil.which("tail"):
        pytest.skip("coreutils sort/tail not available")
    text = _samples_text(300, 15, 3, seed=k)
    path = tmp_path / "samples.txt"
    path.write_bytes(text.encode("latin-1"))
    want = subprocess.run("sort -g -k3 %s | tail -n %d" % (path, k), shell=True, capture_output=True,
                          env={"LC_ALL": "C", "PATH": os.environ.get("PATH", "")}, check=True).stdout
    t = g.Tops(k)
    t.add_text(text)
    t.write(str(tmp_path / "tops_all.txt"))
    assert (tmp_path / "tops_all.txt").read_bytes() == want
    # the same, offering the header whole and each block's lines by index,
    # in several pieces
    head_end = text.index("\n#\n#\n") + 5
    t2 = g.Tops(k)
    t2.add_text(text[:head_end])
    body = text[head_end:]
    nlines = body.count("\n")
    t2.add_lines(body, np.arange(0, nlines, 2))
    t2.add_lines(body, np.arange(1, nlines, 2))
    t2.write(str(tmp_path / "tops_lines.txt"))
    assert (tmp_path / "tops_lines.txt").read_bytes() == want


def test_ess_geyer_on_ar1():
    """ESS of AR(1) series with coefficient a is close to T (1 - a) / (1 + a);
    an independent series gives about T; a constant series gives 0."""
    from gpuropolis_gb300.diagnostics import ess_geyer
    r = np.random.default_rng(0)
    T, n = 4000, 400
    for a in (0.0, 0.5, 0.9):
        e = r.normal(size=(n, T))
        x = np.empty_like(e)
        x[:, 0] = e[:, 0] / np.sqrt(1 - a * a)
        for t in range(1, T):
            x[:, t] = a * x[:, t - 1] + e[:, t]
        ess = ess_geyer(x)
        want = T * (1 - a) / (1 + a)
        assert abs(np.median(ess) / want - 1) < 0.1, (a, np.median(ess), want)
    assert ess_geyer(np.ones((2, 100)))[0] == 0


def test_population_ess_on_short_ar1_runs():
    """Populations of stationary AR(1) chains (tau = (1 + a) / (1 - a)) whose
    runs are 1.5 to 20 autocorrelation times long: the population estimator
    stays within 12% of T / tau, where the per-chain estimator overestimates
    the short runs by more than 2x."""
    from gpuropolis_gb300.diagnostics import ess_geyer, ess_population
    r = np.random.default_rng(1)
    for a, T, m in ((0.9, 800, 200), (0.99, 3000, 400), (0.995, 1000, 800), (0.999, 3000, 1000)):
        e = r.normal(size=(m, T))
        x = np.empty_like(e)
        x[:, 0] = e[:, 0] / np.sqrt(1 - a * a)
        for t in range(1, T):
            x[:, t] = a * x[:, t - 1] + e[:, t]
        want = T * (1 - a) / (1 + a)
        got = ess_population(x)
        assert abs(got / want - 1) < 0.12, (a, T, got, want)
        if T < 3 * (1 + a) / (1 - a):
            assert np.median(ess_geyer(x)) > 2 * want
    assert ess_population(np.ones((3, 50))) == 0.0


def test_variable_leaves_need_three_variables():
    """x2/x3 leaf ops are refused for a univariate handle, before any device
    work; the op-code string prints the variable leaves as X, Y, Z."""
    _lib()
    with pytest.raises(g.GprError, match="n_vars = 3"):
        g.Sampler(4, program_length=7, ops=[g.CONST, g.X2])
    with pytest.raises(g.GprError, match="n_vars"):
        g.Sampler(4, program_length=7, n_vars=2)
    P = np.zeros((7, 1), np.int32)
    P[0, 0], P[1, 0], P[2, 0] = g.PLUS, g.X2, g.X3
    C = np.zeros((7, 1), np.float32)
    assert g.format_expression(P, C, 0) == "(x2+x3)"
    line = g.format_samples(P, C, np.zeros(1), np.zeros(1), 1)
    assert '"+YZ1111"' in line


def test_host_resample_rejects_bad_arguments():
    """The host resampling returns -1 instead of reading past the sorted
    posteriors (a quantile of 1 or more) or dividing by zero (one op)."""
    _lib()
    N, PL = 64, 31
    P, C = H.random_programs(N, PL, seed=1)
    prior, lik = H.mixed_scores(N, seed=2)
    for mode, param, ops in ((0, 1.0, None), (0, -0.1, None), (1, -1.0, None), (2, 0.5, None), (0, 0.5, [1])):
        assert g.host_resample(P.copy(), C.copy(), prior, lik, ops=ops, mode=mode, param=param) == -1
        assert "gpr_host_resample" in g.library().gpr_host_last_error().decode()
    assert g.host_resample(P.copy(), C.copy(), prior, lik, mode=0, param=0.5) >= 0
