"""The `gpuropolis` CLI as a drop-in for the reference's main() (main.cu:1011-1257):
the same arguments give the same samples.txt header byte for byte and, for
the chains whose trajectories agree, the same sample lines byte for byte.
The reference side is the reference's own main() compiled for the host
(oracle/build_ref.py), with the project's transcendental functions in its
proposal random transforms so that proposals can agree bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
oref = pytest.importorskip("oracle.ref")


def _write_data(path, x, y, sd):
    with open(path, "w") as f:
        f.write("# x\ty\tsd\n")
        for a, b, c in zip(x, y, sd):
            f.write("%.9g\t%.9g\t%.9g\n" % (a, b, c))


def _lines(path):
    head, body = [], []
    for line in open(path, encoding="latin-1").read().split("\n"):
        (head if line.startswith("#") else body).append(line)
    return head, [l for l in body if l]


@pytest.mark.parametrize("extra", [[], ["--show-constants", "--thin=1"]])
def test_cli_matches_reference(tmp_path, extra):
    if not oref.available():
        pytest.skip("reference oracle source not available")
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x, y, sd = H.quad_data(60, seed=3)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    o = oref.get(pl=31, project_math=1)
    ref_out, our_out = tmp_path / "ref", tmp_path / "ours"
    ref_out.mkdir(); our_out.mkdir()
    args = ["--in=%s" % data, "--N=256", "--steps=20", "--outer=3", "--seed=12345", "--quiet"] + extra
    r = subprocess.run([o.cli_path] + args + ["--out=%s" % ref_out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([g.CLI_PATH] + args + ["--out=%s" % our_out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rh, rb = _lines(ref_out / "samples.txt")
    oh, ob = _lines(our_out / "samples.txt")
    # the header differs only in the output path line
    assert [l for l in rh if "Output path" not in l] == [l for l in oh if "Output path" not in l]
    assert len(rb) == len(ob) == 256 * 2

    def same_line(a, b):
        """Chain, block, length, degree, the three printed programs, the op
        codes and constants exactly; posterior, prior and likelihood (printed
        %.3f, i.e. up to 11 significant digits for large scores) within 1e-5."""
        fa, fb = a.split("\t"), b.split("\t")
        if len(fa) != len(fb) or fa[:2] != fb[:2] or fa[5:] != fb[5:]:
            return False
        for u, v in zip(fa[2:5], fb[2:5]):
            u, v = float(u), float(v)
            if not (u == v or abs(u - v) <= 1e-5 * max(abs(u), abs(v), 1.0)):
                return False
        return True

    same = np.mean([same_line(a, b) for a, b in zip(rb, ob)])
    assert same >= 0.9, same
    # every line has the reference's layout
    for line in ob:
        f = line.split("\t")
        assert len(f) == (11 + 31 + 1 if extra else 12)   # each line ends with a tab
        assert f[7].startswith('"') and f[7].endswith('"') and f[10].startswith('"')
    assert os.path.exists(our_out / "log.txt")


def test_cli_rejects_bad_arguments(tmp_path):
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    r = subprocess.run([g.CLI_PATH, "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Invalid command line arguments" in r.stderr
    r = subprocess.run([g.CLI_PATH, "--in=%s" % (tmp_path / "missing.txt"), "--out=%s" % tmp_path, "--quiet"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    r = subprocess.run([g.CLI_PATH, "--steps=0"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1


def _run_cli(tmp_path, name, args):
    out = tmp_path / name
    out.mkdir()
    r = subprocess.run([g.CLI_PATH] + args + ["--out=%s" % out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("k", [50, 700, 5000])
def test_cli_tops_matches_sort_tail(tmp_path, k):
    """--tops=K writes what `sort -g -k3 samples.txt | tail -n K` (run-all.sh:45)
    prints in the C locale, with candidates from the device top-k."""
    import shutil
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    if not shutil.which("sort"):
        pytest.skip("coreutils sort not available")
    x, y, sd = H.quad_data(60, seed=3)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    out = _run_cli(tmp_path, "run", ["--in=%s" % data, "--N=512", "--steps=30", "--outer=4", "--seed=7",
                                     "--quiet", "--tops=%d" % k])
    want = subprocess.run("sort -g -k3 %s | tail -n %d" % (out / "samples.txt", k), shell=True,
                          capture_output=True, env={"LC_ALL": "C", "PATH": os.environ.get("PATH", "")},
                          check=True).stdout
    assert (out / "tops.txt").read_bytes() == want


def test_cli_device_resample(tmp_path):
    """--device-resample: with a cutoff that re-draws nothing (quantile 0) the
    run is the host path's byte for byte; with map-delta it re-draws chains on
    the device and completes."""
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x, y, sd = H.quad_data(60, seed=3)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    base = ["--in=%s" % data, "--N=512", "--steps=20", "--outer=4", "--seed=11", "--quiet"]
    a = _run_cli(tmp_path, "host", base + ["--resample=quantile:0"])
    b = _run_cli(tmp_path, "dev", base + ["--resample=quantile:0", "--device-resample"])
    ha, la = _lines(a / "samples.txt")
    hb, lb = _lines(b / "samples.txt")
    assert len(la) == 512 * 3 and la == lb
    assert "(device)" in (b / "log.txt").read_text()
    c = _run_cli(tmp_path, "dev_md", base + ["--resample=map-delta:20", "--device-resample"])
    _, lc = _lines(c / "samples.txt")
    assert len(lc) == 512 * 3 and lc[:512] != la[:512]


def test_cli_gradient_moves_constants_only(tmp_path):
    """--const-proposal=hmc:EPS:L with --struct-every=0: each chain keeps its
    program from block to block (no structure moves, no re-draws at quantile
    0) while its constants move; log.txt records the mode."""
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x, y, sd = H.quad_data(60, seed=3)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    out = _run_cli(tmp_path, "hmc", ["--in=%s" % data, "--N=256", "--steps=10", "--outer=3", "--seed=5", "--quiet",
                                     "--const-proposal=hmc:0.001:4", "--struct-every=0", "--resample=quantile:0",
                                     "--show-constants", "--ops=basic"])
    _, lines = _lines(out / "samples.txt")
    by_chain = {}
    for l in lines:
        f = l.split("\t")
        by_chain.setdefault(f[0], []).append(f)
    assert len(by_chain) == 256
    moved = 0
    for rows in by_chain.values():
        assert len({r[10] for r in rows}) == 1          # the op-code string
        moved += len({tuple(r[11:]) for r in rows}) > 1
    assert moved > 0
    log = (out / "log.txt").read_text()
    assert "hmc:0.001:4" in log and "Structure move every: 0" in log
    r = subprocess.run([g.CLI_PATH, "--const-proposal=hmc:x"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1


def test_cli_three_variables(tmp_path):
    """--vars=3: data lines "x1 x2 x3 y sd" (the header echoes all five
    columns), the op set holding the leaves x1, x2, x3 (printed X, Y, Z in
    the op-code string and x1, x2, x3 in expressions); programs that read x2
    and x3 appear and score finite posteriors."""
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x1, x2, x3, y, sd = H.multivar_data(150, seed=6)
    data = tmp_path / "data3.txt"
    with open(data, "w") as f:
        f.write("# x1\tx2\tx3\ty\tsd\n")
        for row in zip(x1, x2, x3, y, sd):
            f.write("\t".join("%.9g" % v for v in row) + "\n")
    out = _run_cli(tmp_path, "v3", ["--in=%s" % data, "--vars=3", "--N=512", "--steps=50", "--outer=3",
                                    "--seed=11", "--quiet", "--ops=1,3,4,5,6,9,11,20,22,27,28,29,14",
                                    "--resample=map-delta:20"])
    head, lines = _lines(out / "samples.txt")
    data_rows = [h for h in head if h.startswith("# \t") and h.count("\t") == 5]
    assert len(data_rows) == 150
    assert len(lines) > 0
    fields = [l.split("\t") for l in lines]
    codes = [f[10] for f in fields]
    assert any("Y" in c or "Z" in c for c in codes)
    exprs = [f[7] for f in fields]
    assert any("x2" in e or "x3" in e for e in exprs)
    post = np.array([float(f[2]) for f in fields])
    assert np.isfinite(post).any()
    r = subprocess.run([g.CLI_PATH, "--vars=2"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0


def test_cli_adapt(tmp_path):
    """--adapt=T: per-chain scales adapt during the blocks that are not
    written (0..burn) and are kept afterwards; log.txt records it; the run
    writes the blocks after burn-in; --adapt needs a proposal with a scale."""
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x, y, sd = H.quad_data(80, seed=8)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    out = _run_cli(tmp_path, "adapt", ["--in=%s" % data, "--N=256", "--steps=100", "--outer=4", "--burn=1",
                                       "--seed=4", "--quiet", "--ops=basic", "--const-proposal=rw:0.5",
                                       "--adapt=0.3"])
    log = (out / "log.txt").read_text()
    assert "Adapt: per-chain scales toward acceptance 0.3 in blocks 0..1" in log
    _, lines = _lines(out / "samples.txt")
    blocks = sorted({int(l.split("\t")[1]) for l in lines})
    assert blocks == [2, 3] and len(lines) == 2 * 256
    for bad in (["--adapt=0"], ["--adapt=1.5"], ["--adapt=0.5"]):   # the last: reference proposals
        r = subprocess.run([g.CLI_PATH, "--in=%s" % data, "--N=64", "--steps=5", "--outer=1", "--quiet",
                            "--out=%s" % (tmp_path / "x")] + bad, capture_output=True, text=True, timeout=60)
        assert r.returncode != 0, bad


@pytest.mark.parametrize("extra", [[], ["--device-resample"]], ids=["host-resample", "device-resample"])
def test_cli_checkpoint_resume(tmp_path, extra):
    """A run stopped after block 2 with --checkpoint and continued with
    --resume writes, after the first run's lines, exactly the lines the
    uninterrupted run writes for blocks 3 and 4 (chains, seed and the host
    stream's position all come back)."""
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    x, y, sd = H.quad_data(70, seed=9)
    data = tmp_path / "data.txt"
    _write_data(data, x, y, sd)
    base = ["--in=%s" % data, "--N=256", "--steps=20", "--seed=13", "--quiet", "--ops=basic",
            "--const-proposal=rw:0.1", "--resample=quantile:0.5"] + extra
    whole = _run_cli(tmp_path, "whole", base + ["--outer=5"])
    ck = tmp_path / "state.ckpt"
    part = _run_cli(tmp_path, "part", base + ["--outer=3", "--checkpoint=%s" % ck])
    r = subprocess.run([g.CLI_PATH] + base + ["--outer=5", "--resume=%s" % ck, "--out=%s" % part],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    hw, lw = _lines(whole / "samples.txt")
    hp, lp = _lines(part / "samples.txt")
    assert lp == lw and len(lw) == 4 * 256      # blocks 1..4 are written (block 0 is not: o > burn)
    assert "Resumed from" in (part / "log.txt").read_text()
    # a checkpoint for other chains is refused
    r = subprocess.run([g.CLI_PATH] + base + ["--N=128", "--outer=5", "--resume=%s" % ck,
                                              "--out=%s" % (tmp_path / "bad")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode != 0 and "checkpoint" in r.stderr
