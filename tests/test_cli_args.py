"""The CLI refuses bad arguments before it touches a GPU: unknown or
malformed flags (main.cu:111-156 semantics plus this build's additive
flags), and values the reference would assert on (main.cu:1026-1031) or
that have no meaning (a quantile outside [0, 1), a target acceptance outside
(0, 1), adaptation with the reference's scale-free proposals, adaptation
together with checkpoints).  These run on CPU."""
import os
import subprocess

import pytest

g = pytest.importorskip("gpuropolis_gb300")


def _cli(args):
    if not os.path.exists(g.CLI_PATH):
        pytest.skip("CLI not built")
    return subprocess.run([g.CLI_PATH] + args, capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("args,message", [
    (["--vars=2"], "Invalid command line arguments"),
    (["--adapt=0"], "Invalid command line arguments"),
    (["--adapt=1.5"], "Invalid command line arguments"),
    (["--resample=median"], "Invalid command line arguments"),
    (["--rng=mt19937"], "Invalid command line arguments"),
    (["--const-proposal=hmc:x"], "Invalid command line arguments"),
    (["--tops=0"], "Invalid command line arguments"),
    (["--struct-every=-1"], "Invalid command line arguments"),
    (["--steps=0"], "steps must be > 0"),
    (["--N=0"], "N must be > 0"),
    (["--thin=0"], "thin must be >= 1"),
    (["--resample=quantile:1.0"], "--resample"),
    (["--resample=map-delta:-1"], "--resample"),
    (["--adapt=0.3"], "--adapt needs"),
    (["--adapt=0.3", "--const-proposal=rw:0.1", "--checkpoint=/tmp/x"], "do not keep the adaptation"),
    (["--hmc-jitter=0.2"], "Invalid command line arguments"),
    (["--hmc-jitter=1.5:0"], "Invalid command line arguments"),
    (["--hmc-jitter=0.2:0.5"], "--hmc-jitter needs"),
])
def test_cli_rejects(args, message):
    r = _cli(args)
    assert r.returncode != 0
    assert message in r.stderr, r.stderr
