"""Build recipe for the C restatement oracle (TEST INFRASTRUCTURE ONLY):
oracle/gpr_oracle.c -> oracle/_build/libgpr_port.so (git-ignored)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libgpr_port.so")
SRC = os.path.join(HERE, "gpr_oracle.c")
DEPS = [SRC, os.path.join(HERE, "..", "gpuropolis_gb300", "csrc", "gpr_rngmath.h"),
        os.path.join(HERE, "..", "gpuropolis_gb300", "csrc", "gpr_philox.h")]


def build(force=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(map(os.path.getmtime, DEPS)):
        return OUT
    # -fwrapv/-ffp-contract=off: same integer wrap-around and float results as
    # the reference oracle build on x86 and Arm hosts.
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fwrapv", "-ffp-contract=off", "-fopenmp", "-fPIC",
                    "-shared", "-o", OUT + ".tmp", SRC, "-lm"], check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
