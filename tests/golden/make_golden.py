"""Generate the golden vectors in tests/golden/ from the reference's own code
(main.cu compiled for the host by oracle/build_ref.py).  Run in a checkout
that has the reference mounted:  python tests/golden/make_golden.py [case ...]
(all cases when none is named)

Each case stores a seeded initial state, the dataset, the block seed and what
the reference's MH_simple_kernel (main.cu:679-813) produced after `steps`
steps, plus per-chain prior, likelihood, length, node count, f(x) at a few
points and the three printed forms of each program (main.cu:878-976)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref as oref  # noqa: E402
from tests import helpers as H  # noqa: E402

CASES = {
    "pl31_ref_lcg_indep": dict(PL=31, opset=0, philox=0, rw=0.0, data="quad", N=48, steps=30, seed=31337),
    "pl31_ref_philox_indep": dict(PL=31, opset=0, philox=1, rw=0.0, data="quad", N=48, steps=30, seed=4711),
    "pl63_basic_lcg_rw": dict(PL=63, opset=1, philox=0, rw=0.1, data="expdecay", N=48, steps=30, seed=2718),
    # edges: the shortest and the longest programs, an empty dataset
    "pl1_ref_lcg_indep": dict(PL=1, opset=0, philox=0, rw=0.0, data="quad", N=48, steps=30, seed=99),
    "pl255_basic_lcg_rw": dict(PL=255, opset=1, philox=0, rw=0.1, data="expdecay", N=16, steps=20, seed=1234),
    "pl31_basic_lcg_rw_empty": dict(PL=31, opset=1, philox=0, rw=0.1, data="empty", N=48, steps=30, seed=555),
}
XS = np.float32([-1.5, 0.0, 0.25, 2.0, 7.5])


def main(names=None):
    for name, c in CASES.items():
        if names and name not in names:
            continue
        ops = H.OPSET_BASIC if c["opset"] else None
        if c["data"] == "empty":
            x = y = sd = np.zeros(0, np.float32)
        else:
            x, y, sd = (H.quad_data(101, seed=5) if c["data"] == "quad" else H.expdecay_data(250, seed=5))
        P0, C0 = H.random_programs(c["N"], c["PL"], ops=ops, seed=77)
        o = oref.get(pl=c["PL"], opset=c["opset"], philox=c["philox"], project_math=1, rw_sd=c["rw"])
        prior0 = np.array([o.prior(P0, C0, i) for i in range(c["N"])])
        lik0 = np.array([o.likelihood(P0, C0, i, x, y, sd) for i in range(c["N"])])
        length0 = np.array([o.length(P0, C0, i) for i in range(c["N"])], np.float32)
        count0 = np.array([o.count_nodes(P0, C0, i) for i in range(c["N"])], np.int32)
        fx0 = np.array([[o.call(P0, C0, i, v) for v in XS] for i in range(c["N"])], np.float32)
        P1, C1 = P0.copy(), C0.copy()
        prior1, lik1 = o.run_kernel(P1, C1, x, y, sd, c["steps"], c["seed"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), x=x, y=y, sd=sd, P0=P0, C0=C0, prior0=prior0,
                            lik0=lik0, length0=length0, count0=count0, xs=XS, fx0=fx0, P1=P1, C1=C1,
                            prior1=prior1, lik1=lik1, ops=np.int32(o.ops),
                            meta=json.dumps(dict(c, project_math=1)))
        strings = [[o.display("C", P0, C0, i), o.display("%.10f", P0, C0, i), o.display("%.2f", P0, C0, i, True)]
                   for i in range(c["N"])]
        with open(os.path.join(HERE, name + "_strings.json"), "w") as f:
            json.dump(strings, f, indent=0)
        print(name, "written")


if __name__ == "__main__":
    main(sys.argv[1:])
