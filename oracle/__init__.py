"""Oracles for the parity tests -- TEST INFRASTRUCTURE ONLY.

oracle.ref      : the reference's own main.cu compiled for host cores
                  (recipe: oracle/build_ref.py, outputs in oracle/_ref/).
oracle.port     : a plain-C restatement of the reference's algorithm
                  (oracle/gpr_oracle.c), checked against oracle.ref and the
                  committed golden vectors in tests/golden/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package; the product never imports it.
"""
