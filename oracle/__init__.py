"""Oracle for the DG time step: test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package.  It holds
  - charm_oracle.c: a CPU restatement of the reference's algorithm (builds
    anywhere; the checker on GPU machines),
  - build_ref.py + ref_driver.c + p4est_shim/: the reference's own C sources
    compiled against a p4est-subset shim (only where the reference checkout
    exists), used to pin the restatement and to make tests/golden fixtures.
"""
