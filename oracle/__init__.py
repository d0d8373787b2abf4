"""The oracle: CPU restatement of the reference's algorithms plus the reference's own CPU path
built through a single-rank MPI stand-in.  TEST INFRASTRUCTURE ONLY — imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the product package."""
