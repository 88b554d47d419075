"""The oracle: CPU restatement of the reference path (acum_oracle.c) and, where the
reference tree is available, the reference's own sources compiled for the host
(build_ref.sh).  TEST INFRASTRUCTURE ONLY -- imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the product."""
