"""ORACLE — test infrastructure only: the CPU restatement of the osbo/astro
Barnes-Hut step (see astro_oracle.h). Used by tests/, __graft_entry__.smoke()
and bench.py's CPU baseline; never by the product."""
