"""CPU oracle — test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's CPU baseline).

The solver package never imports this. See sb_oracle.c for what it restates and where.
"""
