"""CPU oracle for the N1curl assembly/solve path.

TEST INFRASTRUCTURE: only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline legs may import this package.  The product never does.
"""
