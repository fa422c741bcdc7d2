"""The oracle: CPU restatement of the reference path plus the reference's own
host build.  Test infrastructure only (tests/, __graft_entry__.smoke(), and the
CPU-baseline / reference legs of bench.py)."""
