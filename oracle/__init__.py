"""Test infrastructure: the FP64 oracle, the CPU timing port and the recipe that builds the
reference program for the host.  Imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py -- never by the calcir_gb300 product."""
